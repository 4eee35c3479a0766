"""A second, independent restatement of the reference's EMT and RuNNer HDNNP energies,
written in torch FP64.  EMT:
from compute_emt_1species / compute_emt_2species (src/pes_emt_mod.f90:230-477, 483-1027):
energies must equal the oracle's (oracle/md_oracle.cpp) to round-off, and forces taken by
automatic differentiation of that energy must equal the oracle's hand-derived forces (the
reference's dense derivative tensors).  This pins the oracle's derivative code without
trusting its author twice: only the energy expression is restated, the derivative is
torch's.

Configurations have one projectile: the reference's type1-type1 derivative quirk
(pes_emt_mod.f90:705, eta2 of type2 in the H-H density derivative) only acts between two
projectile atoms, where autograd and the reference deliberately differ (checked too).
HDNNP: the shipped RuNNer C network and a random H/C model with G2 and G3 over two
neighbour elements; energies to 1e-9 relative, autograd forces against the oracle's
forward-mode dG/dx contraction (getshortatomic.f90:263-322) to 1e-8 relative."""
import math

import numpy as np
import pytest

from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams

torch = pytest.importorskip("torch")
BOHR2ANG = 0.529177211
KEYS = ("eta2", "n0", "e0", "lambda", "v0", "kappa", "s0")


def emt_energy(r, simbox, types, prm, nspecies):
    """EMT energy of one bead (torch FP64; r (N, 3) A; types 0-based; prm[type][key])."""
    beta = (16.0 * math.pi / 3.0) ** (1.0 / 3.0) / math.sqrt(2.0)
    nneighs = torch.tensor([12.0, 6.0, 24.0], dtype=torch.float64)
    sp = list(range(nspecies))  # species s = type s (EMT types in table order)
    bs0 = [beta * prm[s]["s0"] for s in sp]
    rcut = max(bs0) * math.sqrt(3.0)
    rr = 4.0 * rcut / (math.sqrt(3.0) + 2)
    acut = 9.21034037197618 / (rr - rcut)
    ig1, ig2 = [], []
    for s in sp:
        rnn = bs0[s] * torch.tensor([1.0, math.sqrt(2.0), math.sqrt(3.0)], dtype=torch.float64)
        x = nneighs / 12.0 / (1 + torch.exp(acut * (rnn - rcut)))
        ig1.append(1.0 / float(torch.sum(x * torch.exp(-prm[s]["eta2"] * (rnn - bs0[s])))))
        ig2.append(1.0 / float(torch.sum(x * torch.exp(-prm[s]["kappa"] / beta * (rnn - bs0[s])))))
    n = r.shape[0]
    box = torch.tensor(simbox, dtype=torch.float64)
    ibox = torch.linalg.inv(box)
    i, j = np.triu_indices(n, 1)
    d = r[i] - r[j]
    w = d @ ibox.T
    w = w - torch.round(w).detach()
    d = w @ box.T
    rij = torch.sqrt((d * d).sum(1))
    keep = rij <= 1.5 * rcut
    i, j, rij = i[keep.numpy()], j[keep.numpy()], rij[keep]
    theta = 1.0 / (1.0 + torch.exp(acut * (rij - rcut)))
    ti, tj = types[i], types[j]
    sig = {k: torch.zeros(n, dtype=torch.float64) for k in ("11", "22", "12", "21")}
    V = {k: torch.zeros((), dtype=torch.float64) for k in ("11", "22", "12", "21")}

    def dens(s, rr_):
        return theta_sel * torch.exp(-prm[s]["eta2"] * (rr_ - bs0[s]))

    def pair(s, rr_):
        return theta_sel * torch.exp(-prm[s]["kappa"] / beta * (rr_ - bs0[s]))

    for (a, b_), key in (((0, 0), "11"), ((1, 1), "22")):
        m = torch.tensor((ti == a) & (tj == b_))
        if not m.any():
            continue
        rr_, theta_sel = rij[m], theta[m]
        s = a
        e = dens(s, rr_)
        sig[key] = sig[key].index_add(0, torch.tensor(i[m.numpy()]), e).index_add(0, torch.tensor(j[m.numpy()]), e)
        V[key] = pair(s, rr_).sum()
    if nspecies == 2:
        m = torch.tensor(ti != tj)  # projectile (type 1) first: i of type 1, j of type 2
        if m.any():
            rr_, theta_sel = rij[m], theta[m]
            sig["21"] = sig["21"].index_add(0, torch.tensor(j[m.numpy()]), dens(0, rr_))
            sig["12"] = sig["12"].index_add(0, torch.tensor(i[m.numpy()]), dens(1, rr_))
            V["21"] = pair(0, rr_).sum()
            V["12"] = pair(1, rr_).sum()
    chi21 = (prm[0]["n0"] / prm[1]["n0"] * math.exp(0.5 / BOHR2ANG * (prm[1]["s0"] - prm[0]["s0"]))
             if nspecies == 2 else 1.0)
    chi12 = 1.0 / chi21
    # the reference's scale factors, pes_emt_mod.f90:762-769 (1 species: :351-353)
    s11 = sig["11"] * ig1[0]
    e_pair = V["11"] * ig2[0] * prm[0]["v0"]
    s1 = s11
    if nspecies == 2:
        s22 = sig["22"] * ig1[1]
        s21 = sig["21"] * ig1[1]
        s12 = sig["12"] * ig1[0]
        e_pair = e_pair + V["22"] * ig2[1] * prm[1]["v0"] + 0.5 * (V["21"] * ig2[1] * prm[1]["v0"] * chi21 +
                                                                  V["12"] * ig2[0] * prm[0]["v0"] * chi12)
        s1 = s11 + chi12 * s12
        s2 = s22 + chi21 * s21
    tiny = float(np.float32(1e-30))
    energy = -e_pair
    for s, sv in enumerate([s1] + ([s2] if nspecies == 2 else [])):
        mask = torch.tensor(types == s)
        x = torch.clamp(sv[mask], min=tiny)
        x = torch.clamp(x, min=1e-9)
        ss = -torch.log(x / 12.0) / (beta * prm[s]["eta2"])
        energy = energy + prm[s]["e0"] * torch.sum((1 + prm[s]["lambda"] * ss) * torch.exp(-prm[s]["lambda"] * ss) - 1)
        vref = 12 * prm[s]["v0"] * torch.sum(torch.exp(-prm[s]["kappa"] * ss))
        energy = energy + 0.5 * vref
    return energy


@pytest.mark.parametrize("case", ["H/Au", "H/Pt", "Pt"])
def test_oracle_forces_equal_autodiff_of_an_independent_energy(oracle_lib, case):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(17)
    if case == "Pt":
        emt = W.emt_params("H", "Pt", with_proj=False)
        pos, cell, fx = W.fcc111_slab(W.LATTICE_A["Pt"], 3)
        u = W.Universe(r=pos[:, None, :].copy(), v=np.zeros((len(pos), 1, 3)), m=np.full(len(pos), 1e4),
                       idx=np.ones(len(pos), np.int32), is_fixed=np.zeros((len(pos), 1, 3), bool), simbox=cell,
                       names=["Pt"], is_proj=np.array([False]), algo=np.array([1001], np.int32))
    else:
        metal = case.split("/")[1]
        emt = W.emt_params("H", metal)
        u = W.h_on_metal(rng, metal, 3, 1.0, 20.0, 30.0, 300.0, z0=1.3)
    u.r[:, 0, :] += rng.normal(scale=0.08, size=u.r[:, 0, :].shape)
    o = OracleUniverse(u, emt)
    o.calc_force(SimParams())
    types = np.asarray(u.idx) - 1
    prm = [{k: float(emt.values[k][t]) for k in KEYS} for t in range(emt.ntypes)]
    r = torch.tensor(u.r[:, 0, :], dtype=torch.float64, requires_grad=True)
    e = emt_energy(r, u.simbox, types, prm, emt.ntypes)
    e.backward()
    f = -r.grad.numpy()
    ev = e.item()
    assert abs(ev - float(o.epot[0])) < 1e-10 * max(1.0, abs(float(o.epot[0]))), (ev, o.epot[0])
    assert np.abs(f - o.f[:, 0, :]).max() < 1e-9, np.abs(f - o.f[:, 0, :]).max()


def _two_h_on_au(rng):
    u = W.h_on_metal(rng, "Au", 3, 1.0, 20.0, 30.0, 300.0, z0=1.4)
    h2 = u.r[0:1].copy()
    h2[0, 0, 0] += 0.9
    u.r = np.concatenate([u.r[:1], h2, u.r[1:]])
    u.v = np.zeros_like(u.r)
    u.m = np.concatenate([u.m[:1], u.m[:1], u.m[1:]])
    u.idx = np.concatenate([[1, 1], u.idx[1:]]).astype(np.int32)
    u.is_fixed = np.concatenate([u.is_fixed[:1], u.is_fixed[:1], u.is_fixed[1:]])
    return u


def test_oracle_keeps_the_reference_h_h_derivative_quirk(oracle_lib):
    """Two projectile atoms: the oracle's H-H density derivative takes eta2 of the metal, as
    the reference does (pes_emt_mod.f90:705), so its forces differ from the derivative of the
    energy; with eta2 of H set equal to the metal's the two agree again."""
    from oracle.oracle import OracleUniverse
    u = _two_h_on_au(np.random.default_rng(5))
    types = np.asarray(u.idx) - 1
    for same_eta in (False, True):
        emt = W.emt_params("H", "Au")
        if same_eta:
            emt.values["eta2"][0] = emt.values["eta2"][1]
        o = OracleUniverse(u, emt)
        o.calc_force(SimParams())
        prm = [{k: float(emt.values[k][t]) for k in KEYS} for t in range(emt.ntypes)]
        r = torch.tensor(u.r[:, 0, :], dtype=torch.float64, requires_grad=True)
        e = emt_energy(r, u.simbox, types, prm, 2)
        e.backward()
        d = np.abs(-r.grad.numpy() - o.f[:, 0, :]).max()
        assert abs(e.item() - float(o.epot[0])) < 1e-10 * max(1.0, abs(float(o.epot[0])))
        if same_eta:
            assert d < 1e-9, d
        else:
            assert d > 1e-4, d


# ---------------------------------------------------------------------------------------
# RuNNer HDNNP (compute_nene): a torch restatement of the energy from the symmetry-function
# definitions (atomsymfunction2.f90, atomsymfunction3Andi.f90, getcutoff.f90), the scaling of
# getshortatomic.f90:174-236 and the network of calconenn.f90:83-153, with its own periodic
# neighbour search; forces by autograd against the oracle's forward-mode dG/dx contraction.
# ---------------------------------------------------------------------------------------
ANG2BOHR = 1.0 / BOHR2ANG
HA2EV = 27.21138602


def _cutoff(kind, r, rc):
    x = r / rc
    if kind == 1:
        return 0.5 * (torch.cos(math.pi * x) + 1.0)
    if kind == 6:
        return ((15.0 - 6.0 * x) * x - 10.0) * x ** 3 + 1.0
    raise ValueError(kind)


def _act(a, x):
    return {"t": torch.tanh, "l": lambda v: v, "p": lambda v: torch.log(torch.exp(v) + 1.0),
            "s": torch.sigmoid}[a](x)


def hdnnp_energy(model, elem, r_ang, simbox):
    """Total energy (eV) of one configuration; r_ang a leaf tensor (N, 3) in A."""
    box = np.asarray(simbox, float)
    x = r_ang * ANG2BOHR
    lat = torch.tensor(box.T * ANG2BOHR)  # rows: lattice vectors (bohr)
    n = x.shape[0]
    rc_max = max(sf.rc for sfs in model.sfs for sf in sfs)
    # image range from the plane spacings
    inv = np.linalg.inv(box.T * ANG2BOHR)
    reach = [int(math.ceil(rc_max * np.linalg.norm(inv[:, d]))) for d in range(3)]
    shifts = np.array([(a, b, c) for a in range(-reach[0], reach[0] + 1) for b in range(-reach[1], reach[1] + 1)
                       for c in range(-reach[2], reach[2] + 1)], float)
    sh = torch.tensor(shifts) @ lat  # (S, 3)
    zs = np.array([model.z[e] for e in elem])
    etot = torch.zeros((), dtype=torch.float64)
    for i in range(n):
        e = elem[i]
        pos = (x[None, :, :] + sh[:, None, :]).reshape(-1, 3)  # every image of every atom
        zn = np.tile(zs, len(shifts))
        d = pos - x[i]
        r2 = (d * d).sum(1)
        self_mask = np.zeros(len(zn), bool)
        self_mask[np.where(np.all(shifts == 0, axis=1))[0][0] * n + i] = True
        keep = ((r2.detach().numpy() <= rc_max ** 2) & ~self_mask)
        d, zn = d[keep], zn[keep]
        r = torch.sqrt(r2[keep])  # (the atom itself, at distance 0, is out before the square root)
        G = []
        for sf in model.sfs[e]:
            inside = r <= sf.rc
            if sf.type == 2:
                m = torch.tensor((zn == sf.e1)) & inside
                rr = r[m]
                G.append(torch.sum(torch.exp(-sf.eta * (rr - sf.rshift) ** 2) * _cutoff(model.cutoff_type, rr, sf.rc)))
            else:
                q3, q4 = np.triu_indices(len(r), 1)
                ok = (((zn[q3] == sf.e1) & (zn[q4] == sf.e2)) | ((zn[q3] == sf.e2) & (zn[q4] == sf.e1)))
                q3, q4 = q3[ok], q4[ok]
                rij, rik = r[q3], r[q4]
                djk = d[q3] - d[q4]
                rjk = torch.sqrt((djk * djk).sum(1))
                m = (rij <= sf.rc) & (rik <= sf.rc) & (rjk <= sf.rc)
                rij, rik, rjk = rij[m], rik[m], rjk[m]
                cos = (d[q3][m] * d[q4][m]).sum(1) / (rij * rik)
                plam = 1.0 + sf.lam * cos
                ang = torch.where(plam > 0, plam, torch.zeros_like(plam)) ** sf.zeta
                fc = (_cutoff(model.cutoff_type, rij, sf.rc) * _cutoff(model.cutoff_type, rik, sf.rc) *
                      _cutoff(model.cutoff_type, rjk, sf.rc))
                G.append(2.0 ** (1.0 - sf.zeta) * torch.sum(ang * torch.exp(-sf.eta * (rij ** 2 + rik ** 2 + rjk ** 2))
                                                         * fc))
        G = torch.stack(G)
        if model.scalesym:
            smin = torch.tensor(np.asarray(model.smin[e], float))
            smax = torch.tensor(np.asarray(model.smax[e], float))
            G = (G - smin) / (smax - smin) * (model.scmax - model.scmin) + model.scmin
        nodes, w = model.nodes[e], np.asarray(model.weights[e], float)
        val, ic = G, 0
        for layer in range(1, len(nodes)):
            W_ = torch.tensor(w[ic:ic + nodes[layer - 1] * nodes[layer]].reshape(nodes[layer - 1], nodes[layer]))
            ic += nodes[layer - 1] * nodes[layer]
            b = torch.tensor(w[ic:ic + nodes[layer]])
            ic += nodes[layer]
            s = val @ W_ + b
            acts = model.acts[e][layer - 1]
            val = torch.stack([_act(acts[k], s[k]) for k in range(nodes[layer])])
        etot = etot + val[0]
    return etot * HA2EV


def _wrapped(r, box):
    f = r @ np.linalg.inv(box).T
    f -= np.floor(f)
    return f @ box.T


@pytest.mark.parametrize("case", ["shipped C network", "random H/C G2+G3"])
def test_hdnnp_oracle_forces_equal_autodiff(oracle_lib, case):
    from pathlib import Path

    from md_tian2_gb300 import nene
    from oracle.oracle import NNOracle
    gold = Path(__file__).resolve().parent / "golden"
    if case.startswith("shipped"):
        m = nene.load_npz(gold / "runner_cgraphene.npz")
        g = np.load(gold / "cgraphene_geometry.npz")
        r0, box = _wrapped(g["r"], g["simbox"]), g["simbox"]
        elem = np.zeros(len(r0), int)
    else:
        rng = np.random.default_rng(3)
        u = W.h_on_graphene(rng, 1.0, z0=1.6, k=3)
        m = nene.random_model(["H", "C"], hidden=(12, 10), act="t", seed=2, neighbours=["H", "C"])
        m.cutoff_type = 6
        r0, box = _wrapped(u.r[:, 0, :], u.simbox), u.simbox
        elem = np.array([0] + [1] * (u.natoms - 1))
    E0, F0 = NNOracle(m).energy_force(elem, r0, box)
    r = torch.tensor(r0, dtype=torch.float64, requires_grad=True)
    e = hdnnp_energy(m, elem, r, box)
    e.backward()
    f = -r.grad.numpy()
    assert abs(e.item() - E0) < 1e-9 * max(1.0, abs(E0)), (e.item(), E0)
    assert np.abs(f - F0).max() < 1e-8 * max(1.0, np.abs(F0).max()), np.abs(f - F0).max()
