"""RuNNer-style high-dimensional NN potential (HDNNP) model and its input files.

Readers follow what md_tian2's read_nene consumes (src/pes_nene_mod.f90:123-5759):
* ``input.nn``: elements, ``global_hidden_layers_short``, ``global_nodes_short``,
  ``global_activation_short``, ``symfunction_short`` (types 2 and 3),
  ``element_symfunction_short``, ``cutoff_type``, ``cutoff_alpha``,
  ``scale_symmetry_functions``, ``center_symmetry_functions``,
  ``scale_min_short_atomic``/``scale_max_short_atomic``, ``normalize_nodes``,
  ``remove_atom_energies`` + ``atom_energy``;
* ``scaling.data`` (readscale, pes_nene_mod.f90:6752-6903): per element and symmetry
  function ``elem sf min max avg``, then ``eshortmin eshortmax``;
* ``weights.XXX.data`` (readweights, pes_nene_mod.f90:6907-7028): one weight per line,
  XXX the nuclear charge, in calconenn order (RuNNer_src/calconenn.f90:90-107).
Symmetry functions are put into RuNNer's canonical order (RuNNer_src/sortsymfunctions.f90:
type, cutoff, eta, zeta, lambda, rshift, element 1, element 2) because the weight files
assume it.  All lengths are in bohr and energies in Hartree, as inside RuNNer.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import constants as C

# nuclear charges for the elements the workloads use (RuNNer's nuccharge table)
Z_OF = {"H": 1, "He": 2, "Li": 3, "C": 6, "N": 7, "O": 8, "Ni": 28, "Cu": 29, "Pd": 46, "Ag": 47,
        "Xe": 54, "Pt": 78, "Au": 79}
ACTS = set("tglcsSeph")


class NNInputError(ValueError):
    """Malformed RuNNer input (the reference would ``stop``)."""


@dataclass
class SymFunc:
    type: int
    eta: float = 0.0
    rshift: float = 0.0
    lam: float = 0.0
    zeta: float = 0.0
    rc: float = 0.0
    e1: int = 0   # neighbour nuclear charges
    e2: int = 0

    def key(self):
        return (self.type, self.rc, self.eta, self.zeta, self.lam, self.rshift, self.e1, self.e2)


@dataclass
class NNModel:
    elements: list                          # symbols, ascending nuclear charge
    sfs: list                               # per element: list[SymFunc] in canonical order
    nodes: list                             # per element: [nsf, h1, ..., 1]
    acts: list                              # per element: list of per-layer activation strings
    weights: list                           # per element: np.ndarray
    smin: list = field(default_factory=list)
    smax: list = field(default_factory=list)
    savg: list = field(default_factory=list)
    scalesym: bool = False
    centersym: bool = False
    scmin: float = 0.0
    scmax: float = 1.0
    cutoff_type: int = 1
    cutoff_alpha: float = 0.0
    normnodes: bool = False
    atom_energy: dict = field(default_factory=dict)  # symbol -> Ha (remove_atom_energies)
    eshort: tuple = (0.0, 0.0)

    @property
    def z(self):
        return [Z_OF[e] for e in self.elements]

    @property
    def nelem(self):
        return len(self.elements)

    @property
    def maxsf(self):
        return max(len(s) for s in self.sfs)

    @property
    def maxcut(self):
        return max(sf.rc for s in self.sfs for sf in s)

    def n_weights(self, e):
        n = self.nodes[e]
        return sum(n[l - 1] * n[l] + n[l] for l in range(1, len(n)))

    def flat(self):
        """Fixed-size arrays shared by the C ABI and the oracle (per element padded)."""
        ne, ms = self.nelem, self.maxsf
        nl = len(self.nodes[0]) - 1
        mx = max(max(n[1:]) for n in self.nodes)
        f = {k: np.zeros((ne, ms)) for k in ("eta", "rshift", "lambda", "zeta", "rc", "smin", "smax", "savg")}
        f["sftype"] = np.zeros((ne, ms), np.int32)
        f["e1"] = np.zeros((ne, ms), np.int32)
        f["e2"] = np.zeros((ne, ms), np.int32)
        for e in range(ne):
            for s, sf in enumerate(self.sfs[e]):
                f["sftype"][e, s] = sf.type
                f["eta"][e, s], f["rshift"][e, s], f["lambda"][e, s] = sf.eta, sf.rshift, sf.lam
                f["zeta"][e, s], f["rc"][e, s], f["e1"][e, s], f["e2"][e, s] = sf.zeta, sf.rc, sf.e1, sf.e2
                f["smin"][e, s] = self.smin[e][s] if self.smin else 0.0
                f["smax"][e, s] = self.smax[e][s] if self.smax else 1.0
                f["savg"][e, s] = self.savg[e][s] if self.savg else 0.0
        f["nsf"] = np.array([len(s) for s in self.sfs], np.int32)
        f["z"] = np.array(self.z, np.int32)
        f["nodes"] = np.array(self.nodes, np.int32)
        act = np.full((ne, nl, mx), ord("l"), np.uint8)
        for e in range(ne):
            for l in range(nl):
                for n in range(self.nodes[e][l + 1]):
                    act[e, l, n] = ord(self.acts[e][l][n])
        f["act"] = act
        mw = max(self.n_weights(e) for e in range(ne))
        w = np.zeros((ne, mw))
        for e in range(ne):
            w[e, :len(self.weights[e])] = self.weights[e]
        f["weights"] = w
        f["atom_energy"] = np.array([self.atom_energy.get(el, 0.0) for el in self.elements])
        f["nlayers"], f["maxnodes"], f["maxweights"] = nl, mx, mw
        return f


def _num(s: str) -> float:
    return float(s.replace("d", "e").replace("D", "e"))


def sort_symfunctions(sfs: list) -> list:
    """Canonical order of RuNNer_src/sortsymfunctions.f90 (successive stable passes on
    type, cutoff, eta, zeta, lambda, rshift, element 1, element 2 = one lexicographic
    sort); duplicates are an error (sortsymfunctions.f90:405-440)."""
    out = sorted(sfs, key=lambda s: s.key())
    for a, b in zip(out, out[1:]):
        if (a.type == b.type and abs(a.rc - b.rc) < 1e-4 and abs(a.eta - b.eta) < 1e-4 and abs(a.zeta - b.zeta) < 1e-4
                and abs(a.lam - b.lam) < 1e-4 and abs(a.rshift - b.rshift) < 1e-4 and a.e1 == b.e1 and a.e2 == b.e2):
            raise NNInputError("ERROR: a symmetry function is specified twice!")
    return out


def read_input_nn(path) -> dict:
    opts = {"elements": None, "hidden": None, "nodes": None, "acts": None, "sf": [], "esf": [],
            "cutoff_type": 1, "cutoff_alpha": 0.0, "scalesym": False, "centersym": False, "scmin": 0.0,
            "scmax": 1.0, "normnodes": False, "remove_atom_energies": False, "atom_energy": {}}
    for raw in Path(path).read_text().splitlines():
        line = raw.split("#")[0].split("!")[0].strip()
        if not line:
            continue
        w = line.split()
        key = w[0].lower()
        if key == "elements":
            opts["elements"] = w[1:]
        elif key == "number_of_elements":
            opts["nelem"] = int(w[1])
        elif key in ("global_hidden_layers_short", "global_hidden_layers_short_atomic"):
            opts["hidden"] = int(w[1])
        elif key in ("global_nodes_short", "global_nodes_short_atomic"):
            opts["nodes"] = [int(x) for x in w[1:]]
        elif key in ("global_activation_short", "global_activation_short_atomic"):
            opts["acts"] = w[1:]
        elif key == "symfunction_short":
            opts["sf"].append(w[1:])
        elif key == "element_symfunction_short":
            opts["esf"].append(w[1:])
        elif key == "cutoff_type":
            opts["cutoff_type"] = int(w[1])
        elif key == "cutoff_alpha":
            opts["cutoff_alpha"] = _num(w[1])
        elif key == "scale_symmetry_functions":
            opts["scalesym"] = True
        elif key == "center_symmetry_functions":
            opts["centersym"] = True
        elif key == "scale_min_short_atomic":
            opts["scmin"] = _num(w[1])
        elif key == "scale_max_short_atomic":
            opts["scmax"] = _num(w[1])
        elif key == "normalize_nodes":
            opts["normnodes"] = True
        elif key == "remove_atom_energies":
            opts["remove_atom_energies"] = True
        elif key == "atom_energy":
            opts["atom_energy"][w[1]] = _num(w[2])
    if not opts["elements"]:
        raise NNInputError("input.nn: elements keyword missing")
    if opts["hidden"] is None or opts["nodes"] is None or opts["acts"] is None:
        raise NNInputError("input.nn: network architecture keywords missing")
    if len(opts["nodes"]) < opts["hidden"] or len(opts["acts"]) < opts["hidden"] + 1:
        raise NNInputError("input.nn: global_nodes_short/global_activation_short too short")
    for a in opts["acts"][:opts["hidden"] + 1]:
        if a not in ACTS:
            raise NNInputError(f"Error: Unknown activation function {a}")
    return opts


def _parse_sf(center_z, words, nelem_z):
    """symfunction_short / element_symfunction_short words -> list of SymFunc."""
    t = int(words[1])
    if t == 2:
        if len(words) == 6:   # symfunction_short E 2 E2 eta rs rc
            return [SymFunc(2, eta=_num(words[3]), rshift=_num(words[4]), rc=_num(words[5]), e1=Z_OF[words[2]])]
        if len(words) == 5:   # element_symfunction_short E 2 eta rs rc (all neighbour elements)
            return [SymFunc(2, eta=_num(words[2]), rshift=_num(words[3]), rc=_num(words[4]), e1=z) for z in nelem_z]
    if t == 3:
        if len(words) == 8:   # symfunction_short E 3 E2 E3 eta lambda zeta rc
            z2, z3 = sorted((Z_OF[words[2]], Z_OF[words[3]]))
            return [SymFunc(3, eta=_num(words[4]), lam=_num(words[5]), zeta=_num(words[6]), rc=_num(words[7]), e1=z2, e2=z3)]
        if len(words) == 6:
            return [SymFunc(3, eta=_num(words[2]), lam=_num(words[3]), zeta=_num(words[4]), rc=_num(words[5]), e1=z, e2=z)
                    for z in nelem_z]
    raise NNInputError(f"symmetry function type {words[1]} / form {' '.join(words)} not supported (G2/G3 only)")


def read_runner(inp_dir) -> NNModel:
    """Read input.nn, scaling.data and weights.XXX.data from ``inp_dir``."""
    d = Path(inp_dir)
    o = read_input_nn(d / "input.nn")
    elements = sorted(o["elements"], key=lambda e: Z_OF[e])
    zs = [Z_OF[e] for e in elements]
    sfs = {e: [] for e in elements}
    for words in o["sf"]:
        sfs[words[0]].extend(_parse_sf(Z_OF[words[0]], words, zs))
    for words in o["esf"]:
        sfs[words[0]].extend(_parse_sf(Z_OF[words[0]], words, zs))
    sf_list = [sort_symfunctions(sfs[e]) for e in elements]
    hidden = o["hidden"]
    nodes = [[len(sf_list[e])] + o["nodes"][:hidden] + [1] for e in range(len(elements))]
    acts = [[o["acts"][l] * nodes[e][l + 1] for l in range(hidden + 1)] for e in range(len(elements))]
    # scaling.data
    smin, smax, savg = [], [], []
    lines = [l.split() for l in (d / "scaling.data").read_text().splitlines() if l.strip()]
    k = 0
    for e in range(len(elements)):
        mi, ma, av = [], [], []
        for _ in range(len(sf_list[e])):
            if k >= len(lines) or len(lines[k]) != 5:
                raise NNInputError("scaling.data: expected 'elem sf min max avg' lines")
            mi.append(_num(lines[k][2]))
            ma.append(_num(lines[k][3]))
            av.append(_num(lines[k][4]))
            k += 1
        smin.append(np.array(mi))
        smax.append(np.array(ma))
        savg.append(np.array(av))
    eshort = (0.0, 0.0)
    if k < len(lines) and len(lines[k]) == 2:
        eshort = (_num(lines[k][0]), _num(lines[k][1]))
    model = NNModel(elements=elements, sfs=sf_list, nodes=nodes, acts=acts, weights=[], smin=smin, smax=smax,
                    savg=savg, scalesym=o["scalesym"], centersym=o["centersym"], scmin=o["scmin"], scmax=o["scmax"],
                    cutoff_type=o["cutoff_type"], cutoff_alpha=o["cutoff_alpha"], normnodes=o["normnodes"],
                    atom_energy=o["atom_energy"] if o["remove_atom_energies"] else {}, eshort=eshort)
    for e, el in enumerate(elements):
        f = d / f"weights.{Z_OF[el]:03d}.data"
        if not f.exists():
            raise NNInputError(f"weights file {f.name} missing")
        vals = []
        for line in f.read_text().splitlines():
            w = line.split()
            if not w:
                continue
            if len(w) != 1:
                raise NNInputError(f"{f.name}: one weight per line expected")
            vals.append(_num(w[0]))
        nw = model.n_weights(e)
        if len(vals) < nw:
            raise NNInputError(f"{f.name}: {len(vals)} weights, network needs {nw}")
        model.weights.append(np.array(vals[:nw]))
    return model


# ---------------------------------------------------------------------------
# Synthetic models with the benchmark configurations' shapes
# ---------------------------------------------------------------------------
def acsf_set(center: str, neighbours: list, rc_ang: float = 6.5) -> list:
    """8 G2 (eta log-spaced 0.001-0.5 1/A^2, r_s = 0) per neighbour element and 16 G3
    (zeta in {1,4,16} x lambda = +-1 x eta in {0.001,0.01,0.1} 1/A^2 without the two
    zeta = 16, eta = 0.1 entries) over neighbour pairs; cosine cutoff at rc_ang.
    Returned in bohr units and RuNNer's canonical order."""
    a2b = C.ANG2BOHR
    rc = rc_ang * a2b
    etas2 = np.geomspace(0.001, 0.5, 8) / a2b ** 2
    out = []
    zs = sorted(Z_OF[n] for n in neighbours)
    for z in zs:
        for eta in etas2:
            out.append(SymFunc(2, eta=float(eta), rshift=0.0, rc=rc, e1=z))
    pairs = [(a, b) for i, a in enumerate(zs) for b in zs[i:]]
    for (z1, z2) in pairs:
        for eta in (0.001, 0.01, 0.1):
            for zeta in (1.0, 4.0, 16.0):
                if zeta == 16.0 and eta == 0.1:
                    continue
                for lam in (1.0, -1.0):
                    out.append(SymFunc(3, eta=eta / a2b ** 2, lam=lam, zeta=zeta, rc=rc, e1=z1, e2=z2))
    return sort_symfunctions(out)


def radial_set(center: str, neighbours: list, rc_ang: float = 6.5) -> list:
    """24 radial functions per centre element, no angular ones: for metal neighbours 20
    shifted Gaussians (r_s = 0.8 ... 6.5 A every 0.3 A, eta = 4 1/A^2), for H neighbours
    4 (r_s = 1, 2, 3, 4 A, eta = 1 1/A^2).  The 0.3 A grid resolves the neighbour shells
    and the region of EMT's cutoff; equal spacing lets the FP32 kernels evaluate a group
    with three exponentials.  Cosine cutoff at rc_ang."""
    a2b = C.ANG2BOHR
    rc = rc_ang * a2b
    out = []
    for z in sorted(Z_OF[n] for n in neighbours):
        if z == Z_OF["H"]:
            grid, eta = [1.0 + 1.0 * k for k in range(4)], 1.0
        else:
            grid, eta = [0.8 + 0.3 * k for k in range(20)], 4.0
        for rs in grid:
            out.append(SymFunc(2, eta=eta / a2b ** 2, rshift=rs * a2b, rc=rc, e1=z))
    return sort_symfunctions(out)


def random_model(elements: list, hidden=(25, 25), act="t", seed: int = 0, neighbours=None,
                 descriptor: str = "acsf") -> NNModel:
    """Seeded Glorot-uniform network with the ACSF set above for every element."""
    rng = np.random.default_rng(seed)
    elements = sorted(elements, key=lambda e: Z_OF[e])
    neighbours = neighbours or elements
    make = {"acsf": acsf_set, "radial": radial_set}[descriptor]
    sfs = [make(e, neighbours) for e in elements]
    nodes = [[len(s)] + list(hidden) + [1] for s in sfs]
    acts = [[act * n[l + 1] for l in range(len(hidden))] + ["l"] for n in nodes]
    weights = []
    for n in nodes:
        w = []
        for l in range(1, len(n)):
            lim = np.sqrt(6.0 / (n[l - 1] + n[l]))
            w.extend(rng.uniform(-lim, lim, size=n[l - 1] * n[l]))
            w.extend(np.zeros(n[l]))
        weights.append(np.array(w))
    ns = [len(s) for s in sfs]
    return NNModel(elements=elements, sfs=sfs, nodes=nodes, acts=acts, weights=weights,
                   smin=[np.zeros(k) for k in ns], smax=[np.ones(k) for k in ns], savg=[np.zeros(k) for k in ns])


# ---------------------------------------------------------------------------
# Compact single-file storage (npz) of a model: what the three RuNNer files hold
# ---------------------------------------------------------------------------
def save_npz(model: NNModel, path) -> None:
    d = {"elements": np.array(model.elements), "nodes": np.array(model.nodes, np.int32),
         "opts": np.array([model.scalesym, model.centersym, model.normnodes, model.cutoff_type], np.int32),
         "fopts": np.array([model.scmin, model.scmax, model.cutoff_alpha, model.eshort[0], model.eshort[1]]),
         "atom_energy": np.array([model.atom_energy.get(e, np.nan) for e in model.elements])}
    for e, el in enumerate(model.elements):
        d[f"sf_{e}"] = np.array([[sf.type, sf.eta, sf.rshift, sf.lam, sf.zeta, sf.rc, sf.e1, sf.e2] for sf in model.sfs[e]])
        d[f"w_{e}"] = model.weights[e]
        d[f"act_{e}"] = np.array(["".join(a) for a in model.acts[e]])
        d[f"scale_{e}"] = np.stack([model.smin[e], model.smax[e], model.savg[e]])
    np.savez(path, **d)


def load_npz(path) -> NNModel:
    z = np.load(path)
    elements = [str(e) for e in z["elements"]]
    sfs, weights, acts, smin, smax, savg = [], [], [], [], [], []
    for e in range(len(elements)):
        sfs.append([SymFunc(int(r[0]), r[1], r[2], r[3], r[4], r[5], int(r[6]), int(r[7])) for r in z[f"sf_{e}"]])
        weights.append(np.array(z[f"w_{e}"]))
        acts.append([str(a) for a in z[f"act_{e}"]])
        sc = z[f"scale_{e}"]
        smin.append(sc[0].copy()); smax.append(sc[1].copy()); savg.append(sc[2].copy())
    o, fo = z["opts"], z["fopts"]
    ae = {el: float(v) for el, v in zip(elements, z["atom_energy"]) if np.isfinite(v)}
    return NNModel(elements=elements, sfs=sfs, nodes=[list(map(int, n)) for n in z["nodes"]], acts=acts,
                   weights=weights, smin=smin, smax=smax, savg=savg, scalesym=bool(o[0]), centersym=bool(o[1]),
                   scmin=float(fo[0]), scmax=float(fo[1]), cutoff_type=int(o[3]), cutoff_alpha=float(fo[2]),
                   normnodes=bool(o[2]), atom_energy=ae, eshort=(float(fo[3]), float(fo[4])))


def rescale_first_layer(model: NNModel, old_smin: list, old_smax: list) -> None:
    """After the scaling columns of a scaled network changed from (old_smin, old_smax) to
    the model's current ones, change its first-layer weights and biases so that the
    network computes the same function of the raw symmetry functions: with scaled
    x = a G + b (scale_symmetry_functions, no centring), x_old = k x_new + c with
    k = a_old / a_new and c = b_old - k b_new, folded into W1 and b1."""
    if model.centersym or not model.scalesym:
        raise ValueError("rescale_first_layer needs scale_symmetry_functions without centring")
    span = model.scmax - model.scmin
    for e in range(model.nelem):
        n0, n1 = model.nodes[e][0], model.nodes[e][1]
        a_o = span / (np.asarray(old_smax[e]) - np.asarray(old_smin[e]))
        b_o = model.scmin - a_o * np.asarray(old_smin[e])
        a_n = span / (np.asarray(model.smax[e]) - np.asarray(model.smin[e]))
        b_n = model.scmin - a_n * np.asarray(model.smin[e])
        k = a_o / a_n
        c = b_o - k * b_n
        w = np.asarray(model.weights[e], dtype=np.float64).copy()
        W = w[:n0 * n1].reshape(n0, n1)
        w[n0 * n1:n0 * n1 + n1] += c @ W
        w[:n0 * n1] = (W * k[:, None]).reshape(-1)
        model.weights[e] = w


def set_scaling(model: NNModel, G: np.ndarray, elem: np.ndarray, margin: float = 0.0) -> None:
    """Fill scaling.data columns (min, max, average per element and function) from raw
    descriptors G (rows = atoms) the way RuNNer's scaling mode does, and switch on
    scale_symmetry_functions."""
    for e in range(model.nelem):
        rows = G[elem == e][:, :len(model.sfs[e])]
        if len(rows) == 0:
            continue
        mn, mx = rows.min(0), rows.max(0)
        # a degenerate range (one atom, or a function that never fires) gets a width of
        # 10 % of its magnitude (at least 1e-3) so that the scaling stays finite
        flat = (mx - mn) < 1e-12
        pad = np.where(flat, np.maximum(0.05 * np.abs(mn), 5e-4), 0.0)
        mn, mx = mn - pad, mx + pad
        w = mx - mn
        model.smin[e] = mn - margin * w
        model.smax[e] = mx + margin * w
        model.savg[e] = rows.mean(0)
    model.scalesym = True
