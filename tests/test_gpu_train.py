"""The GPU training gradient (energy + force loss) against central finite differences
of the same loss evaluated with the FP64 HDNNP oracle."""
import numpy as np
import pytest

from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams
from md_tian2_gb300.surrogate import Dataset, Trainer

pytestmark = pytest.mark.gpu


def _tiny_dataset(n=3, seed=0):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(seed)
    emt = W.emt_params()
    us, es, fs = [], [], []
    for t in range(n):
        u = W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=1.2 + 0.4 * t)
        u.r[1:] += rng.normal(scale=0.08, size=u.r[1:].shape)
        o = OracleUniverse(u, emt)
        o.calc_force(SimParams())
        us.append(u)
        es.append(o.epot[0])
        fs.append(o.f[:, 0, :].copy())
    return Dataset(us, np.array(es), fs)


def _oracle_loss(model, data, wE, wF):
    from oracle.oracle import NNOracle
    o = NNOracle(model)
    L = 0.0
    for u, e, f in zip(data.universes, data.energy, data.forces):
        elem = np.array([model.elements.index(u.names[i - 1]) for i in u.idx])
        E, F = o.energy_force(elem, u.r[:, 0, :], u.simbox)
        N = u.natoms
        L += wE * ((E - e) / N) ** 2 + wF * np.sum((F - f) ** 2) / (3 * N)
    return L / len(data.universes)


def test_training_gradient_matches_finite_differences(built_lib, oracle_lib):
    data = _tiny_dataset()
    model = nene.random_model(["H", "Au"], hidden=(8, 8), act="p", seed=2, neighbours=["Au"])
    model.weights = [np.asarray(w, np.float32).astype(np.float64) for w in model.weights]  # FP32 master values
    tr = Trainer(data, model)  # sets scaling from the GPU descriptors
    wE, wF = 3.0, 1.0
    g64 = tr.gradient([0, 1, 2], wE, wF, "fp64")
    g32 = tr.gradient([0, 1, 2], wE, wF, "fp32")
    tr.close()
    mw = max(model.n_weights(e) for e in range(model.nelem))
    rng = np.random.default_rng(5)
    picks = [(e, int(k)) for e in range(model.nelem) for k in rng.choice(model.n_weights(e), 6, replace=False)]
    for e, k in picks:
        w0 = model.weights[e][k]
        h = 1e-4 * max(1.0, abs(w0))
        model.weights[e][k] = w0 + h
        lp = _oracle_loss(model, data, wE, wF)
        model.weights[e][k] = w0 - h
        lm = _oracle_loss(model, data, wE, wF)
        model.weights[e][k] = w0
        fd = (lp - lm) / (2 * h)
        g = g64[e * mw + k]
        assert abs(g - fd) <= 1e-5 * max(abs(fd), 1e-6) + 1e-9, (e, k, g, fd)
    scale = np.abs(g64).max()
    assert np.abs(g32 - g64).max() < 2e-3 * scale


@pytest.mark.parametrize("prec,bar", [("bf16", 3e-2), ("bf16x3", 2e-3)])
def test_gemm_training_gradient(built_lib, oracle_lib, prec, bar):
    """The training gradient with the network's products as BF16 GEMMs (FP32 accumulation)
    against the FP64 gradient, on every weight: within 3e-2 of the largest component with
    BF16 operands (8 significant bits), within 2e-3 -- the FP32 kernel's bar -- with split
    BF16 operands; a second call on another row set reuses the buffers."""
    data = _tiny_dataset()
    model = nene.random_model(["H", "Au"], hidden=(8, 8), act="p", seed=2, neighbours=["Au"])
    model.weights = [np.asarray(w, np.float32).astype(np.float64) for w in model.weights]
    tr = Trainer(data, model)
    g64 = tr.gradient([0, 1, 2], 3.0, 1.0, "fp64")
    g16 = tr.gradient([0, 1, 2], 3.0, 1.0, prec)
    g16b = tr.gradient([2, 0], 3.0, 1.0, prec)
    g64b = tr.gradient([2, 0], 3.0, 1.0, "fp64")
    tr.close()
    for a, b in ((g16, g64), (g16b, g64b)):
        scale = np.abs(b).max()
        assert np.abs(a - b).max() < bar * scale, (np.abs(a - b).max(), scale)
        assert np.corrcoef(a, b)[0, 1] > 0.999


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
def test_training_reduces_loss(built_lib, oracle_lib, prec):
    data = _tiny_dataset(n=6, seed=1)
    model = nene.random_model(["H", "Au"], hidden=(16, 16), act="p", seed=3, neighbours=["Au"])
    tr = Trainer(data, model)
    hist = tr.train(epochs=200, batch=6, lr=3e-3, lr_final=1e-3, w_energy=1.0, w_force=1.0, precision=prec)
    tr.close()
    assert hist[-1][2] < 0.5 * hist[0][2]
