"""The allocation-free EMT entry point (mdt_emt_force_noalloc) against the regular
context path and the FP64 oracle, called through the C ABI on device buffers the test owns.

This entry point is for callers that may not allocate device memory themselves; it
keeps its pair scratch in a file-scope device array shared by all calls.  The test
runs two different configurations back to back so that a stale scratch array from the
first call would show up in the second.  It lives in its own file, collected last."""
import ctypes as ct

import numpy as np
import pytest

from md_tian2_gb300 import workloads as W
from md_tian2_gb300._lib import load
from md_tian2_gb300.engine import Engine, SimParams

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-10   # eV/A, the FP64 EMT bar of the parity tests
EPOT_TOL = 1e-9     # eV


def _config(seed, k):
    rng = np.random.default_rng(seed)
    u = W.h_on_metal(rng, "Au", k, 1.0, 20.0, 30.0, 300.0, z0=1.4)
    u.r[1:] += rng.normal(scale=0.05, size=u.r[1:].shape)
    return u


def _context_path(u, emt):
    eng = Engine(0)
    eng.read_emt(emt)
    eng.define([u])
    eng.upload()
    eng.calc_force(SimParams())
    out = eng.download()
    eng.close()
    return out["f"].reshape(-1, 3), out["epot"][0], out["dens"]


def _oracle(u, emt):
    from oracle.oracle import OracleUniverse
    o = OracleUniverse(u, emt)
    o.calc_force(SimParams())
    return o.f[:, 0, :], float(o.epot[0]), o.dens[:, 0]


def _noalloc(lib, u, emt, torch, idx_override=None):
    dev = torch.device("cuda", 0)
    n = u.natoms
    r = torch.tensor(u.r[:, 0, :], dtype=torch.float64, device=dev)
    x, y, z = (r[:, d].contiguous() for d in range(3))
    idx = torch.tensor(u.idx if idx_override is None else idx_override, dtype=torch.int32, device=dev)
    f = torch.zeros((3, n), dtype=torch.float64, device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    dens = torch.zeros(n, dtype=torch.float64, device=dev)
    box = np.ascontiguousarray(u.simbox.T.reshape(-1), np.float64)
    prm = [np.ascontiguousarray(a, np.float64) for a in emt.arrays()]
    pes = np.ascontiguousarray(emt.pes.T, np.int32)
    torch.cuda.synchronize()
    rc = lib.mdt_emt_force_noalloc(n, idx.data_ptr(), x.data_ptr(), y.data_ptr(), z.data_ptr(), box.ctypes.data,
                                   emt.ntypes, *[a.ctypes.data for a in prm], pes.ctypes.data, f[0].data_ptr(),
                                   f[1].data_ptr(), f[2].data_ptr(), e.data_ptr(), dens.data_ptr(), None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return f.T.cpu().numpy(), float(e.cpu()[0]), dens.cpu().numpy()


def test_noalloc_matches_context_path_twice(built_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    lib = load()
    emt = W.emt_params()
    for seed, k in ((1, 4), (2, 3)):  # two calls in a row, different sizes
        u = _config(seed, k)
        f_ref, e_ref, d_ref = _context_path(u, emt)
        f_o, e_o, d_o = _oracle(u, emt)
        f, e, d = _noalloc(lib, u, emt, torch)
        assert np.abs(f - f_ref).max() < FORCE_TOL
        assert abs(e - e_ref) < EPOT_TOL
        np.testing.assert_allclose(d, d_ref, rtol=1e-12)
        assert np.abs(f - f_o).max() < FORCE_TOL
        assert abs(e - e_o) < EPOT_TOL
        np.testing.assert_allclose(d, d_o, rtol=1e-12)


def test_noalloc_type_outside_table_gives_nan_energy(built_lib):
    """A 1-based type index beyond the parameter table's ntypes (here 3 with two types)
    makes the energy NaN instead of silently dropping the atom."""
    torch = pytest.importorskip("torch")
    lib = load()
    emt = W.emt_params()
    u = _config(3, 3)
    idx = np.array(u.idx, np.int32)
    idx[4] = 3
    _, e, _ = _noalloc(lib, u, emt, torch, idx_override=idx)
    assert np.isnan(e)
    _, e_ok, _ = _noalloc(lib, u, emt, torch)  # the next call is clean again
    assert np.isfinite(e_ok)


def test_noalloc_rejects_oversized_configuration(built_lib):
    lib = load()
    emt = W.emt_params()
    prm = [np.ascontiguousarray(a, np.float64) for a in emt.arrays()]
    pes = np.ascontiguousarray(emt.pes.T, np.int32)
    box = np.eye(3).reshape(-1) * 30.0
    rc = lib.mdt_emt_force_noalloc(257, None, None, None, None, box.ctypes.data, emt.ntypes,
                                   *[a.ctypes.data for a in prm], pes.ctypes.data, None, None, None, None, None, None)
    assert rc == -6  # MDT_ERR_TOO_LARGE
