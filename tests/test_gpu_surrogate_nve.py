"""NVE energy drift of the surrogate path: velocity Verlet with no friction, all atoms
free, 8 H/Au(111) trajectories for 2 ps, forces from the shipped surrogate on the
thread-per-atom kernel (FP32, and the tensor-core network with split BF16 operands), total
energy from the per-trajectory FP64 sums of the kernel's FP32 evaluation of the same states
(surrogate.nve_drift; for the tensor-core run that separates the dynamics' drift from the
readout of its own energies, which is reported and bounded separately).  The plain BF16
network (MDT_PREC_BF16) does not meet the target: its weights rounded to 8 bits shift the
potential by O(10) meV per atom, so its forces are not the gradient of the FP32 energy; the
bench reports its drift beside the others.  The secular drift (mean
slope of linear fits of E_tot(t)) must stay below the 1 meV/ps target and every trajectory
below 3 meV/ps (tighter than the FP64 EMT test of tests/test_gpu_propagators.py, whose
potential has steps at its pair cutoff; the network's cutoff function is smooth); no bead may
fall back to EMT (a fallback switches the potential and would be counted as drift)."""
import numpy as np
import pytest

from md_tian2_gb300.surrogate import nve_drift, shipped_surrogate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_surrogate_nve_drift(built_lib, prec):
    d = nve_drift(shipped_surrogate(), prec)
    assert d["radial_kernel"] and d["steps_ok"]
    assert d["fallbacks"] == 0
    assert abs(d["mean_meV_per_ps"]) < 1.0, d["slopes_meV_per_ps"]
    assert np.all(np.abs(d["slopes_meV_per_ps"]) < 3.0), d["slopes_meV_per_ps"]
    if prec == "bf16x3":
        assert d["readout_rms_meV"] < 5.0, d["readout_rms_meV"]
