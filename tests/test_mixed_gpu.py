"""The mixed-precision form against the plain FP64 path, on the same scenes.

FP32 element arithmetic changes every step's rounding, so the two runs agree to a relative
error rather than bit for bit. The bars: L/L0 of the 10 x 60 Taylor rod within 1e-4 relative
of the FP64 run (the error bar the mixed-precision forms are held to), its mushroom diameter
within 1e-3; on the coarse perforation, the slug's residual velocity within 1 %, the eroded
count within a few per cent, and the energy balance to within 1 % of the FP64 run's.
"""
import numpy as np
import pytest

from neofiz_gb300 import ExplicitSolver, Integration, _abi, scenes

pytestmark = pytest.mark.gpu


def _run_rod(precision, integration=Integration.REDUCED):
    s, mesh, info = scenes.taylor_rod(ExplicitSolver, integration=integration)
    s.setPrecision(precision)
    s.runUntil(80e-6)
    m = s.measure()
    return s, m.length / info["length"], m.mushroom_diameter


@pytest.mark.parametrize("integration", [Integration.REDUCED, Integration.FULL])
def test_rod_length_ratio_within_1e4(gpu_lib, integration):
    _, ratio64, mush64 = _run_rod(_abi.PRECISION_FP64, integration)
    s, ratio32, mush32 = _run_rod(_abi.PRECISION_MIXED, integration)
    assert abs(ratio32 - ratio64) <= 1e-4 * ratio64, (ratio32, ratio64)
    assert abs(mush32 - mush64) <= 1e-3 * mush64, (mush32, mush64)
    assert s.statusWord() == 0


def _slug_velocity(s, mesh, slug_elements):
    vr = s.velocityR()
    m = s.readField(_abi.FIELD_MASS)
    nodes = np.unique(mesh.conn.reshape(-1, 4)[slug_elements].reshape(-1))
    return float(np.sum(m[nodes] * vr[nodes]) / np.sum(m[nodes]))


def test_perforation_errors_against_fp64(gpu_lib):
    out = {}
    for prec in (_abi.PRECISION_FP64, _abi.PRECISION_MIXED):
        s, mesh, info = scenes.perforation(ExplicitSolver, cell=1.0e-3, gap=0.5e-3)
        s.setPrecision(prec)
        k0 = s.kineticEnergy()
        s.run(1500)
        a = s._auditC()
        w = info["wall"]
        c = info["contact"]
        balance = (a.centred_kinetic_energy + a.strain_energy + a.plastic_dissipation
                   + a.hourglass_energy + s.erodedEnergy() + w.energyLoss()
                   + w.frictionDissipation() + c.dissipation() + c.energy()) / k0
        out[prec] = (_slug_velocity(s, mesh, info["slug"]), s.erodedElements(), balance)
        assert s.statusWord() == 0
    v64, n64, b64 = out[_abi.PRECISION_FP64]
    v32, n32, b32 = out[_abi.PRECISION_MIXED]
    assert abs(v32 - v64) <= 0.01 * abs(v64), (v32, v64)
    assert abs(n32 - n64) <= max(3, 0.05 * n64), (n32, n64)
    assert abs(b32 - b64) <= 0.01, (b32, b64)


def test_precision_switch_and_reads(gpu_lib):
    """Reads, audits and a switch back to FP64 work in mixed mode."""
    s, mesh, _ = scenes.taylor_rod(ExplicitSolver, nr=4, nz=24)
    s.setPrecision(_abi.PRECISION_MIXED)
    s.run(200)
    sig = s.stress()
    assert sig.shape == (4 * mesh.elementCount,) and np.all(np.isfinite(sig))
    assert s.plasticDissipation() > 0.0
    s.setPrecision(_abi.PRECISION_FP64)
    s.run(50)
    assert np.all(np.isfinite(s.stress()))
    assert s.statusWord() == 0
