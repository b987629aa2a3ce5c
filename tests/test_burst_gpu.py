"""The burst measurement in the batched kernel against the oracle's batch: FP64 bit for bit
to the traversed peak; the compensated form within its error."""
import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from neofiz_gb300.batch import BatchSolver
from oracle.oracle import OracleBatch

pytestmark = pytest.mark.gpu


def _tubes():
    return [scenes.burst_instance(slenderness=s) for s in (25.0, 32.0, 40.0)]


def _run(cls, precision):
    b = cls(_tubes(), scenes.Formulation.AXISYMMETRIC, cfl=scenes.BURST_CFL, precision=precision)
    b.setBurst(scenes.BURST_SAMPLE_STEPS, 25.0e-3, scenes.BURST_PEAK_MARGIN, traceCapacity=2000)
    b.run()
    return b.burstResults(), b.burstTrace(), b.state()


def test_fp64_burst_batch_equals_the_oracle(gpu_lib):
    g, gt, gs = _run(BatchSolver, _abi.PRECISION_FP64)
    o, ot, os_ = _run(OracleBatch, _abi.PRECISION_FP64)
    assert g["traversed"].all() and o["traversed"].all()
    for k in g:
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(gt, ot)
    assert np.array_equal(gs["steps"], os_["steps"]) and gs["done"].all()
    # the measured burst sits within 1 % of the thin-wall closed form (BurstCase's audit)
    for k, inst in enumerate(_tubes()):
        exact = inst.pressure[0] / scenes.BURST_OVERSHOOT
        assert abs(g["peak_capacity"][k] / exact - 1.0) < 0.01


def test_compensated_burst_tracks_fp64(gpu_lib):
    g, _, _ = _run(BatchSolver, _abi.PRECISION_FP64)
    c, _, _ = _run(BatchSolver, _abi.PRECISION_COMPENSATED)
    assert c["traversed"].all()
    np.testing.assert_allclose(c["peak_capacity"], g["peak_capacity"], rtol=1e-4)
    np.testing.assert_allclose(c["peak_strain"], g["peak_strain"], rtol=1e-2)
