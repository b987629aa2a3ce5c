"""The adjoint behind its forward/backward function interface (neofiz_gb300.adjoint, the twin
of the Java binding's GpuAdjoint): forward returns each case's objective, backward(seed) the
seed-weighted gradients; on a short run the gradients equal central differences of forward
itself, on the oracle (CPU) and on the device."""
import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from neofiz_gb300.adjoint import AdjointFunction, rod_parameters, rod_template


def _rods(n=3, t_end=8.0e-6):
    rods = scenes.taylor_sweep(n, seed=11, t_end=t_end)
    for r in rods:
        r.update(nr=3, nz=12, speed=200.0)
    return rods


def _check(batch_class, objective):
    rods = _rods()
    params = rod_parameters(rods)
    f = AdjointFunction(rod_template(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6,
                        objective=objective, checkpoint_every=50, batch_class=batch_class)
    y = f(params)
    seed = np.array([1.0, -2.0, 0.5])
    g = f.backward(seed)
    ones = f.backward(np.ones(3))
    assert g.shape == (3, len(_abi.PARAM_NAMES))
    assert np.array_equal(g, seed[:, None] * ones)
    # the same objective and gradients as the batch's own adjoint entry points
    b = batch_class(rod_template(rods)(params), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(50)
    v, grads = b.adjointBackward(objective)
    b.close()
    assert np.allclose(y, v, rtol=1e-14, atol=0.0)
    assert np.array_equal(ones, grads)
    # central differences of forward itself (the steps are fixed by the unperturbed run's
    # step count only through t_end, so keep the perturbations small)
    steps = None
    for k, name in enumerate(("A", "B", "n", "C", "m", "kinematic", "friction")):
        h = 1.0e-6 * params[:, k]
        pp, pm = params.copy(), params.copy()
        pp[:, k] += h
        pm[:, k] -= h
        fd = (f(pp) - f(pm)) / (2.0 * h)
        assert np.allclose(ones[:, k], fd, rtol=2e-4, atol=1e-12), (name, ones[:, k], fd)
    f.close()
    return y, ones


@pytest.mark.parametrize("objective", [_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM])
def test_function_on_the_oracle(objective):
    from oracle.oracle import OracleBatch
    _check(OracleBatch, objective)


@pytest.mark.gpu
@pytest.mark.parametrize("objective", [_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM])
def test_function_on_the_device_matches_the_oracle(gpu_lib, objective):
    from neofiz_gb300.batch import BatchSolver
    from oracle.oracle import OracleBatch
    yd, gd = _check(BatchSolver, objective)
    rods = _rods()
    fo = AdjointFunction(rod_template(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6,
                         objective=objective, checkpoint_every=50, batch_class=OracleBatch)
    yo = fo(rod_parameters(rods))
    go = fo.backward(np.ones(3))
    assert np.array_equal(yd, yo)
    assert np.allclose(gd, go, rtol=1e-9, atol=1e-300)
