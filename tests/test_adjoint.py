"""The FP64 reference adjoint (oracle) on the CPU: gradients of L/L0 and of the mushroom
diameter after N steps, against central finite differences of the plain path run for the same
N steps, and independent of the checkpoint interval.

Over a short run (a few hundred steps) the measurement is smooth in the parameters and central
differences with h = 1e-6 relative agree with the adjoint to about 1e-7; the bar here is 1e-5.
Over thousands of steps the frozen decisions (elastic or plastic points, stick or slip) switch
under any finite perturbation and the difference quotients scatter by ~1e-4 with h, which is
why the long-run comparison lives in the benchmark, with that scatter reported beside it."""
import dataclasses

import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from oracle.oracle import OracleBatch, OracleSolver

H = 1.0e-6


def _rod(t_end=10.0e-6, nr=3, nz=12):
    rod = scenes.taylor_sweep(1, seed=5)[0]
    rod.update(nr=nr, nz=nz, t_end=t_end, mu=0.09, speed=200.0)
    return rod


def _gradients(rod, every):
    b = OracleBatch(scenes.sweep_instances([rod]), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(every)
    steps = int(b.state()["steps"][0])
    out = {}
    for obj in (_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM):
        v, g = b.adjointBackward(obj)
        out[obj] = (v[0], g[0])
    b.close()
    return steps, out


def _measure(rod, steps, pname=None, value=None):
    jc0 = scenes._rod_jc(rod)
    mat0 = scenes.rod_material_with(jc0)
    mat, mu = mat0, rod["mu"]
    if pname in ("A", "B", "n", "C", "m"):
        field = {"A": "a", "B": "b", "n": "n", "C": "c", "m": "m"}[pname]
        jc = dataclasses.replace(jc0, **{field: value})
        mat = scenes.rod_material_with(jc).withKinematicHardening(mat0.kinematicHardening)
    elif pname == "kinematic":
        mat = mat0.withKinematicHardening(value)
    elif pname == "friction":
        mu = value
    s, mesh, info = scenes.taylor_rod(OracleSolver, nr=rod["nr"], nz=rod["nz"],
                                      speed=rod["speed"], friction=mu, material=mat)
    s.run(steps)
    m = s.measure()
    return np.array([m.length / info["length"], m.mushroom_diameter])


def test_reference_adjoint_matches_central_differences():
    rod = _rod()
    steps, grads = _gradients(rod, every=20)
    base = _measure(rod, steps)
    assert grads[_abi.OBJECTIVE_LENGTH_RATIO][0] == pytest.approx(base[0], rel=1e-14)
    assert grads[_abi.OBJECTIVE_MUSHROOM][0] == pytest.approx(base[1], rel=1e-14)
    jc0 = scenes._rod_jc(rod)
    p0 = {"A": jc0.a, "B": jc0.b, "n": jc0.n, "C": jc0.c, "m": jc0.m,
          "kinematic": scenes.rod_material_with(jc0).kinematicHardening, "friction": rod["mu"]}
    for k, name in enumerate(_abi.PARAM_NAMES):
        dp = H * p0[name]
        fd = (_measure(rod, steps, name, p0[name] + dp)
              - _measure(rod, steps, name, p0[name] - dp)) / (2.0 * dp)
        for obj in (0, 1):
            ad = grads[obj][1][k]
            assert ad == pytest.approx(fd[obj], rel=1e-5), (name, obj, ad, fd[obj])


def test_gradients_do_not_depend_on_the_checkpoint_interval():
    rod = _rod(t_end=6.0e-6)
    ref = None
    for every in (1, 7, 1000):
        steps, grads = _gradients(rod, every)
        if ref is None:
            ref = grads
        for obj in grads:
            assert grads[obj][0] == ref[obj][0]
            assert np.array_equal(grads[obj][1], ref[obj][1]), (every, obj)


def test_adjoint_needs_a_fresh_fp64_batch():
    rod = _rod(t_end=2.0e-6)
    b = OracleBatch(scenes.sweep_instances([rod]), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    with pytest.raises(RuntimeError):
        b.adjointBackward(_abi.OBJECTIVE_LENGTH_RATIO)
    b.run()
    with pytest.raises(RuntimeError):
        b.adjointForward(10)
