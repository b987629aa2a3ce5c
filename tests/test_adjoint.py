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
    for k, name in enumerate(_abi.PARAM_NAMES[:7]):
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


def _tube_law():
    """Copper with rate and thermal terms (C, m, Taylor-Quinney) and kinematic hardening, so
    every parameter of the capacity gradient is exercised."""
    from neofiz_gb300.materials import JohnsonCook
    return JohnsonCook.COPPER_OFHC


def _tube(name=None, value=None, t_end=50.0e-6):
    law = _tube_law()
    hkin = 2.0e8
    gf = scenes.TUBE_GF
    if name in ("A", "B", "n", "C", "m"):
        field = {"A": "a", "B": "b", "n": "n", "C": "c", "m": "m"}[name]
        law = dataclasses.replace(law, **{field: value})
    elif name == "kinematic":
        hkin = value
    elif name == "fracture_energy":
        gf = value
    mat = scenes.tube_material(law).withKinematicHardening(hkin)
    return scenes.tube_instance(nz=10, height=2.0e-3, t_end=t_end, scale=0.04, material=mat, gf=gf)


def _capacity(name=None, value=None):
    b = OracleBatch([_tube(name, value)], scenes.Formulation.AXISYMMETRIC, cfl=0.5)
    b.adjointForward(64, 10)
    v, g = b.adjointBackward(_abi.OBJECTIVE_PEAK_CAPACITY)
    b.close()
    return v[0], g[0]


def test_capacity_gradient_matches_central_differences():
    """The tube: pressure edges with a smoothstep ramp, relaxation damping and damage that
    begins before the capacity peak; the peak sampled every 10 steps."""
    value, grad = _capacity()
    law = _tube_law()
    p0 = {"A": law.a, "B": law.b, "n": law.n, "C": law.c, "m": law.m, "kinematic": 2.0e8,
          "fracture_energy": scenes.TUBE_GF}
    assert grad[_abi.PARAM_FRACTURE_ENERGY] != 0.0        # damage shapes the peak
    assert grad[_abi.PARAM_FRICTION] == 0.0               # no wall
    for k, name in enumerate(_abi.PARAM_NAMES):
        if name not in p0:
            continue
        dp = H * p0[name]
        fd = (_capacity(name, p0[name] + dp)[0] - _capacity(name, p0[name] - dp)[0]) / (2 * dp)
        assert grad[k] == pytest.approx(fd, rel=1e-4), (name, grad[k], fd)


def test_fraction_convention_is_the_chain_rule():
    """(A, B, n, C, m, H_kin, mu, Gf) -> (A, B, n, C, m, mu, f, Gf) with H_kin = f B e^n / e:
    the kinematic column by its three dependencies, the others carried over."""
    rod = scenes.taylor_sweep(1, seed=5)[0]
    g = np.arange(1.0, 9.0)
    out = scenes.fraction_gradients(g, rod)
    e, f, b, n = scenes.ROD_FIT_STRAIN, scenes.ROD_KINEMATIC_FRACTION, rod["b"], rod["n"]

    def hkin(bb, nn, ff):
        return ff * bb * e ** nn / e

    h = 1e-7
    dHdB = (hkin(b * (1 + h), n, f) - hkin(b * (1 - h), n, f)) / (2 * b * h)
    dHdn = (hkin(b, n * (1 + h), f) - hkin(b, n * (1 - h), f)) / (2 * n * h)
    dHdf = (hkin(b, n, f * (1 + h)) - hkin(b, n, f * (1 - h))) / (2 * f * h)
    np.testing.assert_allclose(out[[0, 3, 4]], g[[0, 3, 4]])
    np.testing.assert_allclose(out[1], g[1] + g[5] * dHdB, rtol=1e-7)
    np.testing.assert_allclose(out[2], g[2] + g[5] * dHdn, rtol=1e-7)
    assert out[5] == g[6] and out[7] == g[7]
    np.testing.assert_allclose(out[6], g[5] * dHdf, rtol=1e-7)


def test_several_objectives_in_one_pass_match_single_passes():
    """backward_many([L/L0, mushroom]) on the reference adjoint gives the single passes'
    values and gradients."""
    rods = scenes.adjoint_rods(2)
    for r in rods:
        r["nr"], r["nz"], r["t_end"] = 4, 20, 4.0e-6
    b = OracleBatch(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(17)
    v, g = b.adjointBackwardMany([_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM])
    for w, obj in enumerate((_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM)):
        v1, g1 = b.adjointBackward(obj)
        assert np.array_equal(v[w], v1) and np.array_equal(g[w], g1)
    with pytest.raises(ValueError):
        b.adjointBackwardMany([0, 1, 2, 0])


def _linear_rod_material(sy0=600.0e6, h_iso=2.0e9, h_kin=3.0e8):
    """A J2 steel with linear isotropic and kinematic hardening (no Johnson-Cook law)."""
    from neofiz_gb300.materials import Material
    return Material("linear steel", 200.0e9, 0.29, 7850.0).yielding(sy0, h_iso, h_kin)


def _linear_measure(mat, steps):
    s, mesh, info = scenes.taylor_rod(OracleSolver, nr=3, nz=12, speed=250.0, friction=0.09,
                                      material=mat)
    s.run(steps)
    m = s.measure()
    return np.array([m.length / info["length"], m.mushroom_diameter])


def test_yield_and_isotropic_hardening_gradients_match_central_differences():
    """The hardening moduli of a linear-hardening material (no Johnson-Cook law): d/d sy0 and
    d/d H_iso (and H_kin) against central differences of the plain path."""
    import dataclasses as dc
    mat = _linear_rod_material()
    inst = scenes.sweep_instances([dict(nr=3, nz=12, t_end=8.0e-6, mu=0.09, speed=250.0,
                                        a=1.0, b=1.0, n=0.5, c=0.0)])[0]
    inst = dc.replace(inst, material=mat)
    b = OracleBatch([inst], scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(15)
    steps = int(b.state()["steps"][0])
    grads = {obj: b.adjointBackward(obj)[1][0] for obj in (0, 1)}
    base = {"yield": mat.yieldStress, "isotropic": mat.isotropicHardening,
            "kinematic": mat.kinematicHardening}
    for name, k in (("yield", _abi.PARAM_YIELD), ("isotropic", _abi.PARAM_ISOTROPIC),
                    ("kinematic", _abi.PARAM_KINEMATIC)):
        dp = H * base[name]
        def at(v):
            p = dict(base)
            p[name] = v
            return _linear_measure(_linear_rod_material(p["yield"], p["isotropic"],
                                                        p["kinematic"]), steps)
        fd = (at(base[name] + dp) - at(base[name] - dp)) / (2.0 * dp)
        for obj in (0, 1):
            assert grads[obj][k] == pytest.approx(fd[obj], rel=1e-5), (name, obj)
    # a Johnson-Cook rod has no yield or isotropic-hardening dependence
    rod = _rod()
    _, jc = _gradients(rod, every=20)
    assert jc[0][1][_abi.PARAM_YIELD] == 0.0 and jc[0][1][_abi.PARAM_ISOTROPIC] == 0.0


def test_full_run_gradients_match_central_differences_on_the_oracle():
    """The reference adjoint over the 10 x 60 rod's whole 80 us run (about 3800 steps, every
    kind of frozen decision switching many times): d(L/L0) and d(mushroom) with respect to
    the wall friction, n and C against central differences (h = 1e-6 relative) within 1e-4.
    The reverse solves the return map to its converged root; at the forward's tolerance the
    friction gradient of L/L0 was off by 3.4e-3 over this run."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "adjoint_gpu_helpers", os.path.join(os.path.dirname(__file__), "test_adjoint_gpu.py"))
    helpers = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(helpers)
    rod = scenes.adjoint_rods(1)[0]
    b = OracleBatch(scenes.sweep_instances([rod]), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(200)
    steps = int(b.state()["steps"][0])
    grads = {obj: b.adjointBackward(obj)[1][0] for obj in (0, 1)}
    b.close()
    names = ("friction", "n", "C")
    fd = helpers._fd_full_run(OracleBatch, rod, steps, names)
    for name in names:
        k = _abi.PARAM_NAMES.index(name)
        for obj in (0, 1):
            ad, ref = grads[obj][k], fd[name][obj]
            assert abs(ad - ref) <= 1e-4 * abs(ref), (name, obj, ad, ref)
