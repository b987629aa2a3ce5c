"""The adjoint kernel against the FP64 reference adjoint of the oracle, on a small batch."""
import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from neofiz_gb300.batch import BatchSolver
from oracle.oracle import OracleBatch

pytestmark = pytest.mark.gpu


def _rods(t_end=12.0e-6):
    rods = scenes.taylor_sweep(3, seed=21)
    for r, (nr, nz) in zip(rods, [(10, 60), (4, 20), (6, 30)]):
        r["nr"], r["nz"], r["t_end"] = nr, nz, t_end
    return rods


def _grads(cls, rods, every):
    b = cls(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(every)
    out = {obj: b.adjointBackward(obj) for obj in (0, 1)}
    steps = b.state()["steps"].copy()
    uz = b.read(_abi.FIELD_UZ)
    b.close()
    return out, steps, uz


def test_adjoint_kernel_matches_the_reference_adjoint(gpu_lib):
    rods = _rods()
    g, gsteps, guz = _grads(BatchSolver, rods, every=40)
    o, osteps, ouz = _grads(OracleBatch, rods, every=40)
    assert np.array_equal(gsteps, osteps)
    assert np.array_equal(guz, ouz)                 # the forward pass is the plain path
    for obj in (0, 1):
        assert np.array_equal(g[obj][0], o[obj][0])
        # per-thread partial sums and block trees instead of serial sums: rounding only
        np.testing.assert_allclose(g[obj][1], o[obj][1], rtol=1e-9, atol=0.0)


def test_forward_pass_equals_a_plain_run_and_intervals_agree(gpu_lib):
    rods = _rods(t_end=8.0e-6)
    a, asteps, auz = _grads(BatchSolver, rods, every=13)
    b, bsteps, buz = _grads(BatchSolver, rods, every=200)
    assert np.array_equal(asteps, bsteps) and np.array_equal(auz, buz)
    for obj in (0, 1):
        assert np.array_equal(a[obj][1], b[obj][1])
    p = BatchSolver(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    p.run()
    assert np.array_equal(p.read(_abi.FIELD_UZ), auz)
    assert np.array_equal(p.state()["steps"], asteps)


def test_adjoint_rejects_mixed_batches(gpu_lib):
    b = BatchSolver(scenes.sweep_instances(_rods()[:1]), scenes.Formulation.AXISYMMETRIC,
                    cfl=0.6, precision=_abi.PRECISION_MIXED)
    with pytest.raises(ValueError):
        b.adjointForward(50)


def _tubes():
    from neofiz_gb300.materials import JohnsonCook
    a = scenes.tube_material(JohnsonCook.COPPER_OFHC).withKinematicHardening(2.0e8)
    return [scenes.tube_instance(nz=10, height=2.0e-3, t_end=50.0e-6, scale=0.04, material=a),
            scenes.tube_instance(nz=14, height=2.8e-3, t_end=40.0e-6, scale=0.06, seed=11)]


def test_capacity_adjoint_kernel_matches_the_reference_adjoint(gpu_lib):
    """Pressure edges, damping, damage and the sampled capacity peak on the GPU."""
    out = {}
    for cls in (BatchSolver, OracleBatch):
        b = cls(_tubes(), scenes.Formulation.AXISYMMETRIC, cfl=0.5)
        b.adjointForward(64, 10)
        out[cls] = (b.adjointBackward(_abi.OBJECTIVE_PEAK_CAPACITY), b.state()["steps"].copy(),
                    b.read(_abi.FIELD_UR))
        b.close()
    (gv, gg), gs, gu = out[BatchSolver]
    (ov, og), os_, ou = out[OracleBatch]
    assert np.array_equal(gs, os_) and np.array_equal(gu, ou)
    np.testing.assert_allclose(gv, ov, rtol=1e-13)
    assert og[0][_abi.PARAM_FRACTURE_ENERGY] != 0.0
    np.testing.assert_allclose(gg, og, rtol=1e-9, atol=1e-12 * np.abs(og).max())


def test_several_objectives_in_one_pass_are_bit_identical_to_single_passes(gpu_lib):
    """One recompute carries L/L0 and the mushroom diameter (and a tube's capacity): each
    objective's values and gradients equal its own pass bit for bit."""
    rods = _rods(t_end=6.0e-6)
    b = BatchSolver(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(40)
    objs = [_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM]
    v, g = b.adjointBackwardMany(objs)
    for w, obj in enumerate(objs):
        v1, g1 = b.adjointBackward(obj)
        assert np.array_equal(v[w], v1) and np.array_equal(g[w], g1), obj
    b.close()
    t = BatchSolver([scenes.tube_instance(nz=20, t_end=12.0e-6, scale=0.04)],
                    scenes.Formulation.AXISYMMETRIC, cfl=0.5)
    t.adjointForward(50, 5)
    objs = [_abi.OBJECTIVE_PEAK_CAPACITY, _abi.OBJECTIVE_LENGTH_RATIO]
    v, g = t.adjointBackwardMany(objs)
    for w, obj in enumerate(objs):
        v1, g1 = t.adjointBackward(obj)
        assert np.array_equal(v[w], v1) and np.array_equal(g[w], g1), obj


def test_linear_hardening_gradients_match_the_reference_adjoint(gpu_lib):
    """Yield stress and isotropic hardening modulus of a linear-hardening rod: the kernel's
    gradients against the oracle's reference adjoint."""
    import dataclasses as dc
    from neofiz_gb300.materials import Material
    mat = Material("linear steel", 200.0e9, 0.29, 7850.0).yielding(600.0e6, 2.0e9, 3.0e8)
    rods = _rods(t_end=8.0e-6)
    insts = [dc.replace(x, material=mat) for x in scenes.sweep_instances(rods)]
    out = {}
    for cls in (BatchSolver, OracleBatch):
        b = cls(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.6)
        b.adjointForward(25)
        out[cls] = [b.adjointBackward(obj) for obj in (0, 1)]
        b.close()
    for obj in (0, 1):
        g, o = out[BatchSolver][obj], out[OracleBatch][obj]
        assert np.array_equal(g[0], o[0])
        np.testing.assert_allclose(g[1], o[1], rtol=1e-9, atol=0.0)
        assert np.all(g[1][:, _abi.PARAM_YIELD] != 0.0)


def _fd_full_run(cls, rod, steps, names, h=1.0e-6):
    """Central differences of L/L0 and the mushroom diameter after `steps` steps of the plain
    path, one parameter at a time, the perturbed rods run as one batch."""
    import dataclasses
    jc0 = scenes._rod_jc(rod)
    mat0 = scenes.rod_material_with(jc0)
    p0 = {"A": jc0.a, "B": jc0.b, "n": jc0.n, "C": jc0.c, "m": jc0.m,
          "kinematic": mat0.kinematicHardening, "friction": rod["mu"]}
    insts = []
    for name in names:
        for sgn in (1.0, -1.0):
            inst = scenes.sweep_instances([rod])[0]
            val = p0[name] * (1.0 + sgn * h)
            if name in ("A", "B", "n", "C", "m"):
                f = {"A": "a", "B": "b", "n": "n", "C": "c", "m": "m"}[name]
                inst.material = scenes.rod_material_with(
                    dataclasses.replace(jc0, **{f: val})).withKinematicHardening(
                        mat0.kinematicHardening)
            elif name == "kinematic":
                inst.material = mat0.withKinematicHardening(val)
            else:
                inst.wall = (0.0, val)
            inst.t_end = 1.0
            insts.append(inst)
    b = cls(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.run(max_steps=steps)
    m = b.measure()
    b.close()
    return {name: ((m[2 * k].length - m[2 * k + 1].length) / 25.0e-3 / (2.0 * p0[name] * h),
                   (m[2 * k].mushroom_diameter - m[2 * k + 1].mushroom_diameter)
                   / (2.0 * p0[name] * h)) for k, name in enumerate(names)}


def test_full_run_gradients_match_central_differences(gpu_lib):
    """The 10 x 60 rod of the gradient batch over its whole 80 us (about 3800 steps): the
    kernel's gradients of L/L0 and of the mushroom diameter with respect to A, B, n, C, m, the
    kinematic modulus and the wall friction against central differences of the plain path
    (h = 1e-6 relative), within 1e-4 (the bar for gradients is 1e-3)."""
    rod = scenes.adjoint_rods(1)[0]
    b = BatchSolver(scenes.sweep_instances([rod]), scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.adjointForward(200)
    steps = int(b.state()["steps"][0])
    grads = {obj: b.adjointBackward(obj)[1][0] for obj in (0, 1)}
    b.close()
    assert steps > 3000
    names = ("A", "B", "n", "C", "m", "kinematic", "friction")
    fd = _fd_full_run(BatchSolver, rod, steps, names)
    for k, name in enumerate(names):
        for obj in (0, 1):
            ad, ref = grads[obj][k], fd[name][obj]
            assert abs(ad - ref) <= 1e-4 * abs(ref), (name, obj, ad, ref)
