"""The batched kernel against the same scenes run one at a time on the GPU, and against the
oracle's sweep. An instance's trajectory must be bit-identical to its single-scene twin in the
same precision, under every launch shape the autotuner can pick."""
import numpy as np
import pytest

from neofiz_gb300 import ExplicitSolver, _abi, scenes
from neofiz_gb300.batch import BatchSolver
from oracle.oracle import OracleBatch

pytestmark = pytest.mark.gpu

FIELDS = (_abi.FIELD_UR, _abi.FIELD_UZ, _abi.FIELD_VR, _abi.FIELD_VZ, _abi.FIELD_FR,
          _abi.FIELD_FZ, _abi.FIELD_STRESS, _abi.FIELD_BACK_STRESS, _abi.FIELD_PLASTIC_STRAIN,
          _abi.FIELD_PLASTIC_WORK, _abi.FIELD_HOURGLASS_R, _abi.FIELD_HOURGLASS_Z)


def _rods(count=6, t_end=12.0e-6, seed=11):
    """A few drawn rods, the largest (24 x 120) among them, run for t_end."""
    rods = scenes.taylor_sweep(count, seed=seed)
    rods[0]["nr"], rods[0]["nz"] = 24, 120
    rods[1]["nr"], rods[1]["nz"] = 6, 30
    for r in rods:
        r["t_end"] = t_end
    return rods


def _batch(rods, precision, cls=BatchSolver):
    return cls(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC, cfl=0.6,
               precision=precision)


def _single(rod, precision):
    s, mesh, info = scenes.sweep_rod(ExplicitSolver, rod)
    s.setPrecision(precision)
    s.runUntil(rod["t_end"])
    return s


def _assert_matches_single(b, rods, precision):
    st = b.state()
    meas = b.measure()
    walls = b.wallStats()
    assert not st["status"].any()
    for k, rod in enumerate(rods):
        s = _single(rod, precision)
        assert st["steps"][k] == s.steps(), k
        assert st["time"][k] == s.time(), k
        assert st["timestep"][k] == s.timestep(), k
        for f in FIELDS:
            got, want = b.readInstance(f, k), s.readField(f)
            assert np.array_equal(got, want), (k, f, np.max(np.abs(got - want)))
        m = s.measure()
        assert (meas[k].length, meas[k].mushroom_diameter) == (m.length, m.mushroom_diameter)
        w = s._wallInfo()
        assert (walls[k].contact_count, walls[k].stuck_count) == (w.contact_count, w.stuck_count)
        # the audit totals are summed in another tree: equal to rounding
        assert walls[k].impulse == pytest.approx(w.impulse, rel=1e-12, abs=1e-18)


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_batch_equals_single_scenes(gpu_lib, precision):
    rods = _rods()
    b = _batch(rods, precision)
    b.run()
    assert b.state()["done"].all()
    _assert_matches_single(b, rods, precision)
    b.close()


def test_one_warp_blocks_keep_fp64_bits(gpu_lib):
    """32-thread blocks (for small instances) step the same FP64 trajectories."""
    rods = _rods(count=3, t_end=4.0e-6, seed=23)
    b = _batch(rods, _abi.PRECISION_FP64)
    b.setConfig(32, 0, 8, 40)
    b.run()
    _assert_matches_single(b, rods, _abi.PRECISION_FP64)
    b.close()


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_COMPENSATED])
def test_every_launch_shape_gives_the_same_trajectory(gpu_lib, precision):
    """The mixed form: every shape, bit for bit. The compensated form (its own fast-float
    translation unit, no bit-level twin): bit for bit across 128- and 256-thread blocks and
    across chunking and staging; its one-warp kernels are compiled separately and agree to
    float rounding (displacements within 1e-6 of their largest)."""
    rods = _rods(count=5, t_end=6.0e-6, seed=3)
    ref = None
    shapes = [(128, 0, 1, 7), (256, 0, 2, 64), (256, 1, 1, 1000), (128, 1, 2, 33), (32, 0, 8, 50),
              (32, 1, 2, 19)]
    warp = None
    for threads, stage, bps, chunk in shapes:
        b = _batch(rods, precision)
        b.setConfig(threads, stage, bps, chunk)
        b.run()
        out = [b.read(f) for f in FIELDS]
        b.close()
        if ref is None:
            ref = out
            continue
        if precision == _abi.PRECISION_COMPENSATED and threads == 32:
            for f, x, y in zip(FIELDS[:2], out[:2], ref[:2]):     # displacements
                np.testing.assert_allclose(x, y, rtol=0.0, atol=1e-6 * np.abs(y).max())
            if warp is None:
                warp = out
            else:                                        # one-warp shapes among themselves
                for f, x, y in zip(FIELDS, out, warp):
                    assert np.array_equal(x, y), (threads, stage, bps, chunk, f)
            continue
        for f, x, y in zip(FIELDS, out, ref):
            assert np.array_equal(x, y), (threads, stage, bps, chunk, f)


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_COMPENSATED])
def test_autotuner_keeps_the_state(gpu_lib, precision):
    """Tuning runs trial steps on saved state; the run afterwards matches an untuned one."""
    rods = _rods(count=4, t_end=5.0e-6, seed=5)
    a = _batch(rods, precision)
    cfg = a.tune(trial_steps=16)
    assert cfg["threads"] in (128, 256) and cfg["blocks_per_sm"] >= 1
    a.run()
    b = _batch(rods, precision)
    b.run()
    for f in FIELDS:
        assert np.array_equal(a.read(f), b.read(f)), f
    assert np.array_equal(a.state()["steps"], b.state()["steps"])
    a.close()
    b.close()


def test_batch_fp64_equals_the_oracle_sweep(gpu_lib):
    rods = _rods(count=3, t_end=3.0e-6, seed=9)
    rods[0]["nr"], rods[0]["nz"] = 8, 40
    g = _batch(rods, _abi.PRECISION_FP64)
    g.run()
    o = _batch(rods, _abi.PRECISION_FP64, cls=OracleBatch)
    o.run()
    assert np.array_equal(g.state()["steps"], o.state()["steps"])
    for f in FIELDS:
        assert np.array_equal(g.read(f), o.read(f)), f
    g.close()
    o.close()


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_COMPENSATED])
def test_partial_runs_resume_exactly(gpu_lib, precision):
    """run(max_steps) in pieces equals one run to t_end."""
    rods = _rods(count=4, t_end=4.0e-6, seed=13)
    a = _batch(rods, precision)
    for _ in range(50):
        a.run(max_steps=37)
        if a.state()["done"].all():
            break
    b = _batch(rods, precision)
    b.run()
    assert np.array_equal(a.state()["steps"], b.state()["steps"])
    for f in FIELDS:
        assert np.array_equal(a.read(f), b.read(f)), f


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_COMPENSATED])
def test_length_ratio_within_1e4_of_fp64(gpu_lib, precision):
    """The bar for the batched reduced-precision forms: L/L0 within 1e-4 relative of FP64, over
    a full 80 us impact."""
    rods = _rods(count=6, t_end=80.0e-6, seed=17)
    lengths = {}
    for prec in (_abi.PRECISION_FP64, precision):
        b = _batch(rods, prec)
        b.run()
        assert not b.state()["status"].any()
        lengths[prec] = np.array([m.length for m in b.measure()])
        b.close()
    l64, l32 = lengths[_abi.PRECISION_FP64], lengths[precision]
    assert np.all(np.abs(l32 - l64) <= 1e-4 * l64), np.abs(l32 - l64) / l64


def test_compensated_tube_tracks_fp64(gpu_lib):
    """Pressure edges, damping and damage in the compensated form: the bore's radial
    displacement within 1e-3 of FP64 after 25 us, damage on, no non-finite state."""
    insts = [scenes.tube_instance(t_end=25.0e-6, scale=0.04)]
    out = {}
    for prec in (_abi.PRECISION_FP64, _abi.PRECISION_COMPENSATED):
        b = BatchSolver(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.5, precision=prec)
        b.run()
        assert not b.state()["status"].any()
        out[prec] = b.read(_abi.FIELD_UR)
        b.close()
    a, c = out[_abi.PRECISION_FP64], out[_abi.PRECISION_COMPENSATED]
    assert np.max(np.abs(c - a)) <= 1e-3 * np.max(np.abs(a))


def test_compensated_is_a_batch_form(gpu_lib):
    s, _, _ = scenes.sweep_rod(ExplicitSolver, _rods(count=2)[1])
    with pytest.raises(ValueError):
        s.setPrecision(_abi.PRECISION_COMPENSATED)


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_batch_tube_equals_single_scene(gpu_lib, precision):
    """Pressure edges, relaxation damping and damage: the batched tube is the single tube."""
    from neofiz_gb300 import Integration
    # failure strains Weibull(0.04, 10): damage begins well before 25 us
    insts = [scenes.tube_instance(t_end=25.0e-6, scale=0.04),
             scenes.tube_instance(t_end=20.0e-6, seed=3, nz=12, scale=0.04)]
    b = BatchSolver(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.5, precision=precision)
    b.run()
    s, mesh, _ = scenes.tube(ExplicitSolver, integration=Integration.REDUCED, scale=0.04)
    s.setPrecision(precision)
    s.runUntil(25.0e-6)
    assert b.state()["steps"][0] == s.steps()
    assert s._auditC().max_damage > 0.0 or precision == _abi.PRECISION_MIXED
    for f in FIELDS:
        assert np.array_equal(b.readInstance(f, 0), s.readField(f)), f
