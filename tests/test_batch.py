"""The batched surface on the CPU: the sweep generator, and the oracle's batch (one solver per
instance over a thread pool, as Sweep.over runs a sweep) against the same scenes run one by
one."""
import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from oracle.oracle import OracleBatch, OracleSolver


def test_sweep_draws_are_seeded_and_in_range():
    a = scenes.taylor_sweep(512)
    b = scenes.taylor_sweep(512)
    assert a == b
    assert a != scenes.taylor_sweep(512, seed=scenes.SWEEP_SEED + 1)
    nr = [r["nr"] for r in a]
    nz = [r["nz"] for r in a]
    assert min(nr) == 6 and max(nr) == 24 and min(nz) == 30 and max(nz) == 120
    j = scenes.ROD_JC
    for r in a:
        assert 0.8 * j.a <= r["a"] <= 1.2 * j.a and 0.8 * j.b <= r["b"] <= 1.2 * j.b
        assert 0.8 * j.n <= r["n"] <= 1.2 * j.n and 0.8 * j.c <= r["c"] <= 1.2 * j.c
        assert 0.0 <= r["mu"] <= 0.2 and 150.0 <= r["speed"] <= 250.0
    assert 1000 < np.mean([r["nr"] * r["nz"] for r in a]) < 1250


def test_splitmix64_known_sequence():
    """First outputs for seed 0 of the published generator (the same finaliser as
    java.util.SplittableRandom)."""
    g = scenes.SplitMix64(0)
    assert [g.next() for _ in range(3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4,
                                            0x06C45D188009454F]


def _small_rods(t_end=4.0e-6):
    rods = scenes.taylor_sweep(3, seed=7)
    for r, (nr, nz) in zip(rods, [(3, 12), (4, 15), (2, 9)]):
        r["nr"], r["nz"], r["t_end"] = nr, nz, t_end
    return rods


def test_oracle_batch_equals_single_scenes():
    rods = _small_rods()
    b = OracleBatch(scenes.sweep_instances(rods), scenes.Formulation.AXISYMMETRIC,
                    cfl=0.6)
    b.run()
    st = b.state()
    meas = b.measure()
    for k, rod in enumerate(rods):
        s, mesh, info = scenes.sweep_rod(OracleSolver, rod)
        s.runUntil(rod["t_end"])
        assert st["steps"][k] == s.steps() and st["time"][k] == s.time()
        for field in (_abi.FIELD_UR, _abi.FIELD_UZ, _abi.FIELD_VR, _abi.FIELD_VZ):
            assert np.array_equal(b.readInstance(field, k), s.readField(field))
        assert np.array_equal(b.readInstance(_abi.FIELD_STRESS, k), s.readField(_abi.FIELD_STRESS))
        m = s.measure()
        assert (meas[k].length, meas[k].mushroom_diameter) == (m.length, m.mushroom_diameter)
    b.close()


def test_batch_rejects_bad_input():
    rods = _small_rods()
    inst = scenes.sweep_instances(rods)
    inst[1].hourglass = -1.0
    with pytest.raises(ValueError):
        OracleBatch(inst, scenes.Formulation.AXISYMMETRIC)


def test_oracle_batch_tube_equals_single_scene():
    """Pressure edges, relaxation damping and damage through the batch surface."""
    from neofiz_gb300 import Integration
    inst = scenes.tube_instance(t_end=8.0e-6)
    b = OracleBatch([inst, scenes.tube_instance(t_end=6.0e-6, seed=9)],
                    scenes.Formulation.AXISYMMETRIC, cfl=0.5)
    b.run()
    s, mesh, _ = scenes.tube(OracleSolver, integration=Integration.REDUCED)
    s.runUntil(8.0e-6)
    assert b.state()["steps"][0] == s.steps()
    for f in (_abi.FIELD_UR, _abi.FIELD_UZ, _abi.FIELD_VR, _abi.FIELD_STRESS,
              _abi.FIELD_PLASTIC_STRAIN):
        assert np.array_equal(b.readInstance(f, 0), s.readField(f)), f
