"""Parity of the CUDA path with the oracle, through the C ABI, on the same inputs.

The bar is bit-identical nodal, stress and history fields, and identical eroded, contact-pair,
stick/slip and wall-state sets: the kernels evaluate the reference's expressions in its order
with no fused multiply-add, and share the oracle's deterministic transcendental functions, so
any difference at all is a defect. Running totals (wall impulse, contact energy and
dissipation, eroded energy, the audits) are reduced in a fixed tree order on the device rather
than serially, so they are compared to 1e-12 relative.
"""
import math
import os

import numpy as np
import pytest

from neofiz_gb300 import (Contact, ExplicitSolver, Formulation, Integration, JohnsonCook,
                          Kinematics, Material, Outline, QuadMesh, RigidWall, _abi, scenes)
from neofiz_gb300.solver import material_point_update
from oracle.oracle import OracleSolver, api as oracle_api

pytestmark = pytest.mark.gpu

BITWISE = {
    "ur": _abi.FIELD_UR, "uz": _abi.FIELD_UZ, "vr": _abi.FIELD_VR, "vz": _abi.FIELD_VZ,
    "fr": _abi.FIELD_FR, "fz": _abi.FIELD_FZ, "mass": _abi.FIELD_MASS,
    "stress": _abi.FIELD_STRESS, "back": _abi.FIELD_BACK_STRESS,
    "eps": _abi.FIELD_PLASTIC_STRAIN, "work": _abi.FIELD_PLASTIC_WORK,
    "hgr": _abi.FIELD_HOURGLASS_R, "hgz": _abi.FIELD_HOURGLASS_Z,
    "hgk": _abi.FIELD_HOURGLASS_STIFFNESS,
    "dstrength": _abi.FIELD_DAMAGE_STRENGTH, "dsoft": _abi.FIELD_DAMAGE_SOFTENING,
    "dwidth": _abi.FIELD_DAMAGE_WIDTH,
    "eroded": _abi.FIELD_ERODED, "on_wall": _abi.FIELD_ON_WALL,
    "wall_state": _abi.FIELD_WALL_STATE, "contact_master": _abi.FIELD_CONTACT_MASTER,
    "contact_state": _abi.FIELD_CONTACT_STATE, "surface_edges": _abi.FIELD_SURFACE_EDGES,
    "surface_nodes": _abi.FIELD_SURFACE_NODES, "fixed": _abi.FIELD_FIXED,
}
REL = 1e-12   # tolerance for tree-reduced running totals of small scenes
EPS = 2.0 ** -53


def sum_tol(n_terms):
    """Relative bound for two summation orders of n same-sign terms: each order is within
    (n - 1) eps of the exact sum, so they differ by at most 2 (n - 1) eps."""
    return max(REL, 2.0 * n_terms * EPS)


def assert_bitwise(g, o, label):
    for name, f in BITWISE.items():
        a, b = g.readField(f), o.readField(f)
        assert a.shape == b.shape, f"{label}: {name} shape {a.shape} vs {b.shape}"
        if a.dtype == np.float64:
            ok = np.array_equal(a.view(np.uint64), b.view(np.uint64))
        else:
            ok = np.array_equal(a, b)
        if not ok:
            bad = np.nonzero(a != b)[0]
            raise AssertionError(f"{label}: {name} differs at {bad.size} entries, first "
                                 f"{bad[:5].tolist()}: {a[bad[:3]]} vs {b[bad[:3]]}")
    sg, so = g._state(), o._state()
    for k in ("time", "timestep", "timestep_previous", "reference_timestep", "mass_scale",
              "min_edge_squared", "steps", "eroded_elements", "inverted_elements"):
        assert getattr(sg, k) == getattr(so, k), f"{label}: state {k}"
    assert g.statusWord() == 0


def close(a, b, rel=REL, floor=1e-300):
    return abs(a - b) <= rel * max(abs(a), abs(b), floor)


def assert_totals(g, o, label):
    n_nodes = g._state().node_count
    n_elems = g._state().element_count * g._state().points_per_element
    rel_n, rel_e = sum_tol(n_nodes), sum_tol(n_elems)
    wg, wo = g._wallInfo(), o._wallInfo()
    assert wg.contact_count == wo.contact_count and wg.stuck_count == wo.stuck_count, label
    for k in ("impulse", "energy_loss", "friction_dissipation"):
        assert close(getattr(wg, k), getattr(wo, k), rel_n), f"{label}: wall {k}"
    cg, co = g._contactInfo(), o._contactInfo()
    assert (cg.pair_count, cg.escaped_nodes, cg.segment_count) == \
        (co.pair_count, co.escaped_nodes, co.segment_count), label
    assert cg.max_penetration == co.max_penetration, label
    for k in ("energy", "dissipation"):
        assert close(getattr(cg, k), getattr(co, k), rel_n), f"{label}: contact {k}"
    assert close(g.erodedEnergy(), o.erodedEnergy(), rel_e), label
    ag, ao = g._auditC(), o._auditC()
    for k in ("kinetic_energy", "centred_kinetic_energy"):
        assert close(getattr(ag, k), getattr(ao, k), rel_n, floor=1e-200), f"{label}: audit {k}"
    for k in ("strain_energy", "plastic_dissipation", "hourglass_energy", "fracture_dissipation"):
        assert close(getattr(ag, k), getattr(ao, k), rel_e, floor=1e-200), f"{label}: audit {k}"
    # momenta are sums of terms of both signs: the tolerance is relative to sum |m v|
    m = o.readField(_abi.FIELD_MASS)
    for k, f in (("axial_momentum", _abi.FIELD_VZ), ("radial_momentum", _abi.FIELD_VR)):
        scale = float(np.sum(np.abs(m * o.readField(f))))
        assert abs(getattr(ag, k) - getattr(ao, k)) <= rel_n * max(scale, 1e-300), \
            f"{label}: audit {k}"
    for k in ("max_plastic_strain", "yielded_fraction", "max_damage", "damaged_fraction",
              "failed_fraction", "clamped_points", "most_damaged_element"):
        assert getattr(ag, k) == getattr(ao, k), f"{label}: audit {k}"


def pair(builder, **kw):
    g, mesh, info = builder(ExplicitSolver, **kw)
    o, _, _ = builder(OracleSolver, **kw)
    return g, o, mesh, info


def test_rod_10x60_full_run(gpu_lib):
    """The 10 x 60 axisymmetric Johnson-Cook rod on the Coulomb anvil, to 80 us."""
    g, o, mesh, info = pair(scenes.taylor_rod)
    ng = g.runUntil(80e-6)
    no = o.runUntil(80e-6)
    assert ng == no and ng > 1000
    assert_bitwise(g, o, "rod")
    assert_totals(g, o, "rod")
    mg, mo = g.measure(), o.measure()
    assert mg.length == mo.length and mg.mushroom_diameter == mo.mushroom_diameter


@pytest.mark.parametrize("integ", [Integration.REDUCED, Integration.FULL])
@pytest.mark.parametrize("friction", [0.0, 0.15, float("inf")])
def test_taylor_reference_rules_and_interfaces(gpu_lib, integ, friction):
    g, o, _, _ = pair(scenes.taylor_reference, nr=4, integration=integ, friction=friction)
    g.run(700)
    o.run(700)
    assert_bitwise(g, o, f"taylor {integ.name} mu={friction}")
    assert_totals(g, o, "taylor")


def test_two_blocks_contact_damage_floor(gpu_lib):
    g, o, _, _ = pair(scenes.two_blocks, speed=400.0)
    for chunk in (1, 99, 500):
        g.run(chunk)
        o.run(chunk)
        assert_bitwise(g, o, "two blocks")
    assert_totals(g, o, "two blocks")


def test_perforation_coarse_erosion_and_contact(gpu_lib):
    """The multi-body perforation at 1 mm cells: contact, friction, damage, erosion, gravity."""
    g, o, _, info = pair(scenes.perforation, cell=1.0e-3)
    for chunk in (200, 400):
        g.run(chunk)
        o.run(chunk)
        assert_bitwise(g, o, "perforation")
    assert_totals(g, o, "perforation")
    assert g.erodedElements() > 0
    assert info["contact"].pairCount() > 0


@pytest.mark.parametrize("slots", [0, 3])
def test_perforation_coarse_grid_layouts(gpu_lib, slots):
    """The contact grid's two layouts give the same bits. With 0 slots per cell every step
    files its buckets by the counting sort; with 3, a step whose busiest cell holds more than
    three segment ends falls back to it, so the run mixes both layouts."""
    g, o, _, info = pair(scenes.perforation, cell=1.0e-3)
    g.setGridSlots(slots)
    o.setGridSlots(slots)
    for chunk in (200, 400):
        g.run(chunk)
        o.run(chunk)
        assert_bitwise(g, o, f"perforation, {slots} grid slots")
    assert_totals(g, o, "perforation")
    assert info["contact"].pairCount() > 0


def test_grid_slots_are_validated(gpu_lib):
    g, _, _ = scenes.two_blocks(ExplicitSolver)
    for bad in (-1, 65):
        with pytest.raises(ValueError, match=r"\[0, 64\]"):
            g.setGridSlots(bad)
    g.setGridSlots(64)


def run_both(g, o, marks, label):
    """Steps both solvers to each mark in turn and compares them there, bit for bit."""
    done = 0
    for upto in marks:
        g.run(upto - done)
        o.run(upto - done)
        done = upto
        assert_bitwise(g, o, f"{label}, step {upto}")


def test_perforation_200k_through_impact(gpu_lib):
    """The 199,675-quad perforation exactly as benchmarked: the slug starts 0.5 mm from the
    blocks, so it strikes near step 73. By step 1000 the contact search and pair forces,
    the friction cone, the Johnson-Cook solves of the copper, damage onset, erosion and the
    free-surface rebuilds have all run; every field, set and counter is compared bit for bit
    at steps 100, 500 and 1000."""
    g, o, mesh, info = pair(scenes.perforation, gap=0.5e-3)
    o.setThreads(os.cpu_count() or 1)
    assert mesh.elementCount > 190_000
    run_both(g, o, (100, 500, 1000), "perforation 200k")
    assert_totals(g, o, "perforation 200k")
    assert g.erodedElements() > 0
    assert info["contact"].pairCount() > 0
    copper = ~info["slug"]
    assert np.count_nonzero(g.plasticStrain()[copper]) > 1000   # Johnson-Cook returns ran


def test_perforation_1M_through_impact(gpu_lib):
    """The same scene on the 1.0M-quad lattice (0.051 mm cells), slug 0.25 mm from the
    blocks (impact near step 82), in FP64: 300 steps, compared bit for bit at 150 and 300.
    The contact grid, bucket and hot-list capacities are at their largest here."""
    g, o, mesh, info = pair(scenes.perforation, cell=0.051e-3, gap=0.25e-3)
    o.setThreads(os.cpu_count() or 1)
    assert mesh.elementCount > 990_000
    run_both(g, o, (150, 300), "perforation 1M")
    assert_totals(g, o, "perforation 1M")
    assert info["contact"].pairCount() > 0


@pytest.mark.parametrize("factor", [4.0, 25.0])
def test_mass_scaled_rod_through_impact(gpu_lib, factor):
    """setMassScaling active (ExplicitSolver.java:601-619): every mass times the factor, the
    step at the target, and sqrt(massScale) in every later CFL step (:985-990), on a rod
    that strikes the anvil from the first step."""
    def build(cls):
        s, mesh, info = scenes.taylor_rod(cls, nr=4, nz=24)
        s.setMassScaling(s.timestep() * math.sqrt(factor))
        return s, mesh, info
    g, o, _, _ = pair(build)
    assert g.massScale() == o.massScale() and g.massScale() > 1.0
    run_both(g, o, (1, 300, 800), f"mass scaled x{factor}")
    assert_totals(g, o, "mass scaled")


def test_mass_scaled_stack_with_contact(gpu_lib):
    """MassScalingTest.contactStaysStable (MassScalingTest.java:108-127): two stacked steel
    blocks under gravity on the floor, penalty contact, the step scaled tenfold (the contact
    stiffness follows the scaled step)."""
    MM = 1.0e-3

    def build(cls):
        mesh = Outline.assemble(MM, Outline.rectangle(0.0, 0.0, 8.0 * MM, 4.0 * MM),
                                Outline.rectangle(0.0, 4.0 * MM, 8.0 * MM, 8.0 * MM))
        s = cls(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)
        s.setMassScaling(s.timestep() * 10.0)
        s.setContact(Contact(mesh))
        s.setGravity(0.0, -9.81)
        s.setRigidWall(RigidWall.atZ(0.0))
        return s, mesh, {}
    g, o, _, _ = pair(build)
    run_both(g, o, (10, 1000, 2000), "mass scaled stack")
    assert_totals(g, o, "mass scaled stack")


@pytest.mark.parametrize("integ", [Integration.REDUCED, Integration.FULL])
def test_small_strain_rod(gpu_lib, integ):
    """Kinematics.SMALL_STRAIN: no co-rotation, reference-geometry B matrix, fixed step
    (the kinematics.isFinite() == false branches of ExplicitSolver.java:1219-1504 and
    :985), on the Johnson-Cook rod striking the anvil."""
    def build(cls):
        mesh = QuadMesh.solidCylinder(3.8e-3, 25.0e-3, 4, 24)
        s = cls(mesh, scenes.rod_material(), Formulation.AXISYMMETRIC, integ,
                Kinematics.SMALL_STRAIN, 1.0, 0.6)
        s.setHourglassCoefficient(0.10)
        for n in QuadMesh.axisNodes(4, 24):
            s.fixRadial(n)
        s.setRigidWall(RigidWall.atZ(0.0, 0.09))
        s.setUniformVelocity(0.0, -150.0)
        return s, mesh, {}
    g, o, _, _ = pair(build)
    run_both(g, o, (300, 700), f"small strain {integ.name}")
    assert_totals(g, o, "small strain")
    assert np.count_nonzero(g.plasticStrain()) > 0


@pytest.mark.parametrize("kin", [Kinematics.FINITE_STRAIN, Kinematics.SMALL_STRAIN])
@pytest.mark.parametrize("integ", [Integration.REDUCED, Integration.FULL])
def test_plane_stress_plate(gpu_lib, kin, integ):
    """Formulation.PLANE_STRESS (ExplicitSolver.java:269-299: elastic only, the plane-stress
    lambda 2 lambda mu / (lambda + 2 mu)): a steel plate thrown at the floor under gravity."""
    MM = 1.0e-3

    def build(cls):
        mesh = Outline.rectangle(0.0, 0.0, 12.0 * MM, 6.0 * MM).mesh(0.5 * MM)
        s = cls(mesh, Material.STEEL_4340, Formulation.PLANE_STRESS, integ, kin, 2.0 * MM, 0.5)
        s.setHourglassCoefficient(0.05)
        s.setGravity(0.0, -9.81)
        s.setRigidWall(RigidWall.atZ(0.0, 0.3))
        vr = np.full(mesh.nodeCount, 5.0)
        s.setVelocities(vr, np.full(mesh.nodeCount, -40.0))
        return s, mesh, {}
    g, o, _, _ = pair(build)
    run_both(g, o, (200, 600), f"plane stress {kin.name} {integ.name}")
    assert_totals(g, o, "plane stress")


def test_pressurised_tube(gpu_lib):
    g, o, _, _ = pair(scenes.tube)
    g.run(600)
    o.run(600)
    assert_bitwise(g, o, "tube")
    assert_totals(g, o, "tube")


def test_run_until_matches_step_loop(gpu_lib):
    a, mesh, _ = scenes.taylor_rod(ExplicitSolver, nr=4, nz=24)
    b, _, _ = scenes.taylor_rod(ExplicitSolver, nr=4, nz=24)
    n = a.runUntil(10e-6)
    b.run(n)
    assert_bitwise(a, b, "run_until")


def test_run_until_keeps_the_last_steps_totals(gpu_lib):
    """runUntil replays predicated steps in chunks of sixteen. The steps past the bound do
    nothing, and the totals still describe the last step taken: contact pairs, penetration
    and wall counts equal the oracle's after the same run."""
    g, o, _, _ = pair(scenes.two_blocks, speed=400.0)
    t_end = 2.0e-6                     # 21 steps: pairs and wall contacts are both active
    n = g.runUntil(t_end)
    assert n % 16 != 0, "the bound should fall inside a chunk of sixteen"
    assert o.runUntil(t_end) == n
    assert g._contactInfo().pair_count > 0 and g._wallInfo().contact_count > 0
    assert_bitwise(g, o, "run_until")
    assert_totals(g, o, "run_until")


def test_repeat_runs_are_identical(gpu_lib):
    """ThreadingTest's property on the device: the answer does not depend on the schedule."""
    a, _, _ = scenes.perforation(ExplicitSolver, cell=1.0e-3)
    b, _, _ = scenes.perforation(ExplicitSolver, cell=1.0e-3)
    a.run(300)
    for _ in range(3):
        b.run(100)
    assert_bitwise(a, b, "repeat")


def _random_points(rng, n):
    sig = rng.normal(0.0, 3e8, (n, 4))
    back = rng.normal(0.0, 5e7, (n, 4))
    back[:, :3] -= back[:, :3].mean(axis=1, keepdims=True)
    eps = np.abs(rng.normal(0.0, 0.2, n))
    work = np.abs(rng.normal(0.0, 2e8, n))
    strain = rng.normal(0.0, 2e-3, (n, 4))
    return sig.reshape(-1), back.reshape(-1), eps, work, strain.reshape(-1)


@pytest.mark.parametrize("kind", ["linear", "jc", "jc-damage", "elastic"])
def test_material_points_random(gpu_lib, kind):
    """J2.update over random states and increments, device against oracle, bit for bit,
    including the Johnson-Cook solve, damage onset and softening."""
    rng = np.random.default_rng(42)
    n = 4096
    if kind == "linear":
        m = Material.STEEL_4340.yielding(800e6, 1e9, 2e9)
    elif kind == "elastic":
        m = Material.STEEL_4340
    else:
        m = Material.COPPER_OFHC.withKinematicHardening(1e8).withJohnsonCook(JohnsonCook.COPPER_OFHC)
    state_g = _random_points(rng, n)
    state_o = tuple(x.copy() for x in state_g)
    dmg_g = dmg_o = None
    if kind == "jc-damage":
        dmg_g = {"failure_strain": np.abs(rng.normal(0.3, 0.1, n)) + 0.01,
                 "fracture_energy": np.full(n, 2e4), "youngs_modulus": np.full(n, m.youngsModulus),
                 "geometry": np.tile([1e-6, 1e-3, 1e-4, -2e-4, 1e-3], n).astype(np.float64),
                 "strength": np.zeros(n), "softening": np.zeros(n), "width": np.zeros(n)}
        dmg_o = {k: v.copy() for k, v in dmg_g.items()}
    for step in range(30):
        inc = rng.normal(0.0, 2e-3, 4 * n)
        dg_g = material_point_update(m, *state_g[:4], inc, 1e-8, damage=dmg_g)
        dg_o = material_point_update(m, *state_o[:4], inc, 1e-8, damage=dmg_o,
                                     binding=oracle_api())
        assert np.array_equal(dg_g.view(np.uint64), dg_o.view(np.uint64)), f"dgamma step {step}"
        for a, b in zip(state_g[:4], state_o[:4]):
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), f"state step {step}"
        if dmg_g is not None:
            for k in ("strength", "softening", "width"):
                assert np.array_equal(dmg_g[k].view(np.uint64), dmg_o[k].view(np.uint64)), k
    if kind == "jc-damage":
        assert np.count_nonzero(dmg_g["strength"]) > 100


def test_validation_messages_match(gpu_lib):
    """The device library raises the reference's exceptions and messages."""
    g, mesh, _ = scenes.taylor_rod(ExplicitSolver, nr=2, nz=6)
    with pytest.raises(RuntimeError, match="setDamage"):
        g.setErosion(1.0)
    with pytest.raises(ValueError, match="cannot shorten"):
        g.setMassScaling(0.5 * g.timestep())
    with pytest.raises(ValueError, match="angular frequency"):
        g.setRelaxationDamping(0.1, 0.0)
    with pytest.raises(ValueError, match="hourglass"):
        g.setHourglassCoefficient(-1.0)
    with pytest.raises(ValueError, match="failure strain"):
        g.setDamage(1e3, np.zeros(mesh.elementCount))
