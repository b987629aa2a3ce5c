"""The oracle pinned against the reference's own known answers (CPU only).

The reference ships no stored vectors and cannot run here (no JDK), so the CPU restatement in
oracle/refcpu.c is checked against what the reference's tests and README assert:
closed forms (GravityTest, J2Test, FiniteStrainTest, HourglassTest), conservation and
bookkeeping identities (ContactTest, ErosionTest, MassScalingTest, TaylorImpactTest), thread
determinism (ThreadingTest) and the published Taylor-impact table (README.md:306-312).
Citations are to src/test/java/org/neofiz/ in the reference.
"""
import math
import os

import numpy as np
import pytest

from neofiz_gb300 import (Contact, Formulation, Integration, JohnsonCook, Kinematics, Material,
                          Outline, QuadMesh, RigidWall, scenes)
from neofiz_gb300.solver import material_point_update
from oracle.oracle import OracleSolver, api as oracle_api

MM = 1.0e-3


# ----------------------------------------------------------------------------- GravityTest

def test_free_fall_is_exact():
    """GravityTest.freeFallIsExact (:36-59): u = -g t (t + dt) / 2 to 1e-12."""
    mesh = Outline.rectangle(0.0, 0.0, 6.0 * MM, 4.0 * MM).mesh(MM)
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.SMALL_STRAIN, 10.0 * MM, 0.5)
    s.setGravity(0.0, -9.81)
    s.run(2000)
    t = s.time()
    expected = -0.5 * 9.81 * t * (t + s.timestep())
    uz = s.axialDisplacement()
    assert np.all(np.abs(uz - expected) <= 1e-12 * abs(expected))
    total = float(s.readField(6).sum())
    assert abs(s.axialMomentum() / total - (-9.81 * t)) <= 1e-9 * 9.81 * t


def test_gravity_is_off_by_default():
    """GravityTest.defaultIsNone (:81-92): an unforced body keeps exactly zero momentum."""
    mesh = Outline.rectangle(0.0, 0.0, 6.0 * MM, 4.0 * MM).mesh(MM)
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.SMALL_STRAIN, 10.0 * MM, 0.5)
    s.run(500)
    assert s.axialMomentum() == 0.0


def test_resting_body_does_not_sink():
    """GravityTest.restingBodyDoesNotSink (:61-80)."""
    mesh = Outline.rectangle(0.0, 0.0, 20.0 * MM, 5.0 * MM).mesh(MM)
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.SMALL_STRAIN, 10.0 * MM, 0.5)
    s.setGravity(0.0, -9.81)
    s.setRigidWall(RigidWall.atZ(0.0))
    s.run(4000)
    lowest = np.min(mesh.z + s.axialDisplacement())
    assert lowest >= -1e-15
    assert abs(s.kineticEnergy()) < 1e-6


# ----------------------------------------------------------------------------- Taylor impact

# README.md:306-312 (4340, 181 m/s, frictionless) and :344-352 (friction sweep, n = 8).
PUBLISHED = [
    # the reference's Taylor-impact table (README.md:306-314) and its Coulomb friction sweep
    # (README.md:344-352): nr, integration, jc, friction, mushroom mm, L/L0, max eps_p, T max,
    # friction dissipation as a percentage of the impact energy
    (4, Integration.REDUCED, True, 0.0, 9.472, 0.9079, 0.50, 443, None),
    (4, Integration.REDUCED, False, 0.0, 9.590, 0.8827, 0.54, None, None),
    (8, Integration.REDUCED, True, 0.0, 9.776, 0.9081, 0.67, 495, None),
    (8, Integration.REDUCED, False, 0.0, 9.855, 0.8843, 0.72, None, None),
    (16, Integration.REDUCED, True, 0.0, 9.965, 0.9080, 0.75, 517, None),
    (16, Integration.REDUCED, False, 0.0, 10.005, 0.8845, 0.83, None, None),
    (8, Integration.FULL, True, 0.0, 9.448, 0.9076, 0.56, 459, None),
    (8, Integration.REDUCED, True, 0.02, 9.651, 0.9082, None, None, 0.46),
    (8, Integration.REDUCED, True, 0.05, 9.476, 0.9085, None, None, 1.02),
    (8, Integration.REDUCED, True, 0.10, 9.259, 0.9088, None, None, 1.67),
    (8, Integration.REDUCED, True, 0.20, 8.987, 0.9093, None, None, 2.21),
    (8, Integration.REDUCED, True, 0.50, 8.921, 0.9102, None, None, 1.48),
    (8, Integration.REDUCED, True, math.inf, 8.928, 0.9106, None, None, 0.0),
]


@pytest.mark.parametrize("nr,integ,jc,mu,mush,ratio,eps,temp,fric", PUBLISHED)
def test_taylor_published_table(nr, integ, jc, mu, mush, ratio, eps, temp, fric):
    s, mesh, info = scenes.taylor_reference(OracleSolver, nr, integration=integ, friction=mu,
                                            jc=jc)
    wall = info["wall"]
    p0, k0 = s.axialMomentum(), s.kineticEnergy()
    s.runUntil(80e-6)
    m = s.measure()
    assert round(m.mushroom_diameter * 1e3, 3) == pytest.approx(mush, abs=1e-9)
    assert round(m.length / info["length"], 4) == pytest.approx(ratio, abs=1e-9)
    if eps is not None:
        assert round(s.maxPlasticStrain(), 2) == pytest.approx(eps, abs=1e-9)
    if temp is not None:
        assert round(s.maxTemperature()) == temp
    if fric is not None:
        assert round(100.0 * wall.frictionDissipation() / k0, 2) == pytest.approx(fric, abs=1e-9)
    # TaylorImpactTest.momentumBalance (:115-122): change in momentum = anvil impulse
    err = abs((s.axialMomentum() - p0) - wall.impulse()) / abs(p0)
    assert err < 1e-11
    # TaylorImpactTest.energyBalance (:124-142): closes to 1 %
    acc = (s.plasticDissipation() + s.kineticEnergy() + s.strainEnergy() + wall.energyLoss()
           + s.hourglassEnergy() + wall.frictionDissipation())
    assert abs(acc / k0 - 1.0) < 0.01
    # TaylorImpactTest.hourglassIsNegligible (:144-163)
    assert s.hourglassEnergy() / k0 < 0.01


def test_the_axis_holds():
    """TaylorImpactTest.theAxisHolds (:75-97): axis nodes stay on the centreline exactly."""
    nr, nz = 3, 8
    mesh = QuadMesh.solidCylinder(0.5 * 7.595e-3, 8.0e-3, nr, nz)
    s = OracleSolver(mesh, Material.STEEL_4340.withJohnsonCook(JohnsonCook.STEEL_4340),
                     Formulation.AXISYMMETRIC, Integration.REDUCED, Kinematics.FINITE_STRAIN,
                     1.0, 0.5)
    for n in QuadMesh.axisNodes(nr, nz):
        s.fixRadial(n)
    s.setRigidWall(RigidWall.atZ(0.0))
    s.setUniformVelocity(0.0, -181.0)
    while s.time() < 20e-6:
        s.step()
    ur = s.radialDisplacement()
    for n in QuadMesh.axisNodes(nr, nz):
        assert ur[n] == 0.0, n
    assert s.maxPlasticStrain() > 0.05


def test_temperature_rise_and_johnson_cook_stiffening():
    """TaylorImpactTest.temperatureRiseIsPhysical and johnsonCookStiffensTheResponse
    (:164-197), on the n = 4 reference run: a rise of 100-400 K, the thermal term below 0.92,
    and the Johnson-Cook rod shortening less and reaching less plastic strain than the
    rate-independent surrogate."""
    jc, _, info = scenes.taylor_reference(OracleSolver, 4)
    surrogate, _, _ = scenes.taylor_reference(OracleSolver, 4, jc=False)
    jc.runUntil(80e-6)
    surrogate.runUntil(80e-6)
    law = JohnsonCook.STEEL_4340
    rise = jc.maxTemperature() - law.roomTemperature
    assert 100.0 < rise < 400.0
    homologous = rise / (law.meltTemperature - law.roomTemperature)
    assert 1.0 - homologous ** law.m < 0.92
    assert jc.measure().length / info["length"] > surrogate.measure().length / info["length"] + 0.015
    assert jc.maxPlasticStrain() < surrogate.maxPlasticStrain()


# ----------------------------------------------------------------------------- J2Test

E, NU, SY = 205.0e9, 0.29, 800.0e6
MU = E / (2.0 * (1.0 + NU))
LAMBDA = E * NU / ((1.0 + NU) * (1.0 - 2.0 * NU))


class Point:
    """J2Test.Point (:29-63): one material point driven through J2.update."""

    def __init__(self, sy, hIso, hKin):
        self.m = Material("pt", E, NU, 7850.0, sy, hIso, hKin)
        self.sig = np.zeros(4)
        self.back = np.zeros(4)
        self.eps = np.zeros(1)
        self.work = np.zeros(1)
        self.sy, self.hIso = sy, hIso

    def strain(self, dRR, dZZ, dTT, dGam):
        return float(material_point_update(self.m, self.sig, self.back, self.eps, self.work,
                                           np.array([dRR, dZZ, dTT, dGam]), 1.0e-8,
                                           binding=oracle_api())[0])

    def shear(self, dGam):
        return self.strain(0.0, 0.0, 0.0, dGam)

    def mises(self):
        s = self.sig
        p = (s[0] + s[1] + s[2]) / 3.0
        a, b, c, d = s[0] - p, s[1] - p, s[2] - p, s[3]
        return math.sqrt(1.5 * (a * a + b * b + c * c + 2.0 * d * d))

    def f(self):
        s, k = self.sig, self.back
        p = (s[0] + s[1] + s[2]) / 3.0
        x = [s[0] - p - k[0], s[1] - p - k[1], s[2] - p - k[2], s[3] - k[3]]
        n = math.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2 + 2.0 * x[3] ** 2)
        return n - math.sqrt(2.0 / 3.0) * (self.sy + self.hIso * self.eps[0])


def exact_shear_plastic_strain(gamma, h):
    root3mu = math.sqrt(3.0) * MU
    return (gamma - SY / root3mu) / (h / root3mu + math.sqrt(3.0))


def test_shear_yields_at_mises_limit():
    """J2Test.shearYieldsAtTheMisesLimit (:64-83)."""
    p = Point(SY, 0.0, 0.0)
    step = 1.0e-6
    last = 0.0
    for _ in range(20000):
        if p.shear(step) > 0.0:
            break
        last = p.sig[3]
    assert last > 0.0
    assert abs(p.sig[3] - SY / math.sqrt(3.0)) <= MU * step * 1.01


def test_flow_stress_follows_hardening_law():
    """J2Test.flowStressFollowsTheHardeningLaw (:100-128): 1e-14 on the hardening law."""
    hIso = 2.0e9
    p = Point(SY, hIso, 0.0)
    plastic = 0
    for _ in range(6000):
        if p.shear(2.0e-6) > 0.0:
            plastic += 1
            assert abs(SY + hIso * p.eps[0] - p.mises()) <= (SY + hIso) * 1e-14
            assert abs(p.f()) <= SY * 1e-14
    assert plastic > 1000
    expected = exact_shear_plastic_strain(6000 * 2.0e-6, hIso)
    assert abs(p.eps[0] - expected) <= expected * 1e-10


def test_plastic_flow_is_incompressible():
    """J2Test.plasticFlowIsExactlyIncompressible (:130-157)."""
    p = Point(SY, 1.0e9, 1.0e9)
    last = 0.0
    for _ in range(4000):
        t = p.sig.copy()
        lt = LAMBDA * -3.0e-6
        expected = -((t[0] + lt + 2 * MU * -1.0e-6) + (t[1] + lt + 2 * MU * -1.0e-6)
                     + (t[2] + lt + 2 * MU * -1.0e-6)) / 3.0
        p.strain(-1.0e-6, -1.0e-6, -1.0e-6, 4.0e-6)
        actual = -(p.sig[0] + p.sig[1] + p.sig[2]) / 3.0
        assert abs(actual - expected) <= max(1.0, abs(expected)) * 1e-13
        last = actual
    assert abs(last) > 1.0e8 and p.eps[0] > 0.0


def test_perfect_plasticity_caps():
    """J2Test.perfectPlasticityCaps (:159-174)."""
    p = Point(SY, 0.0, 0.0)
    for _ in range(20000):
        p.shear(2.0e-6)
    assert abs(p.mises() - SY) <= SY * 1e-12
    expected = exact_shear_plastic_strain(20000 * 2.0e-6, 0.0)
    assert abs(p.eps[0] - expected) <= expected * 1e-10


def test_unloading_is_elastic():
    """J2Test.unloadingIsElastic (:176-196)."""
    p = Point(SY, 2.0e9, 0.0)
    for _ in range(4000):
        p.shear(2.0e-6)
    tau, eps = p.sig[3], p.eps[0]
    assert p.shear(-2.0e-6) == 0.0
    assert abs(p.sig[3] - (tau + MU * -2.0e-6)) <= abs(tau) * 1e-14
    assert p.eps[0] == eps


def test_bauschinger_separates_hardening_kinds():
    """J2Test.bauschingerSeparatesTheTwoHardeningKinds (:198-233)."""
    h = 4.0e9
    kin, iso = Point(SY, 0.0, h), Point(SY, h, 0.0)
    for _ in range(6000):
        kin.shear(2.0e-6)
        iso.shear(2.0e-6)
    assert abs(iso.mises() - kin.mises()) <= SY * 1e-10
    forward = kin.sig[3]

    def reverse_yield(p):
        for _ in range(40000):
            before = p.sig[3]
            if p.shear(-2.0e-6) > 0.0:
                return before
        raise AssertionError("never reached reverse yield")
    rk, ri = reverse_yield(kin), reverse_yield(iso)
    span = forward - rk
    assert abs(span - 2.0 * SY / math.sqrt(3.0)) <= span * 1e-3
    assert ri < rk


def test_infinite_yield_is_linear_elasticity():
    """J2Test.elasticMaterialTakesTheSamePath (:242-256)."""
    p = Point(math.inf, 0.0, 0.0)
    dRR, dZZ, dTT, dG = 3.0e-4, -1.0e-4, 2.0e-4, 5.0e-4
    p.strain(dRR, dZZ, dTT, dG)
    lt = LAMBDA * (dRR + dZZ + dTT)
    assert p.sig[0] == pytest.approx(lt + 2 * MU * dRR, abs=1e-6)
    assert p.sig[3] == pytest.approx(MU * dG, abs=1e-6)
    assert p.eps[0] == 0.0


def test_stress_never_escapes_the_surface():
    """J2Test.stressNeverEscapesTheSurface (:258-273), with a numpy generator."""
    p = Point(SY, 1.0e9, 1.0e9)
    rng = np.random.default_rng(20260918)
    for _ in range(5000):
        g = rng.standard_normal(4) * 1e-3
        p.strain(*g)
        assert p.f() <= SY * 1e-12
        assert math.isfinite(p.mises())
    assert p.eps[0] > 0.1


def test_rate_dependent_solve_degenerates_to_closed_form():
    """RateDependentReturnMapTest.degeneratesToTheClosedForm (:70-96): with B = C = beta = 0
    the Johnson-Cook solve matches the linear return to 1e-12."""
    jc = JohnsonCook(SY, 0.0, 0.5, 0.0, 1.0, 1.0, 293.0, 1793.0, 477.0, 0.0)
    a = Point(SY, 0.0, 0.0)
    b = Point(SY, 0.0, 0.0)
    b.m = Material("jc", E, NU, 7850.0).withJohnsonCook(jc)
    for _ in range(3000):
        a.shear(2.0e-6)
        b.shear(2.0e-6)
    assert abs(a.sig[3] - b.sig[3]) <= abs(a.sig[3]) * 1e-12
    assert abs(a.eps[0] - b.eps[0]) <= a.eps[0] * 1e-10


# ----------------------------------------------------------------------------- Hourglass / finite strain

def _impose(s, uR, uZ):
    dt = s.timestep()
    for i in range(4):
        s.setVelocity(i, uR[i] / dt, uZ[i] / dt)
    s.advance()
    f = np.empty(8)
    f[0::2], f[1::2] = s.forceR(), s.forceZ()
    return f


@pytest.mark.parametrize("form", [Formulation.AXISYMMETRIC, Formulation.PLANE_STRAIN])
def test_hourglass_invisible_to_linear_fields(form):
    """HourglassTest.linearFieldsProduceNoHourglassForce (:87-120)."""
    mesh = QuadMesh([1.00, 2.10, 1.90, 0.85], [0.00, 0.15, 1.20, 0.95], [0, 1, 2, 3])
    uR = 1.0e-3 + 2.0e-3 * mesh.r - 0.7e-3 * mesh.z
    uZ = -0.4e-3 + 1.1e-3 * mesh.r + 1.5e-3 * mesh.z

    def make(q):
        s = OracleSolver(mesh, Material.STEEL_4340, form, Integration.REDUCED, 1.0, 0.5)
        s.setHourglassCoefficient(q)
        return s
    without = _impose(make(0.0), uR, uZ)
    on = make(0.05)
    with_ = _impose(on, uR, uZ)
    scale = np.linalg.norm(without)
    assert scale > 0.0
    assert np.all(np.abs(without - with_) <= scale * 1e-12)
    assert abs(on.hourglassEnergy()) <= on.strainEnergy() * 1e-12


_UNIT = ([1.0, 2.0, 2.0, 1.0], [0.0, 0.0, 1.0, 1.0], [0, 1, 2, 3])


def _hg_solver(mesh, q, integration=Integration.REDUCED):
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, integration, 1.0, 0.5)
    s.setHourglassCoefficient(q)
    return s


def _hourglass(e):
    return np.array([e, -e, e, -e])


def test_the_hourglass_mode_is_free_without_control():
    """HourglassTest.theModeIsFreeWithoutControl (:121-148)."""
    mesh = QuadMesh(*_UNIT)
    e = 1.0e-4
    cheap = _impose(_hg_solver(mesh, 0.0), _hourglass(e), np.zeros(4))
    expensive = _impose(_hg_solver(mesh, 0.0, Integration.FULL), _hourglass(e), np.zeros(4))
    scale = np.linalg.norm(_impose(_hg_solver(mesh, 0.0), e * np.asarray(mesh.r), np.zeros(4)))
    assert np.linalg.norm(cheap) < scale * 1e-12
    assert np.linalg.norm(expensive) > scale * 0.1


def test_hourglass_control_opposes_the_mode():
    """HourglassTest.controlOpposesTheMode (:150-179): antiparallel force, linear in the
    amplitude, energy quadratic."""
    mesh = QuadMesh(*_UNIT)
    e = 1.0e-4
    s = _hg_solver(mesh, 0.05)
    f = _impose(s, _hourglass(e), np.zeros(4))
    energy = s.hourglassEnergy()
    assert sum((1.0 if i % 2 == 0 else -1.0) * f[2 * i] for i in range(4)) < 0.0
    assert energy > 0.0
    twice = _hg_solver(mesh, 0.05)
    f2 = _impose(twice, _hourglass(2.0 * e), np.zeros(4))
    assert abs(np.linalg.norm(f2) / np.linalg.norm(f) - 2.0) <= 1e-9
    assert abs(twice.hourglassEnergy() / energy - 4.0) <= 1e-9


def test_hourglass_coefficient_scales_the_stiffness():
    """HourglassTest.coefficientScalesStiffness (:180-204), on the distorted quad."""
    mesh = QuadMesh([1.00, 2.10, 1.90, 0.85], [0.00, 0.15, 1.20, 0.95], [0, 1, 2, 3])
    e = 1.0e-4
    previous = None
    for q in (0.02, 0.04, 0.08):
        delta = (_impose(_hg_solver(mesh, q), _hourglass(e), np.zeros(4))
                 - _impose(_hg_solver(mesh, 0.0), _hourglass(e), np.zeros(4)))
        if previous is not None:
            assert abs(np.linalg.norm(delta) / np.linalg.norm(previous) - 2.0) <= 1e-9
        previous = delta


def test_rigid_rotation_is_objective():
    """FiniteStrainTest.rigidRotationIsExactlyObjective (:59-110)."""
    mesh = QuadMesh([0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 1.0], [0, 1, 2, 3])
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.FINITE_STRAIN, 1.0, 0.5)

    def move_to(tr, tz):
        dt = s.timestep()
        ur, uz = s.radialDisplacement(), s.axialDisplacement()
        for i in range(4):
            s.setVelocity(i, (tr[i] - (mesh.r[i] + ur[i])) / dt, (tz[i] - (mesh.z[i] + uz[i])) / dt)
        s.advance()

    r = [0.0, 1.0, 1.0, 0.0]
    z = [0.0, 0.0, 1.002, 1.002]
    move_to(r, z)

    def mises(v):
        p = (v[0] + v[1] + v[2]) / 3.0
        return math.sqrt(1.5 * ((v[0] - p) ** 2 + (v[1] - p) ** 2 + (v[2] - p) ** 2 + 2 * v[3] ** 2))
    before = s.centroidStress(0)
    mb = mises(before)
    assert mb > 1.0e6
    for k in range(1, 361):
        a = (math.pi / 2.0) * k / 360
        c, sn = math.cos(a), math.sin(a)
        move_to([c * r[i] - sn * z[i] for i in range(4)], [sn * r[i] + c * z[i] for i in range(4)])
    after = s.centroidStress(0)
    assert abs(mises(after) - mb) <= mb * 1e-9
    assert abs(before[1] - after[0]) <= mb * 1e-9
    assert abs(before[0] - after[1]) <= mb * 1e-9
    assert abs(before[2] - after[2]) <= mb * 1e-9
    assert s.plasticStrain()[0] == 0.0


# ----------------------------------------------------------------------------- contact / erosion

def _two_blocks():
    return Outline.meshOf(MM, Outline.rectangle(0.0, 0.0, 8.0 * MM, 12.0 * MM),
                          Outline.rectangle(13.0 * MM, 2.0 * MM, 21.0 * MM, 8.0 * MM))


def _contact_solver(mesh):
    return OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                        Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)


def _approach(s, mesh, v):
    s.setVelocities(np.where(mesh.r < 10.0 * MM, v, -v), np.zeros(mesh.nodeCount))


def _square_solver(material, kinematics, integration=Integration.REDUCED):
    mesh = QuadMesh([0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 1.0], [0, 1, 2, 3])
    return mesh, OracleSolver(mesh, material, Formulation.PLANE_STRAIN, integration, kinematics,
                              1.0, 0.5)


def _move_to(s, mesh, tr, tz):
    """FiniteStrainTest.moveTo (:48-56)."""
    dt = s.timestep()
    ur, uz = s.radialDisplacement(), s.axialDisplacement()
    for i in range(4):
        s.setVelocity(i, (tr[i] - (mesh.r[i] + ur[i])) / dt, (tz[i] - (mesh.z[i] + uz[i])) / dt)
    s.advance()


def _mises(v):
    p = (v[0] + v[1] + v[2]) / 3.0
    return math.sqrt(1.5 * ((v[0] - p) ** 2 + (v[1] - p) ** 2 + (v[2] - p) ** 2 + 2 * v[3] ** 2))


def test_isochoric_compression_hits_the_exact_yield_state():
    """FiniteStrainTest.largeIsochoricDeformationHitsTheExactYieldState (:193-233)."""
    sy = 800.0e6
    mesh, s = _square_solver(Material.STEEL_4340.yielding(sy, 0.0), Kinematics.FINITE_STRAIN)
    n = 4000
    for i in range(1, n + 1):
        c = 1.0 + (0.5 - 1.0) * i / n
        _move_to(s, mesh, [0.0, 1.0 / c, 1.0 / c, 0.0], [0.0, 0.0, c, c])
    sig = s.centroidStress(0)
    assert s.plasticStrain()[0] > 0.3
    assert abs(-(sig[0] + sig[1] + sig[2]) / 3.0) <= sy * 1e-3
    assert abs(sig[1] + sy / math.sqrt(3.0)) <= sy * 5e-3
    assert abs(_mises(sig) - sy) <= sy * 5e-3


def _stress_after_stretch(kinematics, integration, stretch):
    mesh, s = _square_solver(Material.STEEL_4340, kinematics, integration)
    n = 500
    for i in range(1, n + 1):
        h = 1.0 + (stretch - 1.0) * i / n
        _move_to(s, mesh, [0.0, 1.0, 1.0, 0.0], [0.0, 0.0, h, h])
    return s.centroidStress(0)


@pytest.mark.parametrize("integration", [Integration.REDUCED, Integration.FULL])
def test_formulations_agree_at_small_strain(integration):
    """FiniteStrainTest.formulationsAgreeAtSmallStrain (:235-253)."""
    small = _stress_after_stretch(Kinematics.SMALL_STRAIN, integration, 1.0 + 2.0e-4)
    finite = _stress_after_stretch(Kinematics.FINITE_STRAIN, integration, 1.0 + 2.0e-4)
    scale = _mises(small)
    assert scale > 0.0
    assert np.all(np.abs(np.asarray(small) - np.asarray(finite)) <= scale * 1e-3)


def test_formulations_diverge_at_large_strain():
    """FiniteStrainTest.formulationsDivergeAtLargeStrain (:255-271)."""
    small = _stress_after_stretch(Kinematics.SMALL_STRAIN, Integration.REDUCED, 1.20)
    finite = _stress_after_stretch(Kinematics.FINITE_STRAIN, Integration.REDUCED, 1.20)
    assert _mises(finite) < _mises(small)
    assert abs(_mises(finite) - _mises(small)) > 0.05 * _mises(small)


def test_collision_conserves_momentum():
    """ContactTest.momentumIsConserved (:85-103)."""
    mesh = _two_blocks()
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    _approach(s, mesh, 60.0)
    before = s.radialMomentum()
    s.run(4000)
    assert abs(s.radialMomentum() - before) <= 1e-9 * abs(before)
    assert abs(s.axialMomentum()) <= 1e-12
    assert s.contact().escapedNodes() == 0


def test_without_contact_blocks_interpenetrate():
    """ContactTest.withoutContactTheyInterpenetrate (:64-83)."""
    mesh = _two_blocks()
    s = _contact_solver(mesh)
    _approach(s, mesh, 60.0)
    s.run(3000)
    ur = s.radialDisplacement()
    front = np.max((mesh.r + ur)[mesh.r == 8.0 * MM])
    back = np.min((mesh.r + ur)[mesh.r == 13.0 * MM])
    assert front > back


def _contact_total(s):
    return (s.centredKineticEnergy() + s.strainEnergy() + s.hourglassEnergy()
            + s.contact().energy() + s.contact().dissipation())


def test_elastic_collision_closes_the_energy_budget():
    """ContactTest.elasticCollisionClosesTheEnergyBudget (:104-137): contact happens, nothing
    tunnels, the budget closes within 4 %, and the left block turns around."""
    mesh = _two_blocks()
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    _approach(s, mesh, 60.0)
    initial = _contact_total(s)
    touched = False
    for _ in range(400):
        s.run(20)
        touched = touched or s.contact().pairCount() > 0
    assert touched
    assert s.contact().escapedNodes() == 0
    assert abs(_contact_total(s) / initial - 1.0) < 0.04
    left = np.asarray(mesh.r) < 10.0 * MM
    assert np.mean(np.asarray(s.velocityR())[left]) < 0.0


def test_penetration_stays_a_small_fraction_of_a_cell():
    """ContactTest.penetrationIsBounded (:139-157)."""
    mesh = _two_blocks()
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    _approach(s, mesh, 60.0)
    worst = 0.0
    for _ in range(400):
        s.run(20)
        worst = max(worst, s.contact().maxPenetration())
    assert 0.0 < worst < 0.10 * MM


def test_a_surface_at_rest_does_not_contact_itself():
    """ContactTest.noSelfContactAtRest (:159-177): an L-shaped body (a re-entrant corner)."""
    mesh = Outline.of(0.0, 0.0, 20.0 * MM, 0.0, 20.0 * MM, 6.0 * MM, 6.0 * MM, 6.0 * MM,
                      6.0 * MM, 20.0 * MM, 0.0, 20.0 * MM).mesh(MM)
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    s.run(200)
    assert s.contact().pairCount() == 0
    assert s.contact().escapedNodes() == 0
    assert abs(s.kineticEnergy()) <= 1e-18


def test_a_node_is_not_caught_by_a_surface_it_is_not_facing():
    """ContactTest.facingIsRequired (:179-199): a block crushed against itself."""
    mesh = Outline.rectangle(0.0, 0.0, 3.0 * MM, 3.0 * MM).mesh(MM)
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    for i in range(mesh.nodeCount):
        if mesh.r[i] == 0.0:
            s.setVelocity(i, 120.0, 0.0)
        if mesh.r[i] == 3.0 * MM:
            s.setVelocity(i, -120.0, 0.0)
    s.run(1500)
    assert s.contact().pairCount() == 0


def _slide_speed(mesh, mu):
    s = _contact_solver(mesh)
    c = Contact(mesh).withFriction(mu)
    s.setContact(c)
    for i in range(mesh.nodeCount):
        if mesh.z[i] > 5.5 * MM:
            s.setVelocity(i, 30.0, -40.0)
        if mesh.z[i] == 0.0:
            s.fixAxial(i)
    initial = _contact_total(s)
    for _ in range(30):
        s.run(200)
    assert s.contact().dissipation() >= 0.0
    assert abs(_contact_total(s) / initial - 1.0) < 0.10
    upper = np.asarray(mesh.z) > 5.5 * MM
    return float(np.mean(np.asarray(s.velocityR())[upper]))


def test_friction_opposes_sliding():
    """ContactTest.frictionOpposesSliding (:201-244)."""
    mesh = Outline.meshOf(MM, Outline.rectangle(0.0, 0.0, 20.0 * MM, 5.0 * MM),
                          Outline.rectangle(5.0 * MM, 6.0 * MM, 13.0 * MM, 11.0 * MM))
    free, rough = _slide_speed(mesh, 0.0), _slide_speed(mesh, 0.4)
    assert rough < free
    assert rough > 0.0


def test_surface_covers_every_free_edge():
    """ContactTest.surfaceCoversEveryFreeEdge (:261-268): two 8x12 and 8x6 blocks have a
    perimeter of 40 + 28 cells."""
    mesh = _two_blocks()
    s = _contact_solver(mesh)
    s.setContact(Contact(mesh))
    s.run(1)
    assert s.contact().segmentCount() == 2 * (8 + 12) + 2 * (8 + 6)
    edges, owner, nodes = mesh.surface()
    assert np.array_equal(s.readField(22), edges)
    assert np.array_equal(s.readField(23), nodes)


def test_contact_stiffness_and_erosion_validation():
    """ContactTest.refusesUnstableStiffness (:246-259), ErosionTest.refusesWithoutDamage
    (:159-171), MassScalingTest.willNotRemoveMass (:92-103)."""
    mesh = _two_blocks()
    with pytest.raises(ValueError):
        Contact(mesh).withStiffnessScale(2.0)
    s = _contact_solver(mesh)
    with pytest.raises(RuntimeError, match="setDamage"):
        s.setErosion(1.0)
    with pytest.raises(ValueError, match="cannot shorten"):
        s.setMassScaling(0.5 * s.timestep())


def _stretching(cls, mesh, failure_strain):
    """ErosionTest.stretching (:31-43): a copper bar pulled apart at 80 m/s per end."""
    copper = Material.COPPER_OFHC.withJohnsonCook(JohnsonCook.COPPER_OFHC)
    s = cls(mesh, copper, Formulation.PLANE_STRAIN, Integration.REDUCED,
            Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)
    s.setDamage(np.full(mesh.elementCount, 6.0e3), np.full(mesh.elementCount, failure_strain))
    s.setVelocities(np.where(mesh.r < 10.0 * MM, -80.0, 80.0), np.zeros(mesh.nodeCount))
    return s


def _bar():
    return Outline.rectangle(0.0, 0.0, 20.0 * MM, 4.0 * MM).mesh(MM)


def test_erosion_off_by_default():
    """ErosionTest.offByDefault (:56-71)."""
    s = _stretching(OracleSolver, _bar(), 0.05)
    s.run(4000)
    assert s.erodedElements() == 0
    assert s.maxDamage() > 0.99


def test_bar_separates_and_keeps_momentum():
    """ErosionTest.barSeparates, erodedEnergyIsAccountedFor, invertedElementsAreCountedApart
    (:73-157)."""
    mesh = _bar()
    s = _stretching(OracleSolver, mesh, 0.05)
    s.setErosion(1.0)
    before = s.radialMomentum()
    s.run(4000)
    assert s.erodedElements() > 0
    assert abs(s.radialMomentum() - before) <= 1e-9 * max(1e-12, abs(before)) + 1e-14
    assert s.erodedEnergy() > 0.0
    assert s.erodedEnergy() < 0.05 * s.plasticDissipation()
    assert s.invertedElements() <= s.erodedElements()
    assert s.invertedElements() < 0.5 * mesh.elementCount


def test_surface_is_rebuilt_around_the_hole():
    """ErosionTest.surfaceIsRebuiltAroundTheHole (:116-139): removing an interior element
    adds its four faces to the surface."""
    mesh = Outline.rectangle(0.0, 0.0, 5.0 * MM, 5.0 * MM).mesh(MM)
    assert mesh.surface()[1].size == 20
    dead = np.zeros(mesh.elementCount, dtype=bool)
    rc, zc = mesh.centroidRadii(), mesh.centroidZs()
    middle = np.nonzero((np.abs(rc - 2.5 * MM) < 0.6 * MM) & (np.abs(zc - 2.5 * MM) < 0.6 * MM))[0]
    assert middle.size == 1
    dead[middle[0]] = True
    assert mesh.surface(dead)[1].size == 24


def test_mass_scaling_step_grows_as_square_root():
    """MassScalingTest.stepGrowsAsTheSquareRoot (:38-50)."""
    mesh = Outline.rectangle(0.0, 0.0, 6.0 * MM, 4.0 * MM).mesh(MM)
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)
    dt = s.timestep()
    s.setMassScaling(10.0 * dt)
    assert s.massScale() == pytest.approx(100.0, rel=1e-12)
    s.run(3)
    assert s.timestep() == pytest.approx(10.0 * dt, rel=1e-9)


# ----------------------------------------------------------------------------- threading

def test_threads_are_bit_identical():
    """ThreadingTest (:117-157): a Taylor impact with friction is bit for bit identical at
    2, 3, 5 and 8 threads, and when the count changes mid-run."""
    def run(threads, switch=None):
        s, _, _ = scenes.taylor_reference(OracleSolver, 4, friction=0.15)
        s.setThreads(threads)
        s.run(300)
        if switch:
            s.setThreads(switch)
        s.run(300)
        return [s.readField(f) for f in (0, 1, 2, 3, 4, 5, 7, 9)]
    base = run(1)
    for t, sw in ((2, None), (3, None), (5, None), (8, None), (3, 7)):
        other = run(t, sw)
        for a, b in zip(base, other):
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


# ----------------------------------------------------------------------------- math layer

def test_math_tables_match_their_generator():
    """nf_math_tables.h is what gen_nf_math_tables.py computes (every entry an exact value
    rounded to double)."""
    pytest.importorskip("mpmath")
    import subprocess
    import sys
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "neofiz_gb300", "csrc")
    out = subprocess.run([sys.executable, "gen_nf_math_tables.py"], cwd=csrc,
                         capture_output=True, text=True, check=True).stdout
    with open(os.path.join(csrc, "nf_math_tables.h")) as f:
        assert out.strip() == f.read().strip()


@pytest.mark.parametrize("name,gen", [
    ("log", lambda r: (math.exp(r.uniform(-700, 700)),)),
    ("log", lambda r: (1.0 + r.uniform(-0.01, 0.01),)),
    ("log", lambda r: (r.uniform(1e-320, 1e-308),)),
    ("exp", lambda r: (r.uniform(-708, 709),)),
    ("exp", lambda r: (r.uniform(-1e-3, 1e-3),)),
    ("pow", lambda r: (math.exp(r.uniform(-20, 2)), r.uniform(0.05, 1.6))),
    ("pow", lambda r: (math.exp(r.uniform(-50, 50)), r.uniform(-10, 10))),
    ("pow", lambda r: (1.0 + r.uniform(-1e-6, 1e-6), r.uniform(0.1, 1000))),
])
def test_table_driven_functions_within_half_an_ulp(name, gen):
    """The table-driven log, exp and pow against values exact to 120 bits: within 0.52 ulp
    (the Johnson-Cook law's strain, rate and thermal terms go through these three)."""
    mpmath = pytest.importorskip("mpmath")
    from oracle.oracle import math_fn
    import random
    mpmath.mp.prec = 120
    exact = {"log": mpmath.log, "exp": mpmath.exp, "pow": mpmath.power}[name]
    rnd = random.Random(7)
    worst = 0.0
    for _ in range(4000):
        args = gen(rnd)
        got = math_fn(name, *args) if len(args) == 2 else math_fn(name, args[0])
        want = exact(*[mpmath.mpf(a) for a in args])
        worst = max(worst, float(abs(mpmath.mpf(got) - want) / math.ulp(float(want))))
    assert worst <= 0.52


@pytest.mark.parametrize("name,fn,gen", [
    ("log", math.log, lambda r: (math.exp(r.uniform(-30, 30)),)),
    ("exp", math.exp, lambda r: (r.uniform(-700, 700),)),
    ("pow", math.pow, lambda r: (r.uniform(1e-12, 3.0), r.uniform(0.1, 1.2))),
    ("atan2", math.atan2, lambda r: (r.uniform(-5, 5), r.uniform(-5, 5))),
    ("sin", math.sin, lambda r: (r.uniform(-1.6, 1.6),)),
    ("cos", math.cos, lambda r: (r.uniform(-1.6, 1.6),)),
    ("hypot", math.hypot, lambda r: (r.uniform(-5, 5), r.uniform(-5, 5))),
])
def test_math_layer_within_a_few_ulp(name, fn, gen):
    """nf_math.h against the C library: within 3 ulp on the ranges the path uses."""
    from oracle.oracle import math_fn
    import random
    rnd = random.Random(1234)
    worst = 0.0
    for _ in range(20000):
        args = gen(rnd)
        got = math_fn(name, *args) if len(args) == 2 else math_fn(name, args[0])
        want = fn(*args)
        if want == got:
            continue
        worst = max(worst, abs(got - want) / math.ulp(want))
    assert worst <= 3.0
