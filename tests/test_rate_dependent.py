"""The Johnson-Cook return map at one point on the oracle, re-expressing
solver/RateDependentReturnMapTest.java (:97-302): the solved state lies on the surface at the
strain, rate and temperature the step produced; rate hardening is the law's logarithm;
plastic heating softens; the flow is incompressible; no step ends outside the surface; the
plastic work is the flow stress times the plastic strain increment. The device runs the same
return map and the GPU parity tests hold it to the oracle's bits."""
import math

import numpy as np

from neofiz_gb300 import JohnsonCook, Material
from neofiz_gb300.solver import material_point_update
from oracle.oracle import api as oracle_api, jc_flow_stress

E, NU, DENSITY = 205.0e9, 0.29, 7850.0
MU = E / (2.0 * (1.0 + NU))
LAMBDA = E * NU / ((1.0 + NU) * (1.0 - 2.0 * NU))
SY = 800.0e6
ROOM = 293.0


def law(a, b, n, c, beta):
    return JohnsonCook(a, b, n, c, 1.03, 1.0, ROOM, 1793.0, 477.0, beta)


class Point:
    """RateDependentReturnMapTest.Point: J2.Flow(A, 0, 0, law, beta / (rho cp))."""

    def __init__(self, jc):
        self.jc = jc
        self.m = Material("jc", E, NU, DENSITY).withJohnsonCook(jc)
        self.sig, self.back = np.zeros(4), np.zeros(4)
        self.eps, self.work = np.zeros(1), np.zeros(1)

    def shear(self, dGam, dt):
        return float(material_point_update(self.m, self.sig, self.back, self.eps, self.work,
                                           np.array([0.0, 0.0, 0.0, dGam]), dt,
                                           binding=oracle_api())[0])

    def mises(self):
        s = self.sig
        p = (s[0] + s[1] + s[2]) / 3.0
        a, b, c, d = s[0] - p, s[1] - p, s[2] - p, s[3]
        return math.sqrt(1.5 * (a * a + b * b + c * c + 2.0 * d * d))

    def pressure(self):
        return -(self.sig[0] + self.sig[1] + self.sig[2]) / 3.0

    def temperature(self):
        return self.jc.temperature(float(self.work[0]), DENSITY)


def test_the_solved_state_lands_on_the_surface():
    p = Point(JohnsonCook.STEEL_4340)
    dt, dgam = 2.0e-8, 5.0e-4
    previous = 0.0
    for _ in range(600):
        temperature = p.temperature()
        if p.shear(dgam, dt) == 0.0:
            continue
        rate = (p.eps[0] - previous) / dt
        previous = float(p.eps[0])
        expected = jc_flow_stress(p.m, float(p.eps[0]), rate, temperature)
        assert abs(expected - p.mises()) <= expected * 1e-9
    assert previous > 0.01


def drive(jc, dt):
    p = Point(jc)
    for _ in range(2000):
        p.shear(2.0e-4, dt)
    assert p.eps[0] > 0.1
    return p.mises()


def test_rate_hardening_is_the_logarithm():
    jc = law(SY, 0.0, 0.26, 0.014, 0.0)
    slow, fast = drive(jc, 1.0e-5), drive(jc, 1.0e-9)
    assert fast > slow * 1.02
    assert abs(fast / slow - (1.0 + 0.014 * math.log(1.0e4))) <= 0.02


def test_plastic_heating_softens():
    adiabatic = drive(law(SY, 0.0, 0.26, 0.0, 0.9), 1.0e-8)
    isothermal = drive(law(SY, 0.0, 0.26, 0.0, 0.0), 1.0e-8)
    assert adiabatic < isothermal
    assert abs(isothermal - SY) <= SY * 1e-9


def test_plastic_flow_changes_no_volume():
    p = Point(JohnsonCook.STEEL_4340)
    for _ in range(50):
        p.shear(5.0e-4, 1.0e-8)
        assert abs(p.pressure()) <= 1.0
    assert p.eps[0] > 0.0


def test_the_stress_never_ends_outside_the_surface():
    p = Point(JohnsonCook.STEEL_4340)
    for dgam in (1e-3, 5e-3, 2e-2, 1e-1, 5e-2, 1e-3):
        before = float(p.eps[0])
        temperature = p.temperature()
        p.shear(dgam, 1.0e-8)
        rate = (p.eps[0] - before) / 1.0e-8
        surface = jc_flow_stress(p.m, float(p.eps[0]), rate, temperature)
        assert p.mises() <= surface * (1.0 + 1e-8), dgam


def test_plastic_work_is_flow_stress_times_strain():
    p = Point(JohnsonCook.STEEL_4340)
    expected, previous = 0.0, 0.0
    for _ in range(40):
        p.shear(5.0e-4, 1.0e-8)
        expected += p.mises() * (p.eps[0] - previous)
        previous = float(p.eps[0])
    assert abs(expected - p.work[0]) <= expected * 1e-3
    assert p.work[0] > 0.0
