"""Regularised damage at one material point on the oracle, re-expressing
solver/DamageTest.java (:44-333): the softening triangle's area is G_f / h, the band is
oriented by the flow, the softening return is exact, a fully damaged point keeps only its
pressure, the dissipation deficit is one step in n, the fracture energy is per unit crack
area, snap-back clamps at -E, Johnson-Cook softens through the closed form, and an unreachable
failure strain changes nothing, bit for bit. The same return map runs on the device; the GPU
parity tests hold it to these bits."""
import math

import numpy as np

from neofiz_gb300 import JohnsonCook, Material
from neofiz_gb300.solver import material_point_update
from oracle.oracle import api as oracle_api

E, NU, SY = 205.0e9, 0.29, 800.0e6
MU = E / (2.0 * (1.0 + NU))
LAMBDA = E * NU / ((1.0 + NU) * (1.0 - 2.0 * NU))
GF = 50.0e3
EPS_F = 0.20
DT = 1.0e-8


def box(dr, dz):
    return np.array([dr * dz, dr, 0.0, 0.0, dz])


class Point:
    """DamageTest.Point: one material point driven along a fixed deviatoric axis."""

    def __init__(self, material, failure_strain=EPS_F, dr=0.5e-3, dz=0.5e-3, damage=True):
        self.m = material
        self.sig = np.zeros(4)
        self.back = np.zeros(4)
        self.eps = np.zeros(1)
        self.work = np.zeros(1)
        self.damage = None
        if damage:
            self.damage = {"failure_strain": np.array([failure_strain]),
                           "fracture_energy": np.array([GF]),
                           "youngs_modulus": np.array([E]), "geometry": box(dr, dz),
                           "strength": np.zeros(1), "softening": np.zeros(1),
                           "width": np.zeros(1)}

    @staticmethod
    def linear(hIso, dr=0.5e-3, dz=0.5e-3):
        return Point(Material("pt", E, NU, 7850.0, SY, hIso, 0.0), dr=dr, dz=dz)

    def strain(self, dRR, dZZ, dTT, dGam):
        material_point_update(self.m, self.sig, self.back, self.eps, self.work,
                              np.array([dRR, dZZ, dTT, dGam]), DT, damage=self.damage,
                              binding=oracle_api())

    def pull(self, d):
        self.strain(-0.5 * d, d, -0.5 * d, 0.0)

    def begun(self):
        return self.damage["strength"][0] > 0.0

    def sf(self):
        return float(self.damage["strength"][0])

    def slope(self):
        return float(self.damage["softening"][0])

    def width(self):
        return float(self.damage["width"][0])

    def damage_now(self):
        """Damage.at (Damage.java:342-347)."""
        sf = self.sf()
        if sf <= 0.0:
            return 0.0
        v = -self.slope() * (self.eps[0] - EPS_F) / sf
        return min(1.0, max(0.0, v))

    def dissipation(self, eps):
        """Damage.dissipation: the area under the softening line from onset to eps."""
        x = min(max(eps - EPS_F, 0.0), self.sf() / -self.slope())
        return self.sf() * x + 0.5 * self.slope() * x * x

    def mises(self):
        s = self.sig
        p = (s[0] + s[1] + s[2]) / 3.0
        a, b, c, d = s[0] - p, s[1] - p, s[2] - p, s[3]
        return math.sqrt(1.5 * (a * a + b * b + c * c + 2.0 * d * d))

    def soften_to_failure(self, step):
        while not self.begun():
            self.pull(step)
        self.work_at_onset = float(self.work[0])
        self.strain_at_onset = float(self.eps[0])
        self.softening_steps = 0
        while self.damage_now() < 1.0:
            self.pull(step)
            self.softening_steps += 1
        self.pull(step)
        return float(self.work[0]) - self.work_at_onset


def test_the_triangle_is_exact():
    p = Point.linear(2.0e9)
    while not p.begun():
        p.pull(1.0e-5)
    h, sf = p.width(), p.sf()
    rng = sf / -p.slope()
    full = p.dissipation(EPS_F + rng)
    assert abs(full - GF / h) <= GF / h * 1e-14
    assert abs(full - 0.5 * sf * rng) <= full * 1e-14
    assert abs(p.dissipation(EPS_F + 10.0 * rng) - full) <= full * 1e-14
    assert p.dissipation(EPS_F - 0.01) == 0.0


def test_the_band_is_oriented_by_the_flow():
    dz = 0.4e-3
    for dr in (0.05e-3, 0.4e-3, 4.0e-3):
        p = Point.linear(2.0e9, dr, dz)
        while not p.begun():
            p.pull(1.0e-5)
        assert abs(p.width() - dz) <= dz * 1e-12, dr


def test_softening_is_exactly_on_the_surface():
    p = Point.linear(2.0e9)
    while not p.begun():
        p.pull(1.0e-5)
    sf, slope = p.sf(), p.slope()
    assert slope < 0.0
    checked = 0
    while p.damage_now() < 1.0:
        p.pull(1.0e-5)
        assert abs(max(0.0, sf + slope * (p.eps[0] - EPS_F)) - p.mises()) <= SY * 1e-13
        checked += 1
    assert checked > 100


def test_full_damage_leaves_pressure_only():
    p = Point.linear(2.0e9)
    p.soften_to_failure(1.0e-5)
    assert p.damage_now() == 1.0
    assert p.mises() <= SY * 1e-12
    d = -1.0e-4
    p.strain(d, d, d, 0.0)
    want = -(3.0 * LAMBDA + 2.0 * MU) * d
    pressure = -(p.sig[0] + p.sig[1] + p.sig[2]) / 3.0          # J2.pressure, J2.java:386-389
    assert abs(pressure - want) <= abs(want) * 1e-12
    assert p.mises() <= SY * 1e-12


def test_the_solver_undershoots_by_one_step_in_n():
    previous = None
    for step in (4.0e-5, 2.0e-5, 1.0e-5):
        p = Point.linear(2.0e9)
        spent = p.soften_to_failure(step)
        exact = p.dissipation(p.eps[0]) - p.dissipation(p.strain_at_onset)
        deficit = (exact - spent) / exact
        n = p.softening_steps
        assert abs(deficit - 1.0 / n) <= 0.2 / n, (step, deficit, n)
        if previous is not None:
            assert deficit < 0.6 * previous
        previous = deficit
    assert previous < 0.01


def test_the_fracture_energy_is_per_unit_area():
    """The four band widths run side by side as four points of one call; a point that has
    finished gets zero strain increments, which leave it exactly as it is."""
    widths = np.array([0.1e-3, 0.3e-3, 0.9e-3, 2.7e-3])
    n = widths.size
    m = Material("pt", E, NU, 7850.0, SY, 2.0e9, 0.0)
    sig, back, eps, work = np.zeros(4 * n), np.zeros(4 * n), np.zeros(n), np.zeros(n)
    damage = {"failure_strain": np.full(n, EPS_F), "fracture_energy": np.full(n, GF),
              "youngs_modulus": np.full(n, E),
              "geometry": np.concatenate([box(0.5e-3, w) for w in widths]),
              "strength": np.zeros(n), "softening": np.zeros(n), "width": np.zeros(n)}
    step = 2.0e-6
    onset_work = np.full(n, np.nan)
    extra = np.zeros(n, dtype=int)                   # pulls after full damage (one, as there)
    while np.any(extra < 1):
        live = extra < 1
        d = np.where(live, step, 0.0)
        strain = np.stack([-0.5 * d, d, -0.5 * d, np.zeros(n)], axis=1).ravel()
        begun_before = damage["strength"] > 0.0
        full_before = begun_before & (np.clip(-damage["softening"] * (eps - EPS_F)
                                              / np.where(begun_before, damage["strength"], 1.0),
                                              0.0, 1.0) >= 1.0)
        material_point_update(m, sig, back, eps, work, strain, DT, damage=damage,
                              binding=oracle_api())
        extra += (live & full_before).astype(int)
        newly = np.isnan(onset_work) & (damage["strength"] > 0.0)
        onset_work[newly] = work[newly]
    per_volume = work - onset_work
    per_area = per_volume * damage["width"]
    assert np.all(damage["softening"] != -E)
    assert np.all(np.abs(per_area - per_area[0]) <= per_area[0] * 0.02)
    assert abs(per_area[0] - GF) <= GF * 0.02
    ratio = widths[3] / widths[0]
    assert abs(per_volume[0] / per_volume[3] - ratio) <= ratio * 0.03


def test_snap_back_is_clamped():
    probe = Point.linear(2.0e9)
    while not probe.begun():
        probe.pull(1.0e-5)
    limit = 2.0 * GF * E / (probe.sf() * probe.sf())   # Damage.largestRegularisableElement
    fine = Point.linear(2.0e9, 0.5e-3, 0.5 * limit)
    while not fine.begun():
        fine.pull(1.0e-5)
    assert fine.slope() != -E
    coarse = Point.linear(2.0e9, 0.5e-3, 2.0 * limit)
    while not coarse.begun():
        coarse.pull(1.0e-5)
    assert coarse.slope() == -E
    before = coarse.mises()
    coarse.pull(1.0e-5)
    assert math.isfinite(coarse.mises()) and coarse.mises() < before
    assert 2.0 * MU - (2.0 / 3.0) * E > 0.0


def test_johnson_cook_softens_without_iterating():
    law = JohnsonCook.STEEL_4340
    p = Point(Material.STEEL_4340.withJohnsonCook(law))
    while not p.begun():
        p.pull(1.0e-5)
    sf, slope = p.sf(), p.slope()
    checked = 0
    while p.damage_now() < 1.0:
        p.pull(1.0e-5)
        assert abs(max(0.0, sf + slope * (p.eps[0] - EPS_F)) - p.mises()) <= sf * 1e-13
        checked += 1
    assert checked > 50
    assert sf > law.a


def test_an_unreachable_failure_strain_changes_nothing():
    m = Material("pt", E, NU, 7850.0, SY, 2.0e9, 1.0e9)
    plain = Point(m, damage=False)
    armed = Point(m, failure_strain=10.0)
    for _ in range(4000):
        plain.pull(1.0e-5)
        armed.pull(1.0e-5)
    assert armed.eps[0] > 0.03
    assert np.array_equal(plain.sig, armed.sig)
    assert np.array_equal(plain.back, armed.back)
    assert plain.eps[0] == armed.eps[0] and plain.work[0] == armed.work[0]
    assert armed.damage["strength"][0] == 0.0
