"""DefectBurst (validate/DefectBurst.java:44-495): a copper tube with a Weibull defect field,
fired by a smoothstep bore pressure until its load capacity turns over, then run on past the
peak until a point fails; where and at what pressure it gave way, and how it bulged.

A caller of the timestep, written over the solver's public API exactly as the reference's is
over ExplicitSolver (`fire` takes the solver class, so the same driver runs the GPU solver or
the oracle). The capacity and hoop strain are BurstCase.loadCapacity and BurstCase.hoopStrain
(validate/BurstCase.java:533-569), computed on the host from the sampled fields every 250
steps; the steps between samples run on the device.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

from . import scenes
from .defects import DefectField, Weibull
from .materials import Formulation, Integration, Kinematics
from .mesh import QuadMesh

MEAN_RADIUS = 25.0e-3                  # BurstCase.MEAN_RADIUS
SLENDERNESS = 25.0                     # BurstCase.REFERENCE_SLENDERNESS
THROUGH_WALL = 4
TUBE_LENGTH = 40.0e-3
ALONG_AXIS = 40
CORRELATION = 3.0e-3
MODULUS = 12.0
SCALE = 0.04
FRACTURE_ENERGY = 12.0e3
REFERENCE_VOLUME = 2.0 * math.pi * MEAN_RADIUS * (2.0 * MEAN_RADIUS / SLENDERNESS) * TUBE_LENGTH
POST_PEAK_PERIODS = 60.0
CFL_SAFETY = 0.5


@dataclass(frozen=True)
class Setup:
    """DefectBurst.Setup (DefectBurst.java:272-341)."""
    failureScale: float = SCALE
    fractureEnergy: float = FRACTURE_ENERGY
    correlation: float = CORRELATION
    length: float = TUBE_LENGTH
    slenderness: float = SLENDERNESS
    throughWall: int = THROUGH_WALL
    alongAxis: int = ALONG_AXIS

    @staticmethod
    def nominal() -> "Setup":
        return Setup()

    def perfect(self) -> "Setup":
        return replace(self, failureScale=0.0)

    def withFailureScale(self, s: float) -> "Setup":
        return replace(self, failureScale=s)

    def withFractureEnergy(self, g: float) -> "Setup":
        return replace(self, fractureEnergy=g)

    def withCorrelation(self, c: float) -> "Setup":
        return replace(self, correlation=c)

    def withLength(self, length: float) -> "Setup":
        return replace(self, length=length,
                       alongAxis=int(math.floor(self.alongAxis * length / self.length + 0.5)))

    def withSlenderness(self, s: float) -> "Setup":
        return replace(self, slenderness=s)

    def refined(self, factor: int) -> "Setup":
        return replace(self, throughWall=self.throughWall * factor,
                       alongAxis=self.alongAxis * factor)

    def bandWidth(self) -> float:
        return self.length / self.alongAxis

    def thickness(self) -> float:
        return 2.0 * MEAN_RADIUS / self.slenderness


@dataclass(frozen=True)
class Shot:
    """DefectBurst.Shot (DefectBurst.java:150-161): one firing of one tube."""
    seed: int
    traversed: bool
    peakCapacity: float
    peakStrain: float
    peakApplied: float
    weakestStrain: float
    meanStrain: float
    failureZ: float
    maxDamage: float
    damagedFraction: float
    clampedPoints: int
    fractureEnergy: float
    plasticEnergy: float
    bulgeRatio: float
    steps: int

    def knockdown(self, reference: float) -> float:
        return self.peakCapacity / reference


def reference_pressure(slenderness: float = SLENDERNESS) -> float:
    """DefectBurst.referencePressure: the closed-form burst pressure with no defects."""
    return scenes.burst_pressure(scenes.burst_material().johnsonCook,
                                 2.0 * MEAN_RADIUS / slenderness, MEAN_RADIUS)


def _areas(mesh: QuadMesh, r: np.ndarray, z: np.ndarray) -> np.ndarray:
    c = np.asarray(mesh.conn).reshape(-1, 4)
    a = np.zeros(c.shape[0])
    for k in range(4):
        i, j = c[:, k], c[:, (k + 1) & 3]
        a += r[i] * z[j] - r[j] * z[i]
    return 0.5 * a


def load_capacity(solver, mesh: QuadMesh) -> float:
    """BurstCase.loadCapacity (BurstCase.java:533-553): the hoop stress integrated over the
    current section, over the bore radius times the height."""
    deformed = solver.kinematics() == Kinematics.FINITE_STRAIN
    ur, uz = solver.radialDisplacement(), solver.axialDisplacement()
    r = mesh.r + ur if deformed else np.asarray(mesh.r)
    z = mesh.z + uz if deformed else np.asarray(mesh.z)
    hoop = np.asarray(solver.stress()).reshape(-1, 4)[:, 2]
    hoop_area = 0.0
    for h, a in zip(hoop.tolist(), _areas(mesh, r, z).tolist()):
        hoop_area += h * a                     # in element order, as the reference sums
    return hoop_area / (float(np.min(r)) * (float(np.max(z)) - float(np.min(z))))


def hoop_strain(solver, mesh: QuadMesh, mean_radius: float) -> float:
    """BurstCase.hoopStrain (BurstCase.java:555-569): log hoop strain at mid-wall."""
    r = mesh.r + solver.radialDisplacement()
    return math.log(0.5 * (float(np.min(r)) + float(np.max(r))) / mean_radius)


def bulge_ratio(solver, nr: int, nz: int) -> float:
    """DefectBurst.bulgeRatio (DefectBurst.java:483-494): the largest bore expansion along the
    tube over the mean of them."""
    ur = solver.radialDisplacement()
    bore = [float(ur[j * (nr + 1)]) for j in range(nz + 1)]
    total = 0.0
    for u in bore:
        total += u
    average = total / (nz + 1)
    return max(0.0, max(bore)) / average if average > 0.0 else 1.0


def fire(seed: int, setup: Setup = Setup(), solver_class=None) -> Shot:
    """DefectBurst.fire (DefectBurst.java:370-472)."""
    if solver_class is None:
        from .solver import ExplicitSolver as solver_class
    copper = scenes.burst_material()
    law = copper.johnsonCook
    nr, nz = setup.throughWall, setup.alongAxis
    thickness = setup.thickness()
    inner, outer = MEAN_RADIUS - 0.5 * thickness, MEAN_RADIUS + 0.5 * thickness
    mesh = QuadMesh.cylinderWall(inner, outer, setup.length, nr, nz)
    solver = solver_class(mesh, copper, Formulation.AXISYMMETRIC, Integration.REDUCED,
                          Kinematics.FINITE_STRAIN, 1.0, CFL_SAFETY)
    solver.fixAllAxial()
    weakest = mean = 0.0
    if setup.failureScale > 0.0:
        field = DefectField(Weibull(setup.failureScale, MODULUS), REFERENCE_VOLUME,
                            setup.correlation, seed)
        failure = field.sampleOnto(mesh)
        weakest = float(np.min(failure))
        total = 0.0
        for f in failure.tolist():
            total += f
        mean = total / failure.size
        solver.setDamage(setup.fractureEnergy, failure)

    exact = scenes.burst_pressure(law, thickness, MEAN_RADIUS)
    ceiling = scenes.BURST_OVERSHOOT * exact
    omega = copper.barWaveSpeed() / MEAN_RADIUS
    period = 2.0 * math.pi / omega
    solver.setPressureRamp(ceiling, scenes.BURST_RAMP_PERIODS * period)
    solver.setRelaxationDamping(scenes.BURST_DAMPING, omega)

    traversed = False
    peak_capacity = peak_strain = peak_applied = 0.0
    deadline = scenes.BURST_MAX_PERIODS * period
    while solver.time() < deadline:
        solver.run(scenes.BURST_SAMPLE_STEPS)
        capacity = load_capacity(solver, mesh)
        if capacity > peak_capacity:
            peak_capacity = capacity
            peak_strain = hoop_strain(solver, mesh, MEAN_RADIUS)
            peak_applied = solver.borePressure()
        elif (solver.borePressure() >= ceiling
              and capacity < peak_capacity * (1.0 - scenes.BURST_PEAK_MARGIN)):
            traversed = True
            break

    # past the peak, and kept running until a point fails (DefectBurst.java:429-446)
    run_on = solver.time() + POST_PEAK_PERIODS * period
    damaged = setup.failureScale > 0.0
    while traversed and solver.time() < run_on and (not damaged or solver.maxDamage() < 1.0):
        solver.run(scenes.BURST_SAMPLE_STEPS)

    failure_z, max_damage, damaged_fraction, clamped, fracture = math.nan, 0.0, 0.0, 0, 0.0
    if damaged:
        max_damage = solver.maxDamage()
        damaged_fraction = solver.damagedFraction()
        clamped = int(solver.damage().clampedPoints())
        worst = solver.mostDamagedElement()
        if worst >= 0:
            failure_z = float(mesh.centroidZ(worst))
        fracture = solver.fractureDissipation()
    return Shot(seed, traversed, peak_capacity, peak_strain, peak_applied, weakest, mean,
                failure_z, max_damage, damaged_fraction, clamped, fracture,
                solver.plasticDissipation(), bulge_ratio(solver, nr, nz), int(solver.steps()))
