"""The energy audit on a freely vibrating bar, on the oracle, re-expressing
solver/EnergyAuditTest.java (:35-111): kinetic energy from the half-step velocity biases the
budget of a vibrating body to first order in the step; the centred kinetic energy
(ExplicitSolver.centredKineticEnergy) removes most of it and converges to second order."""
import math

import pytest

from neofiz_gb300 import Formulation, Integration, Kinematics, Material, Outline
from oracle.oracle import OracleSolver

CELL = 1.0e-3
DEPTH = 10.0e-3


def vibrating(cfl, cls=OracleSolver):
    mesh = Outline.rectangle(0.0, 0.0, 20.0 * CELL, 8.0 * CELL).mesh(CELL)
    s = cls(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.FINITE_STRAIN, DEPTH, cfl)
    for i in range(mesh.nodeCount):
        s.setVelocity(i, 60.0 * math.sin(math.pi * mesh.r[i] / (20.0 * CELL)), 0.0)
    return s


def drift(cfl, samples, per, centred, cls=OracleSolver):
    s = vibrating(cfl, cls)
    kinetic = s.centredKineticEnergy if centred else s.kineticEnergy
    initial = kinetic() + s.strainEnergy() + s.hourglassEnergy()
    worst = 0.0
    for _ in range(samples):
        s.run(per)
        total = kinetic() + s.strainEnergy() + s.hourglassEnergy()
        worst = max(worst, abs(total / initial - 1.0))
    return worst


def test_vibration_biases_the_half_step_audit():
    assert drift(0.5, 200, 20, False) > 0.005


def test_centring_removes_the_bias():
    assert drift(0.5, 200, 20, True) < drift(0.5, 200, 20, False) / 5.0


def test_orders_of_convergence():
    half_ratio = drift(0.5, 200, 20, False) / drift(0.125, 200, 80, False)
    centred_ratio = drift(0.5, 200, 20, True) / drift(0.125, 200, 80, True)
    assert 3.0 < half_ratio < 7.0
    assert centred_ratio > 8.0
    assert centred_ratio > 2.0 * half_ratio


@pytest.mark.gpu
def test_the_device_audit_shows_the_same_orders(gpu_lib):
    """The same budget from the device's audit kernels."""
    from neofiz_gb300 import ExplicitSolver
    half_ratio = drift(0.5, 200, 20, False, ExplicitSolver) / drift(0.125, 200, 80, False,
                                                                    ExplicitSolver)
    centred_ratio = drift(0.5, 200, 20, True, ExplicitSolver) / drift(0.125, 200, 80, True,
                                                                      ExplicitSolver)
    assert 3.0 < half_ratio < 7.0
    assert centred_ratio > 8.0 and centred_ratio > 2.0 * half_ratio
