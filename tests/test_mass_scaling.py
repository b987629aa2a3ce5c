"""Mass scaling on the oracle, re-expressing solver/MassScalingTest.java (:52-127) (the
square-root step is in test_oracle_pins.py): gravity is untouched, momentum and kinetic
energy are wrong by exactly the factor, a shorter target is refused and changes nothing, and
the contact stiffness follows the scaled step."""
import math

import numpy as np
import pytest

from neofiz_gb300 import (Contact, Formulation, Integration, Kinematics, Material, Outline,
                          RigidWall)
from oracle.oracle import OracleSolver

MM = 1.0e-3
G = 9.81


def block(scale):
    mesh = Outline.rectangle(0.0, 0.0, 8.0 * MM, 8.0 * MM).mesh(MM)
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.SMALL_STRAIN, 10.0 * MM, 0.5)
    if scale > 1.0:
        s.setMassScaling(s.timestep() * math.sqrt(scale))
    return s


def lowest(s):
    return min(0.0, float(np.min(s.axialDisplacement())))


def test_falling_is_unaffected():
    plain, heavy = block(1.0), block(400.0)
    plain.setGravity(0.0, -G)
    heavy.setGravity(0.0, -G)
    for s in (plain, heavy):
        while s.time() < 200.0e-6:
            s.run(1)
    drop_plain, drop_heavy = lowest(plain), lowest(heavy)
    assert abs(drop_heavy / drop_plain - 1.0) < 0.01
    assert drop_plain < 0.0


def test_inertia_is_wrong_by_the_factor():
    plain, heavy = block(1.0), block(25.0)
    for s in (plain, heavy):
        for i in range(s.mesh.nodeCount):
            s.setVelocity(i, 0.0, -50.0)
    assert abs(heavy.axialMomentum() / plain.axialMomentum() - 25.0) <= 1e-9
    assert abs(heavy.kineticEnergy() / plain.kineticEnergy() - 25.0) <= 1e-9


def test_will_not_remove_mass():
    s = block(1.0)
    now = s.timestep()
    with pytest.raises(ValueError):
        s.setMassScaling(now * 0.5)
    with pytest.raises(ValueError):
        s.setMassScaling(0.0)
    assert s.massScale() == 1.0
    assert s.timestep() == now


def test_contact_stays_stable():
    mesh = Outline.assemble(MM, Outline.rectangle(0.0, 0.0, 8.0 * MM, 4.0 * MM),
                            Outline.rectangle(0.0, 4.0 * MM, 8.0 * MM, 8.0 * MM))
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)
    s.setMassScaling(s.timestep() * 10.0)
    s.setContact(Contact(mesh))
    s.setGravity(0.0, -G)
    s.setRigidWall(RigidWall.atZ(0.0))
    s.run(4000)
    assert math.isfinite(s.kineticEnergy())
    assert s.kineticEnergy() < 1.0e-3
    assert lowest(s) > -MM
