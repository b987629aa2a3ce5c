"""The lattice mesher (neofiz_gb300/mesh.py, Outline), re-expressing mesh/OutlineTest.java and
mesh/AssembleTest.java: exact cell counts and welds, the cell size as every edge, area
convergence, holes, rigid transforms, refusals, and welded versus assembled bodies (the
weld-versus-stack pull runs on the oracle)."""
import math

import numpy as np
import pytest

from neofiz_gb300 import (Contact, Formulation, Integration, Kinematics, Material, Outline,
                          QuadMesh)

H = 1.0e-3
MM = 1.0e-3


def area(mesh):
    return float(mesh.signedAreas().sum())


def test_rectangle_is_exact():
    mesh = Outline.rectangle(0.0, 0.0, 10.0 * H, 6.0 * H).mesh(H)
    assert mesh.elementCount == 60
    assert mesh.nodeCount == 11 * 7
    assert abs(area(mesh) - 60.0 * H * H) < 1e-15


def test_every_edge_is_the_cell_size():
    mesh = Outline.circle(20.0 * H, 20.0 * H, 8.0 * H, 40).mesh(H)
    assert abs(mesh.minimumEdgeLength() - H) < 1e-15


def test_disc_area_converges():
    radius = 20.0 * H
    disc = Outline.circle(0.0, 0.0, radius, 180)
    coarse = abs(area(disc.mesh(2.0 * H)) / (math.pi * radius * radius) - 1.0)
    fine = abs(area(disc.mesh(0.5 * H)) / (math.pi * radius * radius) - 1.0)
    assert fine < coarse
    assert fine < 0.01


def test_holes_are_subtracted():
    plate = Outline.rectangle(0.0, 0.0, 20.0 * H, 20.0 * H)
    bored = plate.withHole(Outline.rectangle(8.0 * H, 8.0 * H, 12.0 * H, 12.0 * H))
    assert abs(plate.area() - 400.0 * H * H) < 1e-18
    assert abs(bored.area() - 384.0 * H * H) < 1e-18
    assert bored.mesh(H).elementCount == 400 - 16
    assert not bored.contains(10.0 * H, 10.0 * H)
    assert bored.contains(2.0 * H, 2.0 * H)


def test_shared_lattice_welds():
    left = Outline.rectangle(0.0, 0.0, 5.0 * H, 5.0 * H)
    touching = Outline.rectangle(5.0 * H, 0.0, 10.0 * H, 5.0 * H)
    apart = Outline.rectangle(9.0 * H, 0.0, 14.0 * H, 5.0 * H)
    joined = Outline.meshOf(H, left, touching)
    assert (joined.elementCount, joined.nodeCount) == (50, 11 * 6)
    separate = Outline.meshOf(H, left, apart)
    assert (separate.elementCount, separate.nodeCount) == (50, 2 * 6 * 6)


def test_rigid_transforms_preserve_area():
    bracket = Outline.of(0.0, 0.0, 30.0 * H, 0.0, 30.0 * H, 12.0 * H,
                         12.0 * H, 12.0 * H, 12.0 * H, 40.0 * H, 0.0, 40.0 * H)
    c = bracket.centre()
    turned = bracket.rotated(math.radians(18.0), c[0], c[1]).restingOn(0.0)
    assert abs(bracket.area() - turned.area()) <= 1e-12 * bracket.area()
    assert abs(turned.bounds()[1]) <= 1e-18
    assert abs(turned.mesh(H).elementCount - bracket.mesh(H).elementCount) < 30


def test_refuses_what_it_cannot_mesh():
    with pytest.raises(ValueError):
        Outline.rectangle(0.0, 0.0, 1.0e-6, 1.0e-6).mesh(H)
    with pytest.raises(ValueError):
        Outline.rectangle(0.0, 0.0, H, H).mesh(0.0)
    with pytest.raises(ValueError):
        Outline.of(0.0, 0.0, 1.0, 1.0)


LOWER = Outline.rectangle(0.0, 0.0, 6.0 * MM, 6.0 * MM)
UPPER = Outline.rectangle(0.0, 6.0 * MM, 6.0 * MM, 12.0 * MM)


def test_touching_shapes_weld_when_meshed_and_not_when_assembled():
    welded = Outline.meshOf(MM, LOWER, UPPER)
    stacked = Outline.assemble(MM, LOWER, UPPER)
    assert welded.elementCount == stacked.elementCount == 72
    assert welded.nodeCount == 7 * 13
    assert stacked.nodeCount == 2 * 7 * 7 == welded.nodeCount + 7


def _lower_block_rise(mesh):
    from oracle.oracle import OracleSolver
    s = OracleSolver(mesh, Material.STEEL_4340, Formulation.PLANE_STRAIN, Integration.REDUCED,
                     Kinematics.FINITE_STRAIN, 10.0 * MM, 0.5)
    s.setContact(Contact(mesh))
    for i in range(mesh.nodeCount):
        if mesh.z[i] > 6.0 * MM:
            s.setVelocity(i, 0.0, 40.0)
    s.run(1500)
    uz = s.axialDisplacement()
    return float(np.max(uz[np.asarray(mesh.z) == 0.0]))


def test_a_weld_carries_tension_and_a_stack_does_not():
    """AssembleTest.aWeldCarriesTensionAndAStackDoesNot: pull the upper block up; welded, the
    lower block's base rises; stacked, it stays."""
    assert _lower_block_rise(Outline.meshOf(MM, LOWER, UPPER)) > 1.0e-6
    assert abs(_lower_block_rise(Outline.assemble(MM, LOWER, UPPER))) < 1.0e-9


def test_an_assembled_stack_has_a_surface_per_body():
    blocks = [Outline.rectangle(0.0, i * 5.0 * MM, 4.0 * MM, (i + 1) * 5.0 * MM) for i in range(6)]
    mesh = Outline.assemble(MM, *blocks)
    edges, owner, nodes = mesh.surface()
    assert len(owner) == 6 * 2 * (4 + 5)
    assert mesh.elementCount == 6 * 4 * 5
