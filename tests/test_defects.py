"""The host-side defect field (neofiz_gb300/defects.py), re-expressing the properties of
core/DefectFieldTest.java and core/WeibullTest.java: the smoothed noise is standard normal with
the Gaussian correlation it is built for, it is a function of position only (two meshes of the
same body see the same field, bit for bit), and the volume law floors as the reference's does.
"""
import math

import numpy as np
import pytest

from neofiz_gb300 import QuadMesh
from neofiz_gb300.defects import DefectField, Weibull

BASE = Weibull(0.42, 20.0)
V0 = 1e-9
LENGTH = 1e-3


def field(seed):
    return DefectField(BASE, V0, LENGTH, seed)


@pytest.mark.parametrize("seed", [1, 7, 20260919])
def test_gaussian_marginal_is_standard(seed):
    """DefectFieldTest.gaussianMarginalIsStandard (:39-65): 300 x 300 points a third of a
    correlation length apart; mean within 0.05 of 0, variance within 0.07 of 1."""
    i, j = np.meshgrid(np.arange(300), np.arange(300), indexing="ij")
    g = field(seed).gaussianAt(0.05 + i.ravel() * 0.37e-3, 0.01 + j.ravel() * 0.41e-3)
    mean = g.mean()
    assert abs(mean) < 0.05
    assert abs((g * g).mean() - mean * mean - 1.0) < 0.07


def test_correlation_follows_the_kernel():
    """DefectFieldTest.correlationFollowsTheKernel (:66-95): exp(-d^2 / 2 l^2) within 0.03."""
    f = field(11)
    i, j = np.meshgrid(np.arange(260), np.arange(260), indexing="ij")
    r = 0.05 + i.ravel() * 0.29e-3
    z = 0.01 + j.ravel() * 0.31e-3
    a = f.gaussianAt(r, z)
    for lengths in (0.25, 0.5, 1.0, 1.5, 2.0):
        d = lengths * LENGTH
        b = f.gaussianAt(r + d, z)
        measured = (a * b).sum() / math.sqrt((a * a).sum() * (b * b).sum())
        assert abs(math.exp(-d * d / (2.0 * LENGTH * LENGTH)) - measured) < 0.03, lengths


def test_correlation_endpoints():
    """DefectFieldTest.correlationEndpoints (:96-107)."""
    f = field(3)
    a = f.gaussianAt(0.06, 0.02)[0]
    assert a == f.gaussianAt(0.06, 0.02)[0]
    assert abs(a - f.gaussianAt(0.06 + 0.02 * LENGTH, 0.02)[0]) < 0.05


def test_two_meshes_of_one_body_see_the_same_field():
    """DefectFieldTest.refiningTheMeshResolvesTheSameField (:109-144): the same seed gives the
    same value at a point, evaluated alone or among any other points; another seed differs;
    sampling a mesh equals evaluating each centroid on its own."""
    f = field(42)
    r, z = np.meshgrid(np.arange(0.051, 0.0999, 0.0037), np.arange(0.001, 0.0199, 0.0031),
                       indexing="ij")
    r, z = r.ravel(), z.ravel()
    together = f.gaussianAt(r, z)
    alone = np.array([field(42).gaussianAt(a, b)[0] for a, b in zip(r, z)])
    assert np.array_equal(together.view(np.uint64), alone.view(np.uint64))
    assert np.all(field(43).gaussianAt(r, z) != together)
    coarse = QuadMesh.cylinderWall(0.05, 0.10, 0.02, 4, 2)
    fine = QuadMesh.cylinderWall(0.05, 0.10, 0.02, 64, 32)
    sampled = f.sampleOnto(coarse)
    rc, zc, area = coarse.centroidRadii(), coarse.centroidZs(), coarse.signedAreas()
    for e in range(coarse.elementCount):
        pointwise = f.failureStrainForVolume(rc[e], zc[e], f.effectiveVolume(rc[e], area[e]))[0]
        assert pointwise == sampled[e], e
    # the fine mesh's centroids see the same field as points evaluated alone
    rf, zf = fine.centroidRadii()[::97], fine.centroidZs()[::97]
    assert np.array_equal(f.gaussianAt(fine.centroidRadii(), fine.centroidZs())[::97],
                          np.array([f.gaussianAt(a, b)[0] for a, b in zip(rf, zf)]))


def test_lattice_gather_and_direct_evaluation_agree():
    """Points far apart (each window's noise evaluated directly) and the same points one at a
    time (each window gathered from a memoised lattice) give the same bits."""
    f = field(5)
    r = np.array([0.001, 0.9, 0.25])
    z = np.array([0.002, 0.7, 0.0])
    far = f.gaussianAt(r, z)
    one = np.array([f.gaussianAt(a, b)[0] for a, b in zip(r, z)])
    assert np.array_equal(far.view(np.uint64), one.view(np.uint64))


def test_the_resolution_floor():
    """DefectFieldTest.theResolutionFloor (:146-176)."""
    f = field(1)
    r = 0.075
    coarse = 4.0 * LENGTH * LENGTH
    assert abs(f.effectiveVolume(r, coarse) - 2.0 * math.pi * r * coarse) <= 2.0 * math.pi * r * coarse * 1e-12
    fine = 0.25 * LENGTH * LENGTH
    ring = 2.0 * math.pi * r * LENGTH * LENGTH
    assert abs(f.effectiveVolume(r, fine) - ring) <= ring * 1e-12
    assert f.effectiveVolume(r, fine) == f.effectiveVolume(r, fine / 1000.0)
    assert abs(f.effectiveVolume(r, coarse) / (LENGTH * coarse) - 2.0 * math.pi * r / LENGTH) < 1e-9
    assert abs(f.effectiveVolume(1e-9, coarse) - 4.0 * LENGTH ** 3) < 4e-18


def test_weibull_volume_law():
    """WeibullTest: minimumOf(1) is the identity, minimumOf composes, forVolume is minimumOf
    the volume ratio, and the median is scale (ln 2)^(1/m)."""
    steel = Weibull(1.0, 20.0)
    assert steel.minimumOf(1.0).scale == steel.scale
    once = steel.minimumOf(12.0)
    twice = steel.minimumOf(3.0).minimumOf(4.0)
    assert abs(once.scale - twice.scale) <= once.scale * 1e-14
    assert steel.minimumOf(8.0).scale == steel.forVolume(8e-6, 1e-6).scale
    assert abs(steel.quantile(0.5) - math.log(2.0) ** (1.0 / 20.0)) < 1e-15
    for s in (1e-6, 0.1, 0.5, 0.9):
        assert abs(steel.quantileFromSurvival(s) - steel.quantile(1.0 - s)) < 1e-12
    with pytest.raises(ValueError):
        Weibull(0.0, 2.0)
    with pytest.raises(ValueError):
        steel.forVolume(0.0, 1.0)
