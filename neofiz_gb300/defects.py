"""Host-side Weibull defect field: per-element failure strains for the damage model.

Restates core/DefectField.java (smoothed hash-seeded white noise, :239-347) and
core/Weibull.java (quantiles, size scaling, :114-164) in numpy. The field is a function of
position only, so the same seed gives the same failure strain at the same place on any mesh
(DefectFieldTest.java:112). The noise hash is the reference's SplitMix64-style mix
(DefectField.java:325-347); the Box-Muller transform and the normal cdf use numpy/scipy
rather than the reference's Cody erfc, so values agree with the reference to rounding, not
bit for bit. The failure strains are set-up data handed to ExplicitSolver.setDamage.
"""
from __future__ import annotations

import math

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_SALT = np.uint64(0xD6E8FEB86659FD93)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _unit_open(bits: np.ndarray) -> np.ndarray:
    return ((bits >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0 ** -53


class Weibull:
    """Two-parameter Weibull (core/Weibull.java:36-164)."""

    def __init__(self, scale: float, modulus: float):
        if not (scale > 0.0):
            raise ValueError(f"scale must be positive, was {scale}")
        if not (modulus > 0.0):
            raise ValueError(f"modulus must be positive, was {modulus}")
        self.scale = float(scale)
        self.modulus = float(modulus)

    def quantile(self, p):
        return self.scale * np.power(-np.log1p(-np.asarray(p)), 1.0 / self.modulus)

    def quantileFromSurvival(self, s):
        return self.scale * np.power(-np.log(np.asarray(s)), 1.0 / self.modulus)

    def minimumOf(self, n: float) -> "Weibull":
        if not (n > 0.0):
            raise ValueError(f"sample count must be positive, was {n}")
        return Weibull(self.scale * n ** (-1.0 / self.modulus), self.modulus)

    def forVolume(self, volume: float, referenceVolume: float) -> "Weibull":
        if not (volume > 0.0):
            raise ValueError(f"volume must be positive, was {volume}")
        if not (referenceVolume > 0.0):
            raise ValueError(f"reference volume must be positive, was {referenceVolume}")
        return self.minimumOf(volume / referenceVolume)


class DefectField:
    """Smoothed Gaussian field mapped through a Weibull law (core/DefectField.java)."""

    CELLS_PER_LENGTH = 3
    KERNEL_RADII = 4.0
    CLAMP_SIGMA = 9.0

    def __init__(self, base: Weibull, referenceVolume: float, correlationLength: float, seed: int):
        if not (referenceVolume > 0.0):
            raise ValueError(f"reference volume must be positive, was {referenceVolume}")
        if not (correlationLength > 0.0):
            raise ValueError(f"correlation length must be positive, was {correlationLength}")
        self.base = base
        self.referenceVolume = referenceVolume
        self.correlationLength = correlationLength
        self.seed = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.cell = correlationLength / self.CELLS_PER_LENGTH
        self.sigmaCells = (correlationLength / math.sqrt(2.0)) / self.cell
        self.radius = int(math.ceil(self.KERNEL_RADII * self.sigmaCells))

    def white(self, i: np.ndarray, j: np.ndarray) -> np.ndarray:
        """Unit normal deviate per lattice site (DefectField.java:325-332)."""
        i = np.asarray(i, dtype=np.int64).astype(np.uint64)
        j = np.asarray(j, dtype=np.int64).astype(np.uint64)
        with np.errstate(over="ignore"):
            h = _mix(np.full(i.shape, self.seed, dtype=np.uint64) + _GOLD)
            h = _mix(h ^ (i * _M1))
            h = _mix(h ^ (j * _M2))
        u1 = _unit_open(h)
        u2 = _unit_open(_mix(h ^ _SALT))
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)

    def gaussianAt(self, r, z) -> np.ndarray:
        """Separable Gaussian window over the lattice noise (DefectField.java:289-319)."""
        r = np.atleast_1d(np.asarray(r, dtype=np.float64))
        z = np.atleast_1d(np.asarray(z, dtype=np.float64))
        gr = r / self.cell
        gz = z / self.cell
        i0 = np.floor(gr).astype(np.int64) - self.radius
        j0 = np.floor(gz).astype(np.int64) - self.radius
        taps = 2 * self.radius + 2
        two = 2.0 * self.sigmaCells * self.sigmaCells
        k = np.arange(taps)
        wr = np.exp(-((gr[:, None] - (i0[:, None] + k)) ** 2) / two)
        wz = np.exp(-((gz[:, None] - (j0[:, None] + k)) ** 2) / two)
        norm = np.sqrt((wr * wr).sum(axis=1) * (wz * wz).sum(axis=1))
        out = np.empty(r.size)
        if r.size == 0:
            return out
        # The noise of a lattice site is the same for every point whose window covers it: when
        # the windows' lattice box is small (a mesh much finer than the lattice), evaluate each
        # site once and gather; the sums below are the same either way.
        ilo, jlo = int(i0.min()), int(j0.min())
        ni, nj = int(i0.max()) - ilo + taps, int(j0.max()) - jlo + taps
        grid = None
        if ni * nj <= min(r.size * taps * taps, 1 << 26):
            gi = np.arange(ilo, ilo + ni, dtype=np.int64)
            gj = np.arange(jlo, jlo + nj, dtype=np.int64)
            grid = self.white(np.broadcast_to(gi[None, :], (nj, ni)),
                              np.broadcast_to(gj[:, None], (nj, ni)))
        chunk = 4096
        for s in range(0, r.size, chunk):
            e = min(r.size, s + chunk)
            ii = i0[s:e, None, None] + k[None, None, :]
            jj = j0[s:e, None, None] + k[None, :, None]
            if grid is not None:
                noise = grid[jj - jlo, ii - ilo]
            else:
                noise = self.white(np.broadcast_to(ii, (e - s, taps, taps)),
                                   np.broadcast_to(jj, (e - s, taps, taps)))
            row = (noise * wr[s:e, None, :]).sum(axis=2)
            out[s:e] = (row * wz[s:e, :]).sum(axis=1)
        return out / norm

    def _transform(self, g: np.ndarray, volume) -> np.ndarray:
        from math import sqrt
        try:
            from scipy.special import erfc
        except ImportError:                       # pragma: no cover
            from math import erfc as _e
            erfc = np.vectorize(_e)
        # one-dimensional arrays throughout: numpy evaluates a 0-d power by a different routine
        # than an array's, and a point's value must not depend on how it was batched
        volume = np.atleast_1d(np.asarray(volume, dtype=np.float64))
        g = np.atleast_1d(np.asarray(g, dtype=np.float64))
        local_scale = self.base.scale * (volume / self.referenceVolume) ** (
            -1.0 / self.base.modulus)
        c = np.clip(g, -self.CLAMP_SIGMA, self.CLAMP_SIGMA)
        cdf = 0.5 * erfc(-c / sqrt(2.0))
        surv = 0.5 * erfc(c / sqrt(2.0))
        weak = local_scale * np.power(-np.log1p(-cdf), 1.0 / self.base.modulus)
        strong = local_scale * np.power(-np.log(surv), 1.0 / self.base.modulus)
        return np.where(c <= 0.0, weak, strong)

    def failureStrainForVolume(self, r, z, volume) -> np.ndarray:
        """DefectField.java:233-236: the field at (r, z) for a given volume."""
        return self._transform(self.gaussianAt(r, z), volume)

    def effectiveVolume(self, centroidRadius, crossSectionArea):
        """DefectField.java:204-208 (axisymmetric rings)."""
        l = self.correlationLength
        inPlane = np.maximum(1.0, np.asarray(crossSectionArea) / (l * l))
        hoop = np.maximum(1.0, 2.0 * math.pi * np.asarray(centroidRadius) / l)
        return l * l * l * inPlane * hoop

    def sampleOnto(self, mesh) -> np.ndarray:
        """DefectField.sampleOnto, DefectField.java:239-248 (axisymmetric size effect)."""
        rc = mesh.centroidRadii()
        zc = mesh.centroidZs()
        g = self.gaussianAt(rc, zc)
        return self._transform(g, self.effectiveVolume(rc, mesh.signedAreas()))
