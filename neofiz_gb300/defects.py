"""Host-side Weibull defect field: per-element failure strains for the damage model.

Restates core/DefectField.java (smoothed hash-seeded white noise, :239-347), core/Normal.java
(Cody's erfc, :50-129) and core/Weibull.java (quantiles, size scaling, :114-164). The
arithmetic runs in libneofiz_host.so (csrc/defect_field.c, built by neofiz_gb300.build) in the
reference's operation order -- the window's sums row by row, Cody's rational erfc, log1p on the
weak side -- over the deterministic elementary functions the kernels and the oracle share, so a
field is bit-identical on every host rather than dependent on a platform's libm. The field is a
function of position only, so the same seed gives the same failure strain at the same place on
any mesh (DefectFieldTest.java:112). The failure strains are set-up data handed to
ExplicitSolver.setDamage.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

_lib = None


def _host():
    """libneofiz_host.so, built on first use."""
    global _lib
    if _lib is None:
        from . import build
        lib = C.CDLL(build.build_host())
        d, i64, u64 = C.c_double, C.c_int64, C.c_uint64
        dp, lp = C.POINTER(C.c_double), C.POINTER(C.c_int64)
        lib.nf_field_gaussian.argtypes = [d, u64, i64, dp, dp, dp]
        lib.nf_field_gaussian.restype = C.c_int
        lib.nf_field_failure_strain.argtypes = [d, d, d, d, u64, i64, dp, dp, dp, dp]
        lib.nf_field_failure_strain.restype = C.c_int
        lib.nf_field_white.argtypes = [u64, i64, lp, lp, dp]
        lib.nf_field_white.restype = None
        lib.nf_normal.argtypes = [i64, dp, dp, dp]
        lib.nf_normal.restype = None
        lib.nf_weibull_quantile.argtypes = [d, d, C.c_int, i64, dp, dp]
        lib.nf_weibull_quantile.restype = None
        lib.nf_weibull_size_factor.argtypes = [d, d]
        lib.nf_weibull_size_factor.restype = d
        _lib = lib
    return _lib


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def normal_cdf(x) -> np.ndarray:
    """Normal.cdf, core/Normal.java:33-35."""
    x = _arr(x)
    out = np.empty_like(x)
    _host().nf_normal(x.size, _p(x), _p(out), None)
    return out


def normal_survival(x) -> np.ndarray:
    """Normal.survival, core/Normal.java:43-45."""
    x = _arr(x)
    out = np.empty_like(x)
    _host().nf_normal(x.size, _p(x), None, _p(out))
    return out


class Weibull:
    """Two-parameter Weibull (core/Weibull.java:36-164)."""

    def __init__(self, scale: float, modulus: float):
        if not (scale > 0.0):
            raise ValueError(f"scale must be positive, was {scale}")
        if not (modulus > 0.0):
            raise ValueError(f"modulus must be positive, was {modulus}")
        self.scale = float(scale)
        self.modulus = float(modulus)

    def _quantile(self, p, survival: int):
        p = _arr(p)
        bad = ~((p >= 0.0) & (p <= 1.0))
        if np.any(bad):
            raise ValueError(f"probability must lie in [0, 1], was {p[bad][0]}")
        out = np.empty_like(p)
        _host().nf_weibull_quantile(self.scale, self.modulus, survival, p.size, _p(p), _p(out))
        return out

    def quantile(self, p):
        """Weibull.quantile, :114-119: scale (-log1p(-p))^(1/m)."""
        return self._quantile(p, 0)

    def quantileFromSurvival(self, s):
        """Weibull.quantileFromSurvival, :126-131: scale (-log s)^(1/m)."""
        return self._quantile(s, 1)

    def minimumOf(self, n: float) -> "Weibull":
        if not (n > 0.0):
            raise ValueError(f"sample count must be positive, was {n}")
        return Weibull(self.scale * _host().nf_weibull_size_factor(float(n), self.modulus),
                       self.modulus)

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
        self.seed = seed & 0xFFFFFFFFFFFFFFFF
        self.cell = correlationLength / self.CELLS_PER_LENGTH
        self.sigmaCells = (correlationLength / math.sqrt(2.0)) / self.cell
        self.radius = int(math.ceil(self.KERNEL_RADII * self.sigmaCells))

    def white(self, i, j) -> np.ndarray:
        """Unit normal deviate per lattice site (DefectField.java:325-332)."""
        i = np.ascontiguousarray(np.atleast_1d(np.asarray(i, dtype=np.int64)))
        j = np.ascontiguousarray(np.broadcast_to(np.asarray(j, dtype=np.int64), i.shape))
        out = np.empty(i.shape)
        lp = C.POINTER(C.c_int64)
        _host().nf_field_white(int(self.seed), i.size, i.ctypes.data_as(lp),
                               j.ctypes.data_as(lp), _p(out))
        return out

    def gaussianAt(self, r, z) -> np.ndarray:
        """Separable Gaussian window over the lattice noise (DefectField.java:289-319)."""
        r, z = _arr(r), _arr(z)
        out = np.empty(r.size)
        st = _host().nf_field_gaussian(self.correlationLength, int(self.seed), r.size, _p(r),
                                       _p(z), _p(out))
        if st:
            raise MemoryError("the defect field's lattice does not fit in host memory")
        return out

    def failureStrainForVolume(self, r, z, volume) -> np.ndarray:
        """DefectField.java:233-236: the field at (r, z) for a given volume, through the
        copula (:262-274) to the volume's Weibull law."""
        r, z = _arr(r), _arr(z)
        volume = np.ascontiguousarray(np.broadcast_to(_arr(volume), r.shape))
        out = np.empty(r.size)
        st = _host().nf_field_failure_strain(self.base.scale, self.base.modulus,
                                             self.referenceVolume, self.correlationLength,
                                             int(self.seed), r.size, _p(r), _p(z), _p(volume),
                                             _p(out))
        if st:
            raise MemoryError("the defect field's lattice does not fit in host memory")
        return out

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
        return self.failureStrainForVolume(rc, zc, self.effectiveVolume(rc, mesh.signedAreas()))
