"""Material records, mirroring the reference's core/ package.

``Formulation`` follows core/Formulation.java:16-31, ``Integration`` solver/Integration.java,
``Kinematics`` solver/Kinematics.java, ``JohnsonCook`` core/JohnsonCook.java:66-102,
``Material`` core/Material.java:20-135 and ``Materials`` core/Materials.java:23-128. The same
validation messages are raised (as ``ValueError``, the Python counterpart of
IllegalArgumentException).
"""
from __future__ import annotations

import enum
import math
from dataclasses import dataclass, replace
from typing import Callable, Optional, Sequence


class Formulation(enum.IntEnum):
    AXISYMMETRIC = 0
    PLANE_STRAIN = 1
    PLANE_STRESS = 2

    def isAxisymmetric(self) -> bool:
        return self is Formulation.AXISYMMETRIC


class Integration(enum.IntEnum):
    FULL = 0
    REDUCED = 1

    def gaussPoints(self) -> int:
        return 4 if self is Integration.FULL else 1


class Kinematics(enum.IntEnum):
    SMALL_STRAIN = 0
    FINITE_STRAIN = 1

    def isFinite(self) -> bool:
        return self is Kinematics.FINITE_STRAIN


@dataclass(frozen=True)
class JohnsonCook:
    """Johnson-Cook flow stress (core/JohnsonCook.java:66-89 for the checks)."""
    a: float
    b: float
    n: float
    c: float
    m: float
    referenceStrainRate: float
    roomTemperature: float
    meltTemperature: float
    specificHeat: float
    taylorQuinney: float

    def __post_init__(self):
        if self.a <= 0:
            raise ValueError("A must be positive")
        if self.b < 0:
            raise ValueError("B must be non-negative")
        if self.n <= 0 or self.n > 1:
            raise ValueError("n must lie in (0, 1]")
        if self.c < 0:
            raise ValueError("C must be non-negative")
        if self.m <= 0:
            raise ValueError("m must be positive")
        if self.referenceStrainRate <= 0:
            raise ValueError("reference strain rate must be positive")
        if self.meltTemperature <= self.roomTemperature:
            raise ValueError("melt temperature must exceed room temperature")
        if self.specificHeat <= 0:
            raise ValueError("specific heat must be positive")
        if self.taylorQuinney < 0 or self.taylorQuinney > 1:
            raise ValueError("Taylor-Quinney fraction must lie in [0, 1]")

    def quasiStatic(self) -> "JohnsonCook":
        """JohnsonCook.java:127-130: C = 0 and beta = 0."""
        return replace(self, c=0.0, taylorQuinney=0.0)

    def isQuasiStatic(self) -> bool:
        return self.c == 0.0 and self.taylorQuinney == 0.0

    def thermalCoefficient(self, density: float) -> float:
        return self.taylorQuinney / (density * self.specificHeat)

    def temperature(self, plasticWorkDensity: float, density: float) -> float:
        return self.roomTemperature + self.taylorQuinney * plasticWorkDensity / (
            density * self.specificHeat)


JohnsonCook.STEEL_4340 = JohnsonCook(792.0e6, 510.0e6, 0.26, 0.014, 1.03,
                                     1.0, 293.0, 1793.0, 477.0, 0.9)
JohnsonCook.COPPER_OFHC = JohnsonCook(90.0e6, 292.0e6, 0.31, 0.025, 1.09,
                                      1.0, 293.0, 1356.0, 383.0, 0.9)


@dataclass(frozen=True, eq=False)
class Material:
    """core/Material.java:20-39. ``yieldStress = inf`` is an elastic material."""
    name: str
    youngsModulus: float
    poissonRatio: float
    density: float
    yieldStress: float = math.inf
    isotropicHardening: float = 0.0
    kinematicHardening: float = 0.0
    johnsonCook: Optional[JohnsonCook] = None

    def __post_init__(self):
        if self.youngsModulus <= 0:
            raise ValueError("E must be positive")
        if self.poissonRatio <= -1.0 or self.poissonRatio >= 0.5:
            raise ValueError(f"nu must lie in (-1, 0.5); got {self.poissonRatio}")
        if self.density <= 0:
            raise ValueError("density must be positive")
        if self.yieldStress <= 0:
            raise ValueError("yield stress must be positive")
        if self.isotropicHardening < 0 or self.kinematicHardening < 0:
            raise ValueError("hardening moduli must be non-negative")
        if self.johnsonCook is not None and self.yieldStress != self.johnsonCook.a:
            raise ValueError(
                f"yield stress {self.yieldStress} disagrees with the Johnson-Cook A of "
                f"{self.johnsonCook.a}; the elastic check and the return map would be working "
                f"on different surfaces")

    def isElastic(self) -> bool:
        return math.isinf(self.yieldStress)

    def isRateDependent(self) -> bool:
        return self.johnsonCook is not None

    def yielding(self, yieldStress: float, isotropic: float, kinematic: float = 0.0) -> "Material":
        return Material(self.name, self.youngsModulus, self.poissonRatio, self.density,
                        yieldStress, isotropic, kinematic)

    def withJohnsonCook(self, law: JohnsonCook) -> "Material":
        """Material.java:87-90: JC replaces linear hardening, keeps H_kin."""
        return Material(self.name, self.youngsModulus, self.poissonRatio, self.density,
                        law.a, 0.0, self.kinematicHardening, law)

    def withKinematicHardening(self, hKin: float) -> "Material":
        return Material(self.name, self.youngsModulus, self.poissonRatio, self.density,
                        self.yieldStress, self.isotropicHardening, hKin, self.johnsonCook)

    def lambda_(self) -> float:
        nu = self.poissonRatio
        return self.youngsModulus * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def mu(self) -> float:
        return self.youngsModulus / (2.0 * (1.0 + self.poissonRatio))

    def dilatationalWaveSpeed(self) -> float:
        return math.sqrt((self.lambda_() + 2.0 * self.mu()) / self.density)

    def shearWaveSpeed(self) -> float:
        return math.sqrt(self.mu() / self.density)

    def barWaveSpeed(self) -> float:
        return math.sqrt(self.youngsModulus / self.density)


Material.STEEL_4340 = Material("AISI 4340", 205.0e9, 0.29, 7850.0)
Material.COPPER_OFHC = Material("OFHC Cu", 117.0e9, 0.34, 8960.0)


class Materials:
    """core/Materials.java: one material everywhere, or one per element."""

    def __init__(self, one: Optional[Material], each: Optional[Sequence[Material]]):
        self._one = one
        self._each = list(each) if each is not None else None
        self._table = None
        if self._each is not None:
            # the device's layout (distinct materials, per-element index), built once here
            # with C-level passes rather than per element in Python
            import numpy as np
            keys = list(map(id, self._each))
            objs = dict(zip(keys, self._each))
            order = list(dict.fromkeys(keys))               # first appearance
            slot = {k: i for i, k in enumerate(order)}
            index = np.fromiter(map(slot.__getitem__, keys), dtype=np.int32, count=len(keys))
            self._table = ([objs[k] for k in order], index)

    @staticmethod
    def uniform(material: Material) -> "Materials":
        if material is None:
            raise ValueError("material must not be null")
        return Materials(material, None)

    @staticmethod
    def of(*byElement: Material) -> "Materials":
        if len(byElement) == 0:
            raise ValueError("need at least one material")
        for e, m in enumerate(byElement):
            if m is None:
                raise ValueError(f"element {e} has no material")
        return Materials(None, byElement)

    @staticmethod
    def byElement(elementCount: int, pick: Callable[[int], Material]) -> "Materials":
        if elementCount < 1:
            raise ValueError("need at least one element")
        return Materials.of(*[pick(e) for e in range(elementCount)])

    def at(self, element: int) -> Material:
        return self._one if self._one is not None else self._each[element]

    def isUniform(self) -> bool:
        return self._one is not None

    def elementCount(self) -> int:
        return -1 if self._each is None else len(self._each)

    def requireCovers(self, elementCount: int) -> None:
        if self._each is not None and len(self._each) != elementCount:
            raise ValueError(f"materials cover {len(self._each)} elements but the mesh has "
                             f"{elementCount}")

    def distinct(self) -> list:
        """Distinct materials in first-appearance order, compared by identity."""
        if self._one is not None:
            return [self._one]
        return list(self._table[0])

    def table(self, elementCount: int):
        """(distinct materials, per-element index into them)."""
        import numpy as np
        if self._one is not None:
            return [self._one], np.zeros(elementCount, dtype=np.int32)
        return list(self._table[0]), self._table[1]

    def fastestWave(self) -> float:
        if self._one is not None:
            return self._one.dilatationalWaveSpeed()
        return max(m.dilatationalWaveSpeed() for m in self._each)
