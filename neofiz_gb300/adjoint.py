"""The adjoint as a function with a hand-written reverse: the Python twin of the Java
binding's org.neofiz.gpu.GpuAdjoint (DifferentiableFunction).

``forward(params)`` builds a sweep from one parameter vector per case (the caller's template:
A, B, n, C, m, the kinematic modulus, the wall friction, the fracture energy, the yield
stress, the isotropic modulus -- the adjoint's parameter order), runs it forward with
checkpoints and returns each case's objective; ``backward(seed)`` runs the reverse sweep
(decisions frozen from the forward pass) and returns seed[k] times case k's gradient. Each
case's objective depends only on its own parameters, so that is the whole vector-Jacobian
product. The reference has no adjoint; the gradients are checked against central differences
and against the FP64 reference adjoint of the oracle.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

from . import _abi
from .batch import BatchSolver
from .materials import Formulation

PARAMETERS = len(_abi.PARAM_NAMES)


class AdjointFunction:
    """forward: parameters (cases x PARAMETERS) -> objective values (cases);
    backward: seed (cases) -> seed-weighted gradients (cases x PARAMETERS)."""

    def __init__(self, template: Callable[[np.ndarray], Sequence], formulation: Formulation,
                 cfl: float, objective: int = _abi.OBJECTIVE_LENGTH_RATIO,
                 checkpoint_every: int = 200, sample_every: int = 0,
                 batch_class=BatchSolver, **batch_kw):
        if objective == _abi.OBJECTIVE_PEAK_CAPACITY and sample_every <= 0:
            raise ValueError("the peak capacity needs a sampling interval")
        self.template = template
        self.formulation = formulation
        self.cfl = cfl
        self.objective = objective
        self.every = checkpoint_every
        self.sample_every = sample_every
        self.batch_class = batch_class
        self.batch_kw = batch_kw
        self._batch = None
        self._values = None
        self._grads = None

    def forward(self, params) -> np.ndarray:
        params = np.asarray(params, dtype=np.float64)
        self.close()
        cases = self.template(params)
        b = self.batch_class(cases, self.formulation, cfl=self.cfl, **self.batch_kw)
        b.adjointForward(self.every, self.sample_every)
        self._batch = b
        self._grads = None
        if self.objective == _abi.OBJECTIVE_PEAK_CAPACITY:
            self._reverse()                   # the sampled peak is known after the reverse
            return self._values.copy()
        m = b.measure()
        if self.objective == _abi.OBJECTIVE_LENGTH_RATIO:
            l0 = np.array([float(np.ptp(c.mesh.z)) for c in cases])
            self._values = np.array([x.length for x in m]) / l0
        else:
            self._values = np.array([x.mushroom_diameter for x in m])
        return self._values.copy()

    __call__ = forward

    def _reverse(self):
        v, g = self._batch.adjointBackward(self.objective)
        self._values = np.asarray(v, dtype=np.float64)
        self._grads = np.asarray(g, dtype=np.float64)

    def backward(self, seed) -> np.ndarray:
        if self._batch is None:
            raise RuntimeError("backward before forward")
        if self._grads is None:
            self._reverse()
        seed = np.asarray(seed, dtype=np.float64)
        return seed[:, None] * self._grads

    def close(self):
        if self._batch is not None:
            self._batch.close()
        self._batch = None


def rod_template(rods, base=None):
    """A template for the Taylor-rod sweeps of neofiz_gb300.scenes: parameter vector k sets
    rod k's Johnson-Cook A, B, n, C, m, kinematic modulus and wall friction."""
    import dataclasses
    from . import scenes

    def build(params):
        out = []
        for rod, p in zip(rods, params):
            inst = scenes.sweep_instances([rod])[0]
            jc = dataclasses.replace(scenes._rod_jc(rod), a=p[0], b=p[1], n=p[2], c=p[3], m=p[4])
            inst.material = scenes.rod_material_with(jc).withKinematicHardening(p[5])
            inst.wall = (inst.wall[0], p[6])
            out.append(inst)
        return out
    return build


def rod_parameters(rods) -> np.ndarray:
    """The parameter vectors of the rods as drawn (the adjoint's order)."""
    from . import scenes
    out = np.zeros((len(rods), PARAMETERS))
    for k, rod in enumerate(rods):
        jc = scenes._rod_jc(rod)
        mat = scenes.rod_material_with(jc)
        out[k, :7] = (jc.a, jc.b, jc.n, jc.c, jc.m, mat.kinematicHardening, rod["mu"])
    return out
