"""Batched scenes: many independent solver instances stepped together on one GPU.

The reference runs a parameter sweep as one ``ExplicitSolver`` per host thread
(``Sweep.over``, app/Sweep.java:82-105); here the whole sweep is one handle
(``nf_batch_*`` in include/neofiz.h). Each ``Instance`` is the sequence

    ExplicitSolver(mesh, material, formulation, REDUCED, kinematics, thickness, cfl)
    setHourglassCoefficient(q); fixRadial/fixAxial(...); setRigidWall(RigidWall.atZ(z, mu));
    setUniformVelocity(vr, vz); step while time < t_end

and its trajectory is bit-identical to that scene run alone through ``ExplicitSolver`` in the
same precision.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _abi
from .materials import Formulation, Kinematics, Material
from .mesh import QuadMesh
from .solver import DeviceError


@dataclass
class Instance:
    mesh: QuadMesh
    material: Material
    t_end: float
    velocity: tuple = (0.0, 0.0)
    wall: Optional[tuple] = None          # (plane, friction) or None
    hourglass: float = 0.05
    fixed_radial: Sequence[int] = field(default_factory=tuple)
    fixed_axial: Sequence[int] = field(default_factory=tuple)
    pressure: tuple = (0.0, 0.0)          # setPressureRamp(pascals, seconds), on the mesh's edges
    damping: Optional[tuple] = None       # setRelaxationDamping(fraction, omega)
    damage: Optional[tuple] = None        # setDamage(gf[E], eps[E]); all instances or none


def _raise(api, handle, status):
    msg = api.batch_last_error(handle)
    msg = msg.decode() if msg else f"status {status}"
    if status == _abi.NF_EINVAL:
        raise ValueError(msg)
    if status == _abi.NF_ESTATE:
        raise RuntimeError(msg)
    raise DeviceError(msg)


class BatchSolver:
    """A sweep of independent instances (``nf_batch_create`` ... ``nf_batch_destroy``)."""

    @classmethod
    def _binding(cls):
        from . import _native
        return _native.api()

    def __init__(self, instances: Sequence[Instance], formulation: Formulation,
                 kinematics: Kinematics = Kinematics.FINITE_STRAIN, thickness: float = 1.0,
                 cfl: float = 0.6, precision: int = _abi.PRECISION_FP64):
        self._api = self._binding()
        self._handle = None
        if not instances:
            raise ValueError("a batch needs at least one instance")
        self.instances = list(instances)
        count = len(self.instances)
        nodes = np.array([0] + [i.mesh.nodeCount for i in self.instances], dtype=np.int64)
        elems = np.array([0] + [i.mesh.elementCount for i in self.instances], dtype=np.int64)
        self.node_offset = np.cumsum(nodes).astype(np.int32)
        self.element_offset = np.cumsum(elems).astype(np.int32)
        self._r = np.concatenate([i.mesh.r for i in self.instances]).astype(np.float64)
        self._z = np.concatenate([i.mesh.z for i in self.instances]).astype(np.float64)
        self._conn = np.concatenate([i.mesh.conn for i in self.instances]).astype(np.int32)
        edges = np.array([0] + [i.mesh.pressureEdges.size // 2 for i in self.instances],
                         dtype=np.int64)
        self.pressure_offset = np.cumsum(edges).astype(np.int32)
        self._pedges = (np.concatenate([i.mesh.pressureEdges for i in self.instances])
                        .astype(np.int32) if edges.sum() else np.zeros(2, np.int32))
        damaged = [i.damage is not None for i in self.instances]
        if any(damaged) and not all(damaged):
            raise ValueError("damage is set on every instance of a batch or on none")
        if all(damaged):
            self._gf = np.concatenate([np.broadcast_to(np.asarray(i.damage[0], np.float64),
                                                       (i.mesh.elementCount,))
                                       for i in self.instances]).astype(np.float64)
            self._eps = np.concatenate([np.asarray(i.damage[1], np.float64)
                                        for i in self.instances]).astype(np.float64)
        self._fixed = np.zeros(int(self.node_offset[-1]), dtype=np.uint8)
        for k, inst in enumerate(self.instances):
            n0 = int(self.node_offset[k])
            for n in inst.fixed_radial:
                self._fixed[n0 + n] |= 1
            for n in inst.fixed_axial:
                self._fixed[n0 + n] |= 2
        cm = _abi.BatchMesh()
        cm.instance_count = count
        cm.node_offset = self.node_offset.ctypes.data_as(_abi.c_int32_p)
        cm.element_offset = self.element_offset.ctypes.data_as(_abi.c_int32_p)
        cm.r = self._r.ctypes.data_as(_abi.c_double_p)
        cm.z = self._z.ctypes.data_as(_abi.c_double_p)
        cm.conn = self._conn.ctypes.data_as(_abi.c_int32_p)
        cm.fixed = self._fixed.ctypes.data_as(C.POINTER(C.c_uint8))
        cm.pressure_offset = self.pressure_offset.ctypes.data_as(_abi.c_int32_p)
        cm.pressure_edges = self._pedges.ctypes.data_as(_abi.c_int32_p)
        if all(damaged):
            cm.failure_strain = self._eps.ctypes.data_as(_abi.c_double_p)
            cm.fracture_energy = self._gf.ctypes.data_as(_abi.c_double_p)
        table = (_abi.BatchInstance * count)()
        for k, inst in enumerate(self.instances):
            t = table[k]
            t.material = _abi.material_struct(inst.material)
            t.velocity_r, t.velocity_z = float(inst.velocity[0]), float(inst.velocity[1])
            if inst.wall is None:
                t.wall_plane, t.wall_friction = math.nan, 0.0
            else:
                t.wall_plane, t.wall_friction = float(inst.wall[0]), float(inst.wall[1])
            t.hourglass = float(inst.hourglass)
            t.t_end = float(inst.t_end)
            t.pressure, t.pressure_ramp = float(inst.pressure[0]), float(inst.pressure[1])
            if inst.damping is not None:
                t.damping_fraction, t.damping_omega = map(float, inst.damping)
        out = C.c_void_p()
        st = self._api.batch_create(C.byref(cm), table, int(formulation), int(kinematics),
                                    float(thickness), float(cfl), int(precision), C.byref(out))
        if st:
            _raise(self._api, None, st)
        self._handle = out
        self.precision = precision
        self.count = count

    # ------------------------------------------------------------------ lifecycle

    def close(self):
        if self._handle is not None:
            self._api.batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            _raise(self._api, self._handle, st)

    # ------------------------------------------------------------------ shapes

    def tune(self, trial_steps: int = 32) -> dict:
        """The autotuner: times every valid launch shape, keeps the fastest."""
        c = _abi.BatchConfig()
        self._check(self._api.batch_tune(self._handle, int(trial_steps), C.byref(c)))
        return self.config()

    def config(self) -> dict:
        c = _abi.BatchConfig()
        self._check(self._api.batch_get_config(self._handle, C.byref(c)))
        return {"threads": c.threads, "stage_nodes": c.stage_nodes,
                "blocks_per_sm": c.blocks_per_sm, "chunk_steps": c.chunk_steps}

    def setConfig(self, threads: int, stage_nodes: int, blocks_per_sm: int, chunk_steps: int):
        c = _abi.BatchConfig(threads, stage_nodes, blocks_per_sm, chunk_steps)
        self._check(self._api.batch_set_config(self._handle, C.byref(c)))

    # ------------------------------------------------------------------ run

    def run(self, max_steps: int = 1 << 40) -> float:
        """Steps every instance to its t_end (or max_steps more steps); returns device ms."""
        self._check(self._api.batch_run(self._handle, int(max_steps)))
        return self.elapsed()

    def elapsed(self) -> float:
        ms = C.c_double()
        self._check(self._api.batch_elapsed(self._handle, C.byref(ms)))
        return ms.value

    def launchCount(self) -> int:
        n = C.c_int64()
        self._check(self._api.batch_launch_count(self._handle, C.byref(n)))
        return n.value

    # ------------------------------------------------------------------ reads

    def read(self, field: int) -> np.ndarray:
        count, eb = C.c_size_t(), C.c_size_t()
        self._check(self._api.batch_field_size(self._handle, field, C.byref(count), C.byref(eb)))
        dtype = {8: np.float64, 1: np.uint8, 4: np.int32}[eb.value]
        out = np.empty(count.value, dtype=dtype)
        self._check(self._api.batch_read(self._handle, field, out.ctypes.data_as(C.c_void_p),
                                         out.nbytes))
        return out

    def readInstance(self, field: int, k: int) -> np.ndarray:
        a = self.read(field)
        if a.size == self.node_offset[-1]:
            return a[self.node_offset[k]:self.node_offset[k + 1]]
        per = a.size // max(1, int(self.element_offset[-1]))
        return a[per * self.element_offset[k]:per * self.element_offset[k + 1]]

    def state(self) -> dict:
        s = (_abi.BatchProgress * self.count)()
        self._check(self._api.batch_state(self._handle, s))
        return {"time": np.array([x.time for x in s]),
                "timestep": np.array([x.timestep for x in s]),
                "steps": np.array([x.steps for x in s], dtype=np.int64),
                "status": np.array([x.status for x in s], dtype=np.uint32),
                "done": np.array([x.done for x in s], dtype=bool)}

    def measure(self) -> List[_abi.Measure]:
        m = (_abi.Measure * self.count)()
        self._check(self._api.batch_measure(self._handle, m))
        return list(m)

    def wallStats(self) -> List[_abi.WallInfo]:
        w = (_abi.WallInfo * self.count)()
        self._check(self._api.batch_wall_stats(self._handle, w))
        return list(w)

    # ------------------------------------------------------------------ burst measurement

    def setBurst(self, sampleEvery: int, meanRadius, margin: float = 0.005,
                 traceCapacity: int = 0) -> None:
        """BurstCase.run's sampling on every instance (nf_batch_set_burst): capacity, hoop
        strain (about meanRadius[k]) and applied pressure every sampleEvery steps; an instance
        stops once past its capacity peak. sampleEvery 0 turns it off."""
        cfg = _abi.BatchBurst(int(sampleEvery), int(traceCapacity), float(margin))
        self._burstRadius = np.ascontiguousarray(
            np.broadcast_to(np.asarray(meanRadius, np.float64), (self.count,)))
        self._traceCapacity = int(traceCapacity)
        self._check(self._api.batch_set_burst(self._handle, C.byref(cfg),
                                              self._burstRadius.ctypes.data_as(_abi.c_double_p)))

    def burstResults(self) -> dict:
        r = (_abi.BurstResult * self.count)()
        self._check(self._api.batch_burst_results(self._handle, r))
        keys = ("peak_capacity", "peak_strain", "peak_applied", "capacity", "strain",
                "applied", "samples", "traversed")
        return {k: np.array([getattr(x, k) for x in r]) for k in keys}

    def burstTrace(self) -> np.ndarray:
        """[count, traceCapacity, 4]: time, hoop strain, capacity, applied per sample."""
        out = np.zeros((self.count, self._traceCapacity, 4))
        self._check(self._api.batch_burst_trace(self._handle,
                                                out.ctypes.data_as(_abi.c_double_p)))
        return out

    # ------------------------------------------------------------------ adjoint

    def adjointForward(self, checkpointEvery: int = 200, sampleEvery: int = 0) -> float:
        """Runs every instance to its t_end keeping checkpoints (FP64 batches), sampling the
        wall capacity every sampleEvery steps (0: not sampled); device ms."""
        self._check(self._api.batch_adjoint_forward(self._handle, int(checkpointEvery),
                                                    int(sampleEvery)))
        return self.adjointElapsed()[0]

    def adjointBackward(self, objective: int = _abi.OBJECTIVE_LENGTH_RATIO):
        """(values[count], gradients[count, PARAM_COUNT]) of the objective after the forward
        pass's steps (or at its sampled capacity peak), with respect to A, B, n, C, m, the
        kinematic modulus, friction and the fracture energy."""
        values = np.zeros(self.count)
        grads = np.zeros((self.count, _abi.PARAM_COUNT))
        self._check(self._api.batch_adjoint_backward(
            self._handle, int(objective), values.ctypes.data_as(_abi.c_double_p),
            grads.ctypes.data_as(_abi.c_double_p)))
        return values, grads

    def adjointBackwardMany(self, objectives: Sequence[int]):
        """Several objectives in one backward pass (one segment recompute shared):
        (values[len, count], gradients[len, count, PARAM_COUNT]), each objective's gradients
        bit-identical to adjointBackward(objective)."""
        obj = np.asarray(list(objectives), dtype=np.int32)
        values = np.zeros((obj.size, self.count))
        grads = np.zeros((obj.size, self.count, _abi.PARAM_COUNT))
        self._check(self._api.batch_adjoint_backward_many(
            self._handle, obj.ctypes.data_as(_abi.c_int32_p), int(obj.size),
            values.ctypes.data_as(_abi.c_double_p), grads.ctypes.data_as(_abi.c_double_p)))
        return values, grads

    def adjointElapsed(self):
        f, b = C.c_double(), C.c_double()
        self._check(self._api.batch_adjoint_elapsed(self._handle, C.byref(f), C.byref(b)))
        return f.value, b.value

    def elementCycles(self) -> int:
        """Element-steps taken so far: sum over instances of elements x steps."""
        steps = self.state()["steps"]
        elems = np.diff(self.element_offset).astype(np.int64)
        return int(np.sum(steps * elems))
