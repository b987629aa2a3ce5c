"""The drop-in surface: ``ExplicitSolver``, ``RigidWall`` and ``Contact`` with the reference's
method names, argument meaning and error behaviour, backed by libneofiz_gpu.so.

Reference: solver/ExplicitSolver.java (public API :237-1936), solver/RigidWall.java:110-315,
solver/Contact.java:273-404, solver/Damage.java:268-412. Differences, all forced by the state
living on the device:

* getters return copies (numpy arrays) rather than live arrays; callers that wrote into the
  reference's live arrays use the setters (``setVelocity``) or ``writeField``;
* ``setThreads`` is accepted and ignored, the device is the parallelism;
* ``RigidWall`` and ``Contact`` are configurations until they are handed to a solver, after
  which their statistics are read from it.

``IllegalArgumentException`` surfaces as ``ValueError`` and ``IllegalStateException`` as
``RuntimeError``, with the reference's messages.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional, Sequence, Union

import numpy as np

from . import _abi
from .materials import Formulation, Integration, Kinematics, Material, Materials
from .mesh import QuadMesh


class DeviceError(RuntimeError):
    pass


class DeviceTimeout(DeviceError):
    """A bounded device-side wait gave up (NF_ETIMEOUT); the handle can no longer step."""


def _raise(api, handle, status: int):
    msg = api.last_error(handle)
    msg = msg.decode() if msg else f"status {status}"
    if status == _abi.NF_EINVAL:
        raise ValueError(msg)
    if status == _abi.NF_ESTATE:
        raise RuntimeError(msg)
    if status == _abi.NF_ETIMEOUT:
        raise DeviceTimeout(msg)
    raise DeviceError(msg)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_abi.c_double_p)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(_abi.c_int32_p)


class RigidWall:
    """RigidWall.atZ(z[, friction]) (RigidWall.java:110-136); statistics :285-315."""

    def __init__(self, plane: float, friction: float):
        if friction < 0.0 or math.isnan(friction):
            raise ValueError("friction coefficient must be >= 0")
        self._plane = float(plane)
        self._friction = float(friction)
        self._solver = None

    @staticmethod
    def atZ(z: float, friction: float = 0.0) -> "RigidWall":
        return RigidWall(z, friction)

    def plane(self) -> float:
        return self._plane

    def friction(self) -> float:
        return self._friction

    def _stats(self) -> _abi.WallInfo:
        if self._solver is None:
            return _abi.WallInfo()
        return self._solver._wallInfo()

    def impulse(self) -> float:
        return self._stats().impulse

    def energyLoss(self) -> float:
        return self._stats().energy_loss

    def frictionDissipation(self) -> float:
        return self._stats().friction_dissipation

    def contactCount(self) -> int:
        return self._stats().contact_count

    def stuckCount(self) -> int:
        return self._stats().stuck_count


class Contact:
    """new Contact(mesh).withFriction(mu).withDamping(zeta).withStiffnessScale(s)
    (Contact.java:273-364); statistics :366-404."""

    DEFAULT_SCALE = 0.1
    DEFAULT_DAMPING = 0.0

    def __init__(self, mesh: QuadMesh):
        self.mesh = mesh
        self._friction = 0.0
        self._scale = Contact.DEFAULT_SCALE
        self._damping = Contact.DEFAULT_DAMPING
        self._solver = None

    def withFriction(self, mu: float) -> "Contact":
        if mu < 0.0:
            raise ValueError("friction must not be negative")
        self._friction = float(mu)
        self._push()
        return self

    def withDamping(self, zeta: float) -> "Contact":
        if zeta < 0.0 or zeta > 1.0:
            raise ValueError("contact damping is a fraction of critical, so it lies in [0, 1]; "
                             f"was {zeta}")
        self._damping = float(zeta)
        self._push()
        return self

    def withStiffnessScale(self, s: float) -> "Contact":
        if not (s > 0.0) or s >= 2.0:
            raise ValueError("the stiffness scale must lie in (0, 2); a pair is found from both "
                             "sides, so the effective stiffness is twice this and above 2 the "
                             f"contact frequency exceeds what central difference can integrate, "
                             f"was {s}")
        self._scale = float(s)
        self._push()
        return self

    def _push(self):
        if self._solver is not None:
            self._solver._pushContact(self)

    def friction(self) -> float:
        return self._friction

    def _stats(self) -> _abi.ContactInfo:
        if self._solver is None:
            return _abi.ContactInfo()
        return self._solver._contactInfo()

    def pairCount(self) -> int:
        return self._stats().pair_count

    def energy(self) -> float:
        return self._stats().energy

    def dissipation(self) -> float:
        return self._stats().dissipation

    def maxPenetration(self) -> float:
        return self._stats().max_penetration

    def escapedNodes(self) -> int:
        return self._stats().escaped_nodes

    def segmentCount(self) -> int:
        return self._stats().segment_count


class DamageView:
    """Read-only view of the damage state (Damage.java:268-412)."""

    def __init__(self, solver: "ExplicitSolver"):
        self._s = solver

    def _f(self, field):
        return self._s.readField(field)

    def points(self) -> int:
        return self._s._points

    def hasBegun(self, point: int) -> bool:
        return bool(self._f(_abi.FIELD_DAMAGE_STRENGTH)[point] > 0.0)

    def bandWidth(self, point: int) -> float:
        return float(self._f(_abi.FIELD_DAMAGE_WIDTH)[point])

    def strengthAtOnset(self, point: int) -> float:
        return float(self._f(_abi.FIELD_DAMAGE_STRENGTH)[point])

    def softeningModulus(self, point: int) -> float:
        return float(self._f(_abi.FIELD_DAMAGE_SOFTENING)[point])

    def clampedPoints(self) -> int:
        return int(self._s._auditC().clamped_points)

    def at(self, point: int, plasticStrain: float) -> float:
        sf = self.strengthAtOnset(point)
        if sf <= 0.0:
            return 0.0
        d = -self.softeningModulus(point) * (plasticStrain - self._s._failureStrainOf(point)) / sf
        return 0.0 if d <= 0.0 else (1.0 if d >= 1.0 else d)

    def dissipation(self, point: int, plasticStrain: float) -> float:
        sf = self.strengthAtOnset(point)
        if sf <= 0.0:
            return 0.0
        slope = self.softeningModulus(point)
        full = -sf / slope
        excess = plasticStrain - self._s._failureStrainOf(point)
        if excess <= 0.0:
            return 0.0
        excess = min(excess, full)
        return excess * (sf + 0.5 * slope * excess)

    @staticmethod
    def largestRegularisableElement(fractureEnergy, youngsModulus, flowStress):
        return 2.0 * youngsModulus * fractureEnergy / (flowStress * flowStress)

    @staticmethod
    def softeningRange(fractureEnergy, flowStress, width):
        return 2.0 * fractureEnergy / (flowStress * width)


class ExplicitSolver:
    """ExplicitSolver (solver/ExplicitSolver.java), state resident on the GPU.

    Constructor forms, as in the reference (:237-264):
      ExplicitSolver(mesh, material, formulation, thickness, cfl)               full, small strain
      ExplicitSolver(mesh, material, formulation, integration, thickness, cfl)  small strain
      ExplicitSolver(mesh, materials, formulation, integration, kinematics, thickness, cfl)
    """

    @classmethod
    def _binding(cls):
        from . import _native
        return _native.api()

    def __init__(self, mesh: QuadMesh, material: Union[Material, Materials],
                 formulation: Formulation, *args):
        if len(args) == 2:
            integration, kinematics = Integration.FULL, Kinematics.SMALL_STRAIN
            thickness, cfl = args
        elif len(args) == 3:
            integration, thickness, cfl = args
            kinematics = Kinematics.SMALL_STRAIN
        elif len(args) == 4:
            integration, kinematics, thickness, cfl = args
        else:
            raise TypeError("ExplicitSolver(mesh, material, formulation, [integration, "
                            "[kinematics,]] thickness, cflSafety)")
        self._api = self._binding()
        self._handle = None
        materials = material if isinstance(material, Materials) else Materials.uniform(material)
        materials.requireCovers(mesh.elementCount)
        self.mesh = mesh
        self.materials = materials
        self._formulation = Formulation(formulation)
        self._integration = Integration(integration)
        self._kinematics = Kinematics(kinematics)
        self._ppe = self._integration.gaussPoints()
        self._points = mesh.elementCount * self._ppe
        mats, index = materials.table(mesh.elementCount)
        self._matList = mats
        self._matIndex = index
        table = (_abi.MaterialC * len(mats))(*[_abi.material_struct(m) for m in mats])
        cm = _abi.Mesh()
        cm.node_count = mesh.nodeCount
        cm.element_count = mesh.elementCount
        cm.pressure_edge_count = mesh.pressureEdges.size // 2
        cm.r = _dptr(mesh.r)
        cm.z = _dptr(mesh.z)
        cm.conn = _iptr(mesh.conn)
        cm.pressure_edges = _iptr(mesh.pressureEdges) if mesh.pressureEdges.size else None
        out = C.c_void_p()
        st = self._api.create(C.byref(cm), table, len(mats), _iptr(index),
                              int(self._formulation), int(self._integration),
                              int(self._kinematics), float(thickness), float(cfl), C.byref(out))
        if st:
            _raise(self._api, None, st)
        self._handle = out
        self._wall: Optional[RigidWall] = None
        self._contact: Optional[Contact] = None
        self._damage = None
        self._failure = None
        self._hourglass = 0.05
        self._threads = 1

    # ------------------------------------------------------------------ plumbing
    def _call(self, fn, *args):
        st = fn(self._handle, *args)
        if st:
            _raise(self._api, self._handle, st)

    def close(self):
        if self._handle is not None:
            self._api.destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def readField(self, field: int) -> np.ndarray:
        count, eb = C.c_size_t(), C.c_size_t()
        self._call(self._api.field_size, field, C.byref(count), C.byref(eb))
        dtype = {8: np.float64, 4: np.int32, 1: np.uint8}[eb.value]
        out = np.empty(count.value, dtype=dtype)
        self._call(self._api.read_field, field, out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out

    def writeField(self, field: int, values) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._call(self._api.write_field, field, a.ctypes.data_as(C.c_void_p), a.nbytes)

    def _state(self) -> _abi.State:
        s = _abi.State()
        self._call(self._api.get_state, C.byref(s))
        return s

    def _auditC(self) -> _abi.Audit:
        a = _abi.Audit()
        self._call(self._api.audits, C.byref(a))
        return a

    def _wallInfo(self) -> _abi.WallInfo:
        w = _abi.WallInfo()
        self._call(self._api.wall_stats, C.byref(w))
        return w

    def _contactInfo(self) -> _abi.ContactInfo:
        c = _abi.ContactInfo()
        self._call(self._api.contact_stats, C.byref(c))
        return c

    def statusWord(self) -> int:
        w = C.c_uint32()
        self._call(self._api.status_word, C.byref(w))
        return w.value

    def synchronize(self):
        self._call(self._api.synchronize)

    def check(self) -> None:
        """Waits for the queued steps and raises if the device flagged a fault: DeviceTimeout
        when a contact-pass barrier gave up, DeviceError when a nodal velocity or displacement
        stopped being finite (the reference lets NaNs propagate silently)."""
        self._call(self._api.check)

    def setWaitLimit(self, polls: int, nanoseconds: int) -> None:
        """Bounds of each contact-pass barrier wait (0, 0: the defaults); for tests."""
        self._call(self._api.set_wait_limit, int(polls), int(nanoseconds))

    def setGridSlots(self, slots: int) -> None:
        """Slots per cell of the contact pass's direct-indexed grid, 0..64 (default 64); a step
        whose busiest cell holds more takes the counting sort, and 0 sends every step there.
        Both give the same bits; for tests and tuning."""
        self._call(self._api.set_grid_slots, int(slots))

    def setStream(self, stream_handle: int) -> None:
        """Runs this solver's kernels on a caller-owned cudaStream_t (0: its own)."""
        self._call(self._api.set_stream, C.c_void_p(stream_handle or None))

    def setPrecision(self, precision: int) -> None:
        """PRECISION_FP64 (the reference's arithmetic) or PRECISION_MIXED (FP32 element
        arithmetic and state, FP64 kinematics and audits)."""
        self._call(self._api.set_precision, int(precision))

    def profile(self, enable: bool) -> None:
        self._call(self._api.profile, 1 if enable else 0)

    def profileRead(self):
        """(milliseconds per kernel group, steps covered) since profiling was enabled."""
        ms = (C.c_double * 7)()
        steps = C.c_int64()
        self._call(self._api.profile_read, ms, C.byref(steps))
        return dict(zip(_abi.GROUP_NAMES, list(ms))), steps.value

    def launchCount(self) -> int:
        n = C.c_int64()
        self._call(self._api.launch_count, C.byref(n))
        return n.value

    # ------------------------------------------------------------------ setup (:386-808)
    def setThreads(self, n: int) -> None:
        if n < 1:
            raise ValueError("need at least one thread")
        self._threads = n
        self._call(self._api.set_threads, n)

    def threads(self) -> int:
        return self._threads

    def shutdown(self) -> None:
        pass

    def fixRadial(self, node: int) -> None:
        self._call(self._api.fix_radial, int(node))

    def fixAxial(self, node: int) -> None:
        self._call(self._api.fix_axial, int(node))

    def fixAllAxial(self) -> None:
        self._call(self._api.fix_all_axial)

    def setPressureRamp(self, pascals: float, rampSeconds: float) -> None:
        self._call(self._api.set_pressure_ramp, float(pascals), float(rampSeconds))

    def setRelaxationDamping(self, fractionOfCritical: float, angularFrequency: float) -> None:
        self._call(self._api.set_relaxation_damping, float(fractionOfCritical),
                   float(angularFrequency))

    def setHourglassCoefficient(self, q: float) -> None:
        self._call(self._api.set_hourglass_coefficient, float(q))
        self._hourglass = float(q)

    def setRigidWall(self, wall: Optional[RigidWall]) -> None:
        if wall is None:
            self._call(self._api.clear_rigid_wall)
        else:
            self._call(self._api.set_rigid_wall, wall.plane(), wall.friction())
            wall._solver = self
        self._wall = wall

    def setContact(self, contact: Optional[Contact]) -> None:
        if contact is None:
            self._call(self._api.clear_contact)
        else:
            contact._solver = self
            self._pushContact(contact)
        self._contact = contact

    def _pushContact(self, c: Contact):
        self._call(self._api.set_contact, c._friction, c._damping, c._scale)

    def contact(self) -> Optional[Contact]:
        return self._contact

    def setGravity(self, accelerationR: float, accelerationZ: float) -> None:
        self._call(self._api.set_gravity, float(accelerationR), float(accelerationZ))

    def setErosion(self, damageThreshold: float) -> None:
        self._call(self._api.set_erosion, float(damageThreshold))

    def setMassScaling(self, targetStep: float) -> None:
        self._call(self._api.set_mass_scaling, float(targetStep))

    def massScale(self) -> float:
        return self._state().mass_scale

    def setDamage(self, fractureEnergy, failureStrain) -> None:
        E = self.mesh.elementCount
        eps = np.ascontiguousarray(failureStrain, dtype=np.float64)
        if np.ndim(fractureEnergy) == 0:
            gf = np.full(E, float(fractureEnergy))
        else:
            gf = np.ascontiguousarray(fractureEnergy, dtype=np.float64)
            if gf.size != E:
                raise ValueError(f"fracture energy has {gf.size} entries for a mesh of {E} elements")
        if eps.size != E:
            raise ValueError(f"failure strain has {eps.size} entries for a mesh of {E} elements")
        self._call(self._api.set_damage, _dptr(gf), _dptr(eps))
        self._failure = np.repeat(eps, self._ppe)
        self._damage = DamageView(self)

    def damage(self):
        return self._damage

    def _failureStrainOf(self, point: int) -> float:
        return float(self._failure[point])

    def setVelocity(self, node: int, velocityR: float, velocityZ: float) -> None:
        self._call(self._api.set_velocity, int(node), float(velocityR), float(velocityZ))

    def setUniformVelocity(self, velocityR: float, velocityZ: float) -> None:
        self._call(self._api.set_uniform_velocity, float(velocityR), float(velocityZ))

    def setVelocities(self, vr, vz) -> None:
        a = np.ascontiguousarray(vr, dtype=np.float64)
        b = np.ascontiguousarray(vz, dtype=np.float64)
        self._call(self._api.set_velocities, _dptr(a), _dptr(b))

    # ------------------------------------------------------------------ queries
    def integration(self) -> Integration:
        return self._integration

    def kinematics(self) -> Kinematics:
        return self._kinematics

    def formulation(self) -> Formulation:
        return self._formulation

    def borePressure(self) -> float:
        return self._state().bore_pressure

    def timestep(self) -> float:
        return self._state().timestep

    def time(self) -> float:
        return self._state().time

    def steps(self) -> int:
        return int(self._state().steps)

    def isEroded(self, element: int) -> bool:
        g = self.readField(_abi.FIELD_ERODED)
        return bool(g.size and g[element])

    def erodedElements(self) -> int:
        return self._state().eroded_elements

    def erodedEnergy(self) -> float:
        return self._state().eroded_energy

    def invertedElements(self) -> int:
        return self._state().inverted_elements

    def radialDisplacement(self) -> np.ndarray:
        return self.readField(_abi.FIELD_UR)

    def axialDisplacement(self) -> np.ndarray:
        return self.readField(_abi.FIELD_UZ)

    def velocityR(self) -> np.ndarray:
        return self.readField(_abi.FIELD_VR)

    def velocityZ(self) -> np.ndarray:
        return self.readField(_abi.FIELD_VZ)

    def forceR(self) -> np.ndarray:
        return self.readField(_abi.FIELD_FR)

    def forceZ(self) -> np.ndarray:
        return self.readField(_abi.FIELD_FZ)

    def plasticStrain(self) -> np.ndarray:
        return self.readField(_abi.FIELD_PLASTIC_STRAIN)

    def stress(self) -> np.ndarray:
        return self.readField(_abi.FIELD_STRESS)

    def plasticWorkDensity(self) -> np.ndarray:
        return self.readField(_abi.FIELD_PLASTIC_WORK)

    def elementSpeed(self, element: int) -> float:
        vr, vz = self.velocityR(), self.velocityZ()
        s = 0.0
        for k in range(4):
            n = self.mesh.conn[element * 4 + k]
            s += math.sqrt(vr[n] * vr[n] + vz[n] * vz[n])
        return 0.25 * s

    # ------------------------------------------------------------------ run (:936-1075)
    def run(self, steps: int) -> None:
        self._call(self._api.step, int(steps))

    def step(self) -> None:
        self._call(self._api.step, 1)

    def advance(self) -> None:
        self._call(self._api.advance)

    def runUntil(self, tEnd: float, maxSteps: int = 1 << 40) -> int:
        taken = C.c_int64()
        self._call(self._api.run_until, float(tEnd), int(maxSteps), C.byref(taken))
        return taken.value

    # ------------------------------------------------------------------ audits (:875, :1610-1936)
    def centredKineticEnergy(self) -> float:
        return self._auditC().centred_kinetic_energy

    def axialMomentum(self) -> float:
        return self._auditC().axial_momentum

    def radialMomentum(self) -> float:
        return self._auditC().radial_momentum

    def kineticEnergy(self) -> float:
        return self._auditC().kinetic_energy

    def strainEnergy(self) -> float:
        return self._auditC().strain_energy

    def plasticDissipation(self) -> float:
        return self._auditC().plastic_dissipation

    def fractureDissipation(self) -> float:
        return self._auditC().fracture_dissipation

    def maxDamage(self) -> float:
        return self._auditC().max_damage

    def damagedFraction(self) -> float:
        return self._auditC().damaged_fraction

    def failedFraction(self) -> float:
        return self._auditC().failed_fraction

    def mostDamagedElement(self) -> int:
        return self._auditC().most_damaged_element

    def hourglassEnergy(self) -> float:
        return self._auditC().hourglass_energy

    def maxPlasticStrain(self) -> float:
        return self._auditC().max_plastic_strain

    def yieldedFraction(self) -> float:
        return self._auditC().yielded_fraction

    def maxTemperature(self) -> float:
        t = self._auditC().max_temperature
        if math.isnan(t):
            raise RuntimeError("this material has no thermal model; temperature is not defined")
        return t

    def temperature(self, point: int) -> float:
        m = self.materials.at(point // self._ppe)
        if m.johnsonCook is None:
            raise RuntimeError("this material has no thermal model; temperature is not defined")
        return m.johnsonCook.temperature(float(self.plasticWorkDensity()[point]), m.density)

    def elementDamage(self, element: int) -> float:
        if self._damage is None:
            return 0.0
        eps = self.plasticStrain()
        s = 0.0
        for g in range(self._ppe):
            p = element * self._ppe + g
            s += self._damage.at(p, float(eps[p]))
        return s / self._ppe

    def centroidStress(self, element: int) -> np.ndarray:
        sig = self.stress().reshape(-1, 4)
        out = np.zeros(4)
        for g in range(self._ppe):
            out = out + sig[element * self._ppe + g]
        return out / self._ppe

    def elementPlasticStrain(self, element: int) -> float:
        eps = self.plasticStrain()
        s = 0.0
        for g in range(self._ppe):
            s += float(eps[element * self._ppe + g])
        return s / self._ppe

    def plasticFrontRadius(self) -> float:
        eps = self.plasticStrain().reshape(-1, self._ppe)
        c = self.mesh.conn.reshape(-1, 4)
        outer = self.mesh.r[c].max(axis=1)
        yielded = (eps > 0.0).any(axis=1)
        return float(outer[yielded].max()) if yielded.any() else 0.0

    def centroidRadius(self, element: int) -> float:
        b = element * 4
        r = self.mesh.r
        c = self.mesh.conn
        return 0.25 * (r[c[b]] + r[c[b + 1]] + r[c[b + 2]] + r[c[b + 3]])

    def centroidZ(self, element: int) -> float:
        uz = self.axialDisplacement()
        s = 0.0
        for k in range(4):
            n = self.mesh.conn[element * 4 + k]
            s += self.mesh.z[n] + uz[n]
        return 0.25 * s

    def meshZ(self, node: int) -> float:
        return float(self.mesh.z[node])

    def measure(self) -> _abi.Measure:
        m = _abi.Measure()
        self._call(self._api.measure_body, C.byref(m))
        return m


def material_point_update(material: Material, sig, back, epsP, work, strain, strainDt,
                          damage=None, formulation=Formulation.PLANE_STRAIN, binding=None):
    """J2.update over arrays of points (J2.java:163-296) on the device. Arrays are float64,
    updated in place; returns the plastic multipliers."""
    api = binding if binding is not None else ExplicitSolver._binding()
    n = int(np.asarray(epsP).size)
    dg = np.zeros(n)
    d = None
    if damage is not None:
        d = _abi.DamagePoints()
        for name in ("failure_strain", "fracture_energy", "youngs_modulus", "geometry",
                     "strength", "softening", "width"):
            setattr(d, name, _dptr(damage[name]))
    st = api.material_point_update(C.byref(_abi.material_struct(material)), int(formulation), n,
                                   _dptr(sig), _dptr(back), _dptr(epsP), _dptr(work),
                                   _dptr(np.ascontiguousarray(strain, dtype=np.float64)),
                                   float(strainDt), C.byref(d) if d is not None else None,
                                   _dptr(dg))
    if st:
        _raise(api, None, st)
    return dg
