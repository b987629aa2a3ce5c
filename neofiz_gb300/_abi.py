"""ctypes description of the C ABI in include/neofiz.h.

Every library that implements the ABI is bound through ``bind(lib, prefix)``, which declares
argument and return types for each entry point and returns a namespace whose attributes are
the entry points without their prefix (``api.create``, ``api.step`` ...).
"""
from __future__ import annotations

import ctypes as C
import types

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)

NF_OK, NF_EINVAL, NF_ESTATE, NF_EDEVICE, NF_ETIMEOUT, NF_ENOMEM = range(6)
# bits of the device status word (nf_status_word)
STATUS_NONFINITE, STATUS_BUCKET_OVERFLOW, STATUS_TIMEOUT = 1, 4, 8

(FIELD_UR, FIELD_UZ, FIELD_VR, FIELD_VZ, FIELD_FR, FIELD_FZ, FIELD_MASS, FIELD_STRESS,
 FIELD_BACK_STRESS, FIELD_PLASTIC_STRAIN, FIELD_PLASTIC_WORK, FIELD_HOURGLASS_R,
 FIELD_HOURGLASS_Z, FIELD_HOURGLASS_STIFFNESS, FIELD_DAMAGE_STRENGTH, FIELD_DAMAGE_SOFTENING,
 FIELD_DAMAGE_WIDTH, FIELD_ERODED, FIELD_ON_WALL, FIELD_WALL_STATE, FIELD_CONTACT_MASTER,
 FIELD_CONTACT_STATE, FIELD_SURFACE_EDGES, FIELD_SURFACE_NODES, FIELD_FIXED) = range(25)

(GROUP_NODAL, GROUP_ERODE, GROUP_ELEMENT, GROUP_PRESSURE, GROUP_GATHER, GROUP_CONTACT,
 GROUP_END) = range(7)
GROUP_NAMES = ("nodal", "erode", "element", "pressure", "gather", "contact", "end")

PRECISION_FP64, PRECISION_MIXED, PRECISION_COMPENSATED = 0, 1, 2

OBJECTIVE_LENGTH_RATIO, OBJECTIVE_MUSHROOM, OBJECTIVE_PEAK_CAPACITY = 0, 1, 2
(PARAM_A, PARAM_B, PARAM_N, PARAM_C, PARAM_M, PARAM_KINEMATIC, PARAM_FRICTION,
 PARAM_FRACTURE_ENERGY, PARAM_YIELD, PARAM_ISOTROPIC) = range(10)
PARAM_COUNT = 10
PARAM_NAMES = ("A", "B", "n", "C", "m", "kinematic", "friction", "fracture_energy", "yield",
               "isotropic")

WALL_HELD, WALL_STUCK, WALL_SLID, WALL_ARRIVED = 1, 2, 4, 8
CONTACT_PAIR, CONTACT_STICK, CONTACT_SLIP = 1, 2, 4


class Mesh(C.Structure):
    _fields_ = [("node_count", C.c_int32), ("element_count", C.c_int32),
                ("pressure_edge_count", C.c_int32),
                ("r", c_double_p), ("z", c_double_p),
                ("conn", c_int32_p), ("pressure_edges", c_int32_p)]


class MaterialC(C.Structure):
    _fields_ = [("youngs_modulus", C.c_double), ("poisson_ratio", C.c_double),
                ("density", C.c_double), ("yield_stress", C.c_double),
                ("isotropic_hardening", C.c_double), ("kinematic_hardening", C.c_double),
                ("has_johnson_cook", C.c_int32), ("reserved", C.c_int32),
                ("jc_a", C.c_double), ("jc_b", C.c_double), ("jc_n", C.c_double),
                ("jc_c", C.c_double), ("jc_m", C.c_double),
                ("jc_reference_strain_rate", C.c_double),
                ("jc_room_temperature", C.c_double), ("jc_melt_temperature", C.c_double),
                ("jc_specific_heat", C.c_double), ("jc_taylor_quinney", C.c_double)]


class State(C.Structure):
    _fields_ = [("time", C.c_double), ("timestep", C.c_double),
                ("timestep_previous", C.c_double), ("reference_timestep", C.c_double),
                ("mass_scale", C.c_double), ("min_edge_squared", C.c_double),
                ("fastest_wave", C.c_double), ("eroded_energy", C.c_double),
                ("bore_pressure", C.c_double), ("steps", C.c_int64),
                ("eroded_elements", C.c_int32), ("inverted_elements", C.c_int32),
                ("node_count", C.c_int32), ("element_count", C.c_int32),
                ("points_per_element", C.c_int32), ("pressure_edge_count", C.c_int32)]


class Audit(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "kinetic_energy", "centred_kinetic_energy", "strain_energy", "plastic_dissipation",
        "hourglass_energy", "fracture_dissipation", "axial_momentum", "radial_momentum",
        "max_plastic_strain", "yielded_fraction", "max_damage", "damaged_fraction",
        "failed_fraction", "max_temperature")] + [
        ("clamped_points", C.c_int32), ("most_damaged_element", C.c_int32)]


class WallInfo(C.Structure):
    _fields_ = [("plane", C.c_double), ("friction", C.c_double), ("impulse", C.c_double),
                ("energy_loss", C.c_double), ("friction_dissipation", C.c_double),
                ("contact_count", C.c_int32), ("stuck_count", C.c_int32),
                ("present", C.c_int32), ("reserved", C.c_int32)]


class ContactInfo(C.Structure):
    _fields_ = [("friction", C.c_double), ("energy", C.c_double),
                ("dissipation", C.c_double), ("max_penetration", C.c_double),
                ("pair_count", C.c_int32), ("escaped_nodes", C.c_int32),
                ("segment_count", C.c_int32), ("present", C.c_int32)]


class Measure(C.Structure):
    _fields_ = [("z_max", C.c_double), ("z_min", C.c_double), ("length", C.c_double),
                ("mushroom_diameter", C.c_double)]


class DamagePoints(C.Structure):
    _fields_ = [("failure_strain", c_double_p), ("fracture_energy", c_double_p),
                ("youngs_modulus", c_double_p), ("geometry", c_double_p),
                ("strength", c_double_p), ("softening", c_double_p), ("width", c_double_p)]


class BatchMesh(C.Structure):
    _fields_ = [("instance_count", C.c_int32), ("node_offset", c_int32_p),
                ("element_offset", c_int32_p), ("r", c_double_p), ("z", c_double_p),
                ("conn", c_int32_p), ("fixed", C.POINTER(C.c_uint8)),
                ("pressure_offset", c_int32_p), ("pressure_edges", c_int32_p),
                ("failure_strain", c_double_p), ("fracture_energy", c_double_p)]


class BatchInstance(C.Structure):
    _fields_ = [("material", MaterialC), ("velocity_r", C.c_double), ("velocity_z", C.c_double),
                ("wall_plane", C.c_double), ("wall_friction", C.c_double),
                ("hourglass", C.c_double), ("t_end", C.c_double),
                ("pressure", C.c_double), ("pressure_ramp", C.c_double),
                ("damping_fraction", C.c_double), ("damping_omega", C.c_double)]


class BatchConfig(C.Structure):
    _fields_ = [("threads", C.c_int32), ("stage_nodes", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("chunk_steps", C.c_int32)]


class BatchProgress(C.Structure):
    _fields_ = [("time", C.c_double), ("timestep", C.c_double), ("steps", C.c_int64),
                ("status", C.c_uint32), ("done", C.c_int32)]


_H = C.c_void_p
_S = C.c_int
_PROTOS = {
    "create": (_S, [C.POINTER(Mesh), C.POINTER(MaterialC), C.c_int32, c_int32_p, C.c_int32,
                    C.c_int32, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_void_p)]),
    "destroy": (None, [_H]),
    "last_error": (C.c_char_p, [_H]),
    "status_word": (_S, [_H, C.POINTER(C.c_uint32)]),
    "check": (_S, [_H]),
    "set_wait_limit": (_S, [_H, C.c_int64, C.c_int64]),
    "set_grid_slots": (_S, [_H, C.c_int32]),
    "set_threads": (_S, [_H, C.c_int32]),
    "fix_radial": (_S, [_H, C.c_int32]),
    "fix_axial": (_S, [_H, C.c_int32]),
    "fix_all_axial": (_S, [_H]),
    "set_pressure_ramp": (_S, [_H, C.c_double, C.c_double]),
    "set_relaxation_damping": (_S, [_H, C.c_double, C.c_double]),
    "set_hourglass_coefficient": (_S, [_H, C.c_double]),
    "set_rigid_wall": (_S, [_H, C.c_double, C.c_double]),
    "clear_rigid_wall": (_S, [_H]),
    "set_contact": (_S, [_H, C.c_double, C.c_double, C.c_double]),
    "clear_contact": (_S, [_H]),
    "set_gravity": (_S, [_H, C.c_double, C.c_double]),
    "set_erosion": (_S, [_H, C.c_double]),
    "set_mass_scaling": (_S, [_H, C.c_double]),
    "set_damage": (_S, [_H, c_double_p, c_double_p]),
    "set_velocity": (_S, [_H, C.c_int32, C.c_double, C.c_double]),
    "set_uniform_velocity": (_S, [_H, C.c_double, C.c_double]),
    "set_velocities": (_S, [_H, c_double_p, c_double_p]),
    "step": (_S, [_H, C.c_int64]),
    "advance": (_S, [_H]),
    "run_until": (_S, [_H, C.c_double, C.c_int64, C.POINTER(C.c_int64)]),
    "synchronize": (_S, [_H]),
    "set_stream": (_S, [_H, C.c_void_p]),
    "set_precision": (_S, [_H, C.c_int32]),
    "profile": (_S, [_H, C.c_int32]),
    "profile_read": (_S, [_H, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "launch_count": (_S, [_H, C.POINTER(C.c_int64)]),
    "field_size": (_S, [_H, C.c_int32, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "read_field": (_S, [_H, C.c_int32, C.c_void_p, C.c_size_t]),
    "write_field": (_S, [_H, C.c_int32, C.c_void_p, C.c_size_t]),
    "get_state": (_S, [_H, C.POINTER(State)]),
    "audits": (_S, [_H, C.POINTER(Audit)]),
    "wall_stats": (_S, [_H, C.POINTER(WallInfo)]),
    "contact_stats": (_S, [_H, C.POINTER(ContactInfo)]),
    "measure_body": (_S, [_H, C.POINTER(Measure)]),
    "material_point_update": (_S, [C.POINTER(MaterialC), C.c_int32, C.c_int32, c_double_p,
                                   c_double_p, c_double_p, c_double_p, c_double_p, C.c_double,
                                   C.POINTER(DamagePoints), c_double_p]),
    "batch_create": (_S, [C.POINTER(BatchMesh), C.POINTER(BatchInstance), C.c_int32, C.c_int32,
                          C.c_double, C.c_double, C.c_int32, C.POINTER(C.c_void_p)]),
    "batch_destroy": (_S, [_H]),
    "batch_last_error": (C.c_char_p, [_H]),
    "batch_tune": (_S, [_H, C.c_int32, C.POINTER(BatchConfig)]),
    "batch_set_config": (_S, [_H, C.POINTER(BatchConfig)]),
    "batch_get_config": (_S, [_H, C.POINTER(BatchConfig)]),
    "batch_run": (_S, [_H, C.c_int64]),
    "batch_elapsed": (_S, [_H, C.POINTER(C.c_double)]),
    "batch_launch_count": (_S, [_H, C.POINTER(C.c_int64)]),
    "batch_field_size": (_S, [_H, C.c_int32, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "batch_read": (_S, [_H, C.c_int32, C.c_void_p, C.c_size_t]),
    "batch_state": (_S, [_H, C.POINTER(BatchProgress)]),
    "batch_measure": (_S, [_H, C.POINTER(Measure)]),
    "batch_wall_stats": (_S, [_H, C.POINTER(WallInfo)]),
    "batch_adjoint_forward": (_S, [_H, C.c_int32, C.c_int32]),
    "batch_adjoint_backward": (_S, [_H, C.c_int32, c_double_p, c_double_p]),
    "batch_adjoint_backward_many": (_S, [_H, c_int32_p, C.c_int32, c_double_p, c_double_p]),
    "batch_set_burst": (_S, [_H, C.c_void_p, c_double_p]),
    "batch_burst_results": (_S, [_H, C.c_void_p]),
    "batch_burst_trace": (_S, [_H, c_double_p]),
    "batch_adjoint_elapsed": (_S, [_H, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}

ENTRY_POINTS = tuple("nf_" + name for name in _PROTOS)


class BatchBurst(C.Structure):
    _fields_ = [("sample_every", C.c_int32), ("trace_capacity", C.c_int32),
                ("margin", C.c_double)]


class BurstResult(C.Structure):
    _fields_ = [("peak_capacity", C.c_double), ("peak_strain", C.c_double),
                ("peak_applied", C.c_double), ("capacity", C.c_double),
                ("strain", C.c_double), ("applied", C.c_double), ("samples", C.c_int32),
                ("traversed", C.c_int32)]


class FilmInfo(C.Structure):
    _fields_ = [("time", C.c_double), ("steps", C.c_int64), ("eroded", C.c_int32),
                ("contact_pairs", C.c_int32), ("pressure", C.c_double)]


(FILM_PLASTIC_STRAIN, FILM_DAMAGE, FILM_VON_MISES_MPA, FILM_HOOP_STRESS_MPA,
 FILM_SPEED) = range(5)

# The device film (GPU library only: the oracle has no device to capture from).
_FILM_PROTOS = {
    "film_create": (_S, [_H, c_int32_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "film_destroy": (_S, [_H]),
    "film_capture": (_S, [_H]),
    "film_frames": (_S, [_H, c_int32_p]),
    "film_read": (_S, [_H, c_double_p, c_double_p, c_double_p, C.POINTER(C.c_uint8),
                       C.POINTER(FilmInfo), C.POINTER(Audit)]),
    "film_clear": (_S, [_H]),
    "film_last_error": (C.c_char_p, [_H]),
}


def bind(lib: C.CDLL, prefix: str) -> types.SimpleNamespace:
    ns = types.SimpleNamespace()
    protos = dict(_PROTOS)
    if prefix == "nf_":
        protos.update(_FILM_PROTOS)
    for name, (res, args) in protos.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
        setattr(ns, name, fn)
    ns.lib = lib
    ns.prefix = prefix
    return ns


def material_struct(m) -> MaterialC:
    """Fills the C record from a neofiz_gb300.materials.Material."""
    s = MaterialC()
    s.youngs_modulus = m.youngsModulus
    s.poisson_ratio = m.poissonRatio
    s.density = m.density
    s.yield_stress = m.yieldStress
    s.isotropic_hardening = m.isotropicHardening
    s.kinematic_hardening = m.kinematicHardening
    jc = m.johnsonCook
    s.has_johnson_cook = 1 if jc is not None else 0
    if jc is not None:
        s.jc_a, s.jc_b, s.jc_n, s.jc_c, s.jc_m = jc.a, jc.b, jc.n, jc.c, jc.m
        s.jc_reference_strain_rate = jc.referenceStrainRate
        s.jc_room_temperature = jc.roomTemperature
        s.jc_melt_temperature = jc.meltTemperature
        s.jc_specific_heat = jc.specificHeat
        s.jc_taylor_quinney = jc.taylorQuinney
    return s
