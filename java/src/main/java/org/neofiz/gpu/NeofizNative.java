package org.neofiz.gpu;

import java.lang.foreign.Arena;
import java.lang.foreign.FunctionDescriptor;
import java.lang.foreign.Linker;
import java.lang.foreign.MemoryLayout;
import java.lang.foreign.MemorySegment;
import java.lang.foreign.StructLayout;
import java.lang.foreign.SymbolLookup;
import java.lang.invoke.MethodHandle;

import static java.lang.foreign.MemoryLayout.PathElement.groupElement;
import static java.lang.foreign.ValueLayout.ADDRESS;
import static java.lang.foreign.ValueLayout.JAVA_DOUBLE;
import static java.lang.foreign.ValueLayout.JAVA_INT;
import static java.lang.foreign.ValueLayout.JAVA_LONG;

/**
 * The C ABI of libneofiz_gpu.so (include/neofiz.h) bound through java.lang.foreign: the
 * struct layouts, one downcall handle per entry point, and the mapping of nf_status codes to
 * the exceptions the reference's ExplicitSolver throws.
 *
 * <p>Written against the final foreign-function API (JDK 22 and later). The library is looked
 * up as {@code libneofiz_gpu.so} on the library path, or at the path given by the system
 * property {@code neofiz.gpu.lib}.
 */
final class NeofizNative {
    private NeofizNative() {}

    static final int NF_OK = 0, NF_EINVAL = 1, NF_ESTATE = 2, NF_EDEVICE = 3, NF_ETIMEOUT = 4,
            NF_ENOMEM = 5;

    // nf_field
    static final int FIELD_UR = 0, FIELD_UZ = 1, FIELD_VR = 2, FIELD_VZ = 3, FIELD_FR = 4,
            FIELD_FZ = 5, FIELD_MASS = 6, FIELD_STRESS = 7, FIELD_BACK_STRESS = 8,
            FIELD_PLASTIC_STRAIN = 9, FIELD_PLASTIC_WORK = 10, FIELD_HOURGLASS_R = 11,
            FIELD_HOURGLASS_Z = 12, FIELD_HOURGLASS_STIFFNESS = 13, FIELD_DAMAGE_STRENGTH = 14,
            FIELD_DAMAGE_SOFTENING = 15, FIELD_DAMAGE_WIDTH = 16, FIELD_ERODED = 17,
            FIELD_ON_WALL = 18, FIELD_WALL_STATE = 19, FIELD_CONTACT_MASTER = 20,
            FIELD_CONTACT_STATE = 21, FIELD_SURFACE_EDGES = 22, FIELD_SURFACE_NODES = 23,
            FIELD_FIXED = 24;

    static final Linker LINKER = Linker.nativeLinker();
    static final SymbolLookup LIB = SymbolLookup.libraryLookup(
            System.getProperty("neofiz.gpu.lib", "libneofiz_gpu.so"), Arena.global());

    // ------------------------------------------------------------------ layouts

    /** nf_mesh */
    static final StructLayout MESH = MemoryLayout.structLayout(
            JAVA_INT.withName("node_count"), JAVA_INT.withName("element_count"),
            JAVA_INT.withName("pressure_edge_count"), MemoryLayout.paddingLayout(4),
            ADDRESS.withName("r"), ADDRESS.withName("z"), ADDRESS.withName("conn"),
            ADDRESS.withName("pressure_edges"));

    /** nf_material */
    static final StructLayout MATERIAL = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("youngs_modulus"), JAVA_DOUBLE.withName("poisson_ratio"),
            JAVA_DOUBLE.withName("density"), JAVA_DOUBLE.withName("yield_stress"),
            JAVA_DOUBLE.withName("isotropic_hardening"),
            JAVA_DOUBLE.withName("kinematic_hardening"),
            JAVA_INT.withName("has_johnson_cook"), JAVA_INT.withName("reserved"),
            JAVA_DOUBLE.withName("jc_a"), JAVA_DOUBLE.withName("jc_b"),
            JAVA_DOUBLE.withName("jc_n"), JAVA_DOUBLE.withName("jc_c"),
            JAVA_DOUBLE.withName("jc_m"), JAVA_DOUBLE.withName("jc_reference_strain_rate"),
            JAVA_DOUBLE.withName("jc_room_temperature"),
            JAVA_DOUBLE.withName("jc_melt_temperature"),
            JAVA_DOUBLE.withName("jc_specific_heat"), JAVA_DOUBLE.withName("jc_taylor_quinney"));

    /** nf_state */
    static final StructLayout STATE = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("time"), JAVA_DOUBLE.withName("timestep"),
            JAVA_DOUBLE.withName("timestep_previous"), JAVA_DOUBLE.withName("reference_timestep"),
            JAVA_DOUBLE.withName("mass_scale"), JAVA_DOUBLE.withName("min_edge_squared"),
            JAVA_DOUBLE.withName("fastest_wave"), JAVA_DOUBLE.withName("eroded_energy"),
            JAVA_DOUBLE.withName("bore_pressure"), JAVA_LONG.withName("steps"),
            JAVA_INT.withName("eroded_elements"), JAVA_INT.withName("inverted_elements"),
            JAVA_INT.withName("node_count"), JAVA_INT.withName("element_count"),
            JAVA_INT.withName("points_per_element"), JAVA_INT.withName("pressure_edge_count"));

    /** nf_audit */
    static final StructLayout AUDIT = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("kinetic_energy"), JAVA_DOUBLE.withName("centred_kinetic_energy"),
            JAVA_DOUBLE.withName("strain_energy"), JAVA_DOUBLE.withName("plastic_dissipation"),
            JAVA_DOUBLE.withName("hourglass_energy"), JAVA_DOUBLE.withName("fracture_dissipation"),
            JAVA_DOUBLE.withName("axial_momentum"), JAVA_DOUBLE.withName("radial_momentum"),
            JAVA_DOUBLE.withName("max_plastic_strain"), JAVA_DOUBLE.withName("yielded_fraction"),
            JAVA_DOUBLE.withName("max_damage"), JAVA_DOUBLE.withName("damaged_fraction"),
            JAVA_DOUBLE.withName("failed_fraction"), JAVA_DOUBLE.withName("max_temperature"),
            JAVA_INT.withName("clamped_points"), JAVA_INT.withName("most_damaged_element"));

    /** nf_wall_info */
    static final StructLayout WALL_INFO = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("plane"), JAVA_DOUBLE.withName("friction"),
            JAVA_DOUBLE.withName("impulse"), JAVA_DOUBLE.withName("energy_loss"),
            JAVA_DOUBLE.withName("friction_dissipation"), JAVA_INT.withName("contact_count"),
            JAVA_INT.withName("stuck_count"), JAVA_INT.withName("present"),
            JAVA_INT.withName("reserved"));

    /** nf_contact_info */
    static final StructLayout CONTACT_INFO = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("friction"), JAVA_DOUBLE.withName("energy"),
            JAVA_DOUBLE.withName("dissipation"), JAVA_DOUBLE.withName("max_penetration"),
            JAVA_INT.withName("pair_count"), JAVA_INT.withName("escaped_nodes"),
            JAVA_INT.withName("segment_count"), JAVA_INT.withName("present"));

    /** nf_measure */
    static final StructLayout MEASURE = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("z_max"), JAVA_DOUBLE.withName("z_min"),
            JAVA_DOUBLE.withName("length"), JAVA_DOUBLE.withName("mushroom_diameter"));

    /** nf_batch_mesh */
    static final StructLayout BATCH_MESH = MemoryLayout.structLayout(
            JAVA_INT.withName("instance_count"), MemoryLayout.paddingLayout(4),
            ADDRESS.withName("node_offset"), ADDRESS.withName("element_offset"),
            ADDRESS.withName("r"), ADDRESS.withName("z"), ADDRESS.withName("conn"),
            ADDRESS.withName("fixed"), ADDRESS.withName("pressure_offset"),
            ADDRESS.withName("pressure_edges"), ADDRESS.withName("failure_strain"),
            ADDRESS.withName("fracture_energy"));

    /** nf_batch_instance */
    static final StructLayout BATCH_INSTANCE = MemoryLayout.structLayout(
            MATERIAL.withName("material"), JAVA_DOUBLE.withName("velocity_r"),
            JAVA_DOUBLE.withName("velocity_z"), JAVA_DOUBLE.withName("wall_plane"),
            JAVA_DOUBLE.withName("wall_friction"), JAVA_DOUBLE.withName("hourglass"),
            JAVA_DOUBLE.withName("t_end"), JAVA_DOUBLE.withName("pressure"),
            JAVA_DOUBLE.withName("pressure_ramp"), JAVA_DOUBLE.withName("damping_fraction"),
            JAVA_DOUBLE.withName("damping_omega"));

    /** nf_batch_config */
    static final StructLayout BATCH_CONFIG = MemoryLayout.structLayout(
            JAVA_INT.withName("threads"), JAVA_INT.withName("stage_nodes"),
            JAVA_INT.withName("blocks_per_sm"), JAVA_INT.withName("chunk_steps"));

    /** Byte offset of a named member. */
    static long at(StructLayout layout, String name) {
        return layout.byteOffset(groupElement(name));
    }

    static double getD(MemorySegment s, StructLayout l, String name) {
        return s.get(JAVA_DOUBLE, at(l, name));
    }

    static int getI(MemorySegment s, StructLayout l, String name) {
        return s.get(JAVA_INT, at(l, name));
    }

    static void setD(MemorySegment s, StructLayout l, String name, double v) {
        s.set(JAVA_DOUBLE, at(l, name), v);
    }

    static void setI(MemorySegment s, StructLayout l, String name, int v) {
        s.set(JAVA_INT, at(l, name), v);
    }

    static void setA(MemorySegment s, StructLayout l, String name, MemorySegment v) {
        s.set(ADDRESS, at(l, name), v);
    }

    // ------------------------------------------------------------------ entry points

    private static MethodHandle fn(String name, FunctionDescriptor d) {
        return LINKER.downcallHandle(LIB.find(name).orElseThrow(
                () -> new UnsatisfiedLinkError("libneofiz_gpu.so has no " + name)), d);
    }

    private static FunctionDescriptor st(java.lang.foreign.MemoryLayout... args) {
        return FunctionDescriptor.of(JAVA_INT, args);
    }

    static final MethodHandle CREATE = fn("nf_create", st(ADDRESS, ADDRESS, JAVA_INT, ADDRESS,
            JAVA_INT, JAVA_INT, JAVA_INT, JAVA_DOUBLE, JAVA_DOUBLE, ADDRESS));
    static final MethodHandle DESTROY = fn("nf_destroy", st(ADDRESS));
    static final MethodHandle LAST_ERROR = fn("nf_last_error", FunctionDescriptor.of(ADDRESS, ADDRESS));
    static final MethodHandle STATUS_WORD = fn("nf_status_word", st(ADDRESS, ADDRESS));
    static final MethodHandle CHECK = fn("nf_check", st(ADDRESS));
    static final MethodHandle FIX_RADIAL = fn("nf_fix_radial", st(ADDRESS, JAVA_INT));
    static final MethodHandle FIX_AXIAL = fn("nf_fix_axial", st(ADDRESS, JAVA_INT));
    static final MethodHandle FIX_ALL_AXIAL = fn("nf_fix_all_axial", st(ADDRESS));
    static final MethodHandle SET_PRESSURE_RAMP = fn("nf_set_pressure_ramp",
            st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle SET_RELAXATION_DAMPING = fn("nf_set_relaxation_damping",
            st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle SET_HOURGLASS = fn("nf_set_hourglass_coefficient",
            st(ADDRESS, JAVA_DOUBLE));
    static final MethodHandle SET_RIGID_WALL = fn("nf_set_rigid_wall",
            st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle CLEAR_RIGID_WALL = fn("nf_clear_rigid_wall", st(ADDRESS));
    static final MethodHandle SET_CONTACT = fn("nf_set_contact",
            st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle CLEAR_CONTACT = fn("nf_clear_contact", st(ADDRESS));
    static final MethodHandle SET_GRAVITY = fn("nf_set_gravity", st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle SET_EROSION = fn("nf_set_erosion", st(ADDRESS, JAVA_DOUBLE));
    static final MethodHandle SET_MASS_SCALING = fn("nf_set_mass_scaling", st(ADDRESS, JAVA_DOUBLE));
    static final MethodHandle SET_DAMAGE = fn("nf_set_damage", st(ADDRESS, ADDRESS, ADDRESS));
    static final MethodHandle SET_VELOCITY = fn("nf_set_velocity",
            st(ADDRESS, JAVA_INT, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle SET_UNIFORM_VELOCITY = fn("nf_set_uniform_velocity",
            st(ADDRESS, JAVA_DOUBLE, JAVA_DOUBLE));
    static final MethodHandle STEP = fn("nf_step", st(ADDRESS, JAVA_LONG));
    static final MethodHandle ADVANCE = fn("nf_advance", st(ADDRESS));
    static final MethodHandle RUN_UNTIL = fn("nf_run_until",
            st(ADDRESS, JAVA_DOUBLE, JAVA_LONG, ADDRESS));
    static final MethodHandle SYNCHRONIZE = fn("nf_synchronize", st(ADDRESS));
    static final MethodHandle FIELD_SIZE = fn("nf_field_size", st(ADDRESS, JAVA_INT, ADDRESS, ADDRESS));
    static final MethodHandle READ_FIELD = fn("nf_read_field",
            st(ADDRESS, JAVA_INT, ADDRESS, JAVA_LONG));
    static final MethodHandle WRITE_FIELD = fn("nf_write_field",
            st(ADDRESS, JAVA_INT, ADDRESS, JAVA_LONG));
    static final MethodHandle GET_STATE = fn("nf_get_state", st(ADDRESS, ADDRESS));
    static final MethodHandle AUDITS = fn("nf_audits", st(ADDRESS, ADDRESS));
    static final MethodHandle WALL_STATS = fn("nf_wall_stats", st(ADDRESS, ADDRESS));
    static final MethodHandle CONTACT_STATS = fn("nf_contact_stats", st(ADDRESS, ADDRESS));
    static final MethodHandle MEASURE_BODY = fn("nf_measure_body", st(ADDRESS, ADDRESS));

    static final MethodHandle BATCH_CREATE = fn("nf_batch_create", st(ADDRESS, ADDRESS, JAVA_INT,
            JAVA_INT, JAVA_DOUBLE, JAVA_DOUBLE, JAVA_INT, ADDRESS));
    static final MethodHandle BATCH_DESTROY = fn("nf_batch_destroy", st(ADDRESS));
    static final MethodHandle BATCH_LAST_ERROR = fn("nf_batch_last_error",
            FunctionDescriptor.of(ADDRESS, ADDRESS));
    static final MethodHandle BATCH_TUNE = fn("nf_batch_tune", st(ADDRESS, JAVA_INT, ADDRESS));
    static final MethodHandle BATCH_RUN = fn("nf_batch_run", st(ADDRESS, JAVA_LONG));
    static final MethodHandle BATCH_ELAPSED = fn("nf_batch_elapsed", st(ADDRESS, ADDRESS));
    static final MethodHandle BATCH_MEASURE = fn("nf_batch_measure", st(ADDRESS, ADDRESS));
    static final MethodHandle BATCH_ADJOINT_FORWARD = fn("nf_batch_adjoint_forward",
            st(ADDRESS, JAVA_INT, JAVA_INT));
    static final MethodHandle BATCH_ADJOINT_BACKWARD = fn("nf_batch_adjoint_backward",
            st(ADDRESS, JAVA_INT, ADDRESS, ADDRESS));
    static final MethodHandle BATCH_ADJOINT_BACKWARD_MANY = fn("nf_batch_adjoint_backward_many",
            st(ADDRESS, ADDRESS, JAVA_INT, ADDRESS, ADDRESS));
    static final MethodHandle BATCH_ADJOINT_ELAPSED = fn("nf_batch_adjoint_elapsed",
            st(ADDRESS, ADDRESS, ADDRESS));

    // ------------------------------------------------------------------ errors

    /** Throws the reference's exception for a failed call on a solver handle. */
    static void check(int status, MemorySegment handle) {
        if (status == NF_OK) return;
        throw failure(status, message(LAST_ERROR, handle));
    }

    /** Throws the reference's exception for a failed call on a batch handle. */
    static void checkBatch(int status, MemorySegment handle) {
        if (status == NF_OK) return;
        throw failure(status, message(BATCH_LAST_ERROR, handle));
    }

    private static String message(MethodHandle lastError, MemorySegment handle) {
        try {
            MemorySegment p = (MemorySegment) lastError.invokeExact(handle);
            return p.equals(MemorySegment.NULL) ? "" : p.reinterpret(4096).getString(0);
        } catch (Throwable t) {
            return "(no message: " + t + ")";
        }
    }

    static RuntimeException failure(int status, String msg) {
        return switch (status) {
            case NF_EINVAL -> new IllegalArgumentException(msg);
            case NF_ESTATE -> new IllegalStateException(msg);
            case NF_ETIMEOUT -> new DeviceException(msg, true);
            default -> new DeviceException(msg, false);
        };
    }

    static RuntimeException rethrow(Throwable t) {
        if (t instanceof RuntimeException r) return r;
        if (t instanceof Error e) throw e;
        return new IllegalStateException(t);
    }
}
