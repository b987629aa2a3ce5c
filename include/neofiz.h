/*
 * neofiz.h -- C ABI of libneofiz_gpu.so, a GB300 (sm_103a) implementation of the Neofiz
 * explicit central-difference timestep.
 *
 * The reference has no FFI of its own: its surface is the Java class
 * org.neofiz.solver.ExplicitSolver (src/main/java/org/neofiz/solver/ExplicitSolver.java)
 * with its collaborators RigidWall and Contact. Each entry point below replaces one method
 * of that surface and cites it. A Java caller binds these through java.lang.foreign; the
 * binding is plain C: scalars, pointers to caller-owned host arrays, sizes.
 *
 * Ownership: nf_create deep-copies every mesh and material array to the device; nothing
 * passed in is retained. Reads copy device -> caller buffer only when asked. A handle is
 * single-owner and not thread-safe (as ExplicitSolver is); distinct handles may be driven from
 * distinct host threads. Each handle owns one CUDA stream.
 *
 * Errors: every function returns an nf_status. NF_EINVAL corresponds to the reference's
 * IllegalArgumentException and NF_ESTATE to IllegalStateException, with the same messages,
 * readable through nf_last_error. Numerical faults detected on the device (a non-finite
 * nodal value, a bounded wait that ran out) are reported through nf_status_word, never by
 * trapping.
 */
#ifndef NEOFIZ_H
#define NEOFIZ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    NF_OK = 0,
    NF_EINVAL = 1,     /* IllegalArgumentException */
    NF_ESTATE = 2,     /* IllegalStateException */
    NF_EDEVICE = 3,    /* CUDA error, no device, or a device-side status bit */
    NF_ETIMEOUT = 4,   /* a bounded device-side wait gave up */
    NF_ENOMEM = 5
} nf_status;

/* core/Formulation.java:16-23 */
enum { NF_AXISYMMETRIC = 0, NF_PLANE_STRAIN = 1, NF_PLANE_STRESS = 2 };
/* solver/Integration.java:11-27 */
enum { NF_FULL = 0, NF_REDUCED = 1 };
/* solver/Kinematics.java:11-34 */
enum { NF_SMALL_STRAIN = 0, NF_FINITE_STRAIN = 1 };

/* mesh/QuadMesh.java:17-54: flat structure-of-arrays mesh, CCW element winding. */
typedef struct {
    int32_t node_count;
    int32_t element_count;
    int32_t pressure_edge_count;     /* edges, not ints */
    const double *r;                 /* [node_count] reference radial coordinate, m */
    const double *z;                 /* [node_count] reference axial coordinate, m */
    const int32_t *conn;             /* [4 * element_count] */
    const int32_t *pressure_edges;   /* [2 * pressure_edge_count], may be NULL if none */
} nf_mesh;

/* core/Material.java:20-21 and core/JohnsonCook.java:66-69. yield_stress = +inf is an
 * elastic material (Material.java:61-63). */
typedef struct {
    double youngs_modulus;
    double poisson_ratio;
    double density;
    double yield_stress;
    double isotropic_hardening;
    double kinematic_hardening;
    int32_t has_johnson_cook;
    int32_t reserved;
    double jc_a, jc_b, jc_n, jc_c, jc_m;
    double jc_reference_strain_rate;
    double jc_room_temperature;
    double jc_melt_temperature;
    double jc_specific_heat;
    double jc_taylor_quinney;
} nf_material;

typedef struct nf_solver nf_solver;

/* Scalar state of the integrator (ExplicitSolver.java:191-234, getters :622-652, :825-840). */
typedef struct {
    double time;
    double timestep;
    double timestep_previous;
    double reference_timestep;       /* dt0 */
    double mass_scale;
    double min_edge_squared;
    double fastest_wave;
    double eroded_energy;
    double bore_pressure;            /* pressureAt(time), :826-828 */
    int64_t steps;
    int32_t eroded_elements;
    int32_t inverted_elements;
    int32_t node_count;
    int32_t element_count;
    int32_t points_per_element;
    int32_t pressure_edge_count;
} nf_state;

/* Energy, momentum and damage audits (ExplicitSolver.java:875-886, :1610-1860). */
typedef struct {
    double kinetic_energy;
    double centred_kinetic_energy;
    double strain_energy;
    double plastic_dissipation;
    double hourglass_energy;
    double fracture_dissipation;
    double axial_momentum;
    double radial_momentum;
    double max_plastic_strain;
    double yielded_fraction;
    double max_damage;
    double damaged_fraction;
    double failed_fraction;
    double max_temperature;          /* NaN when no element has a Johnson-Cook law */
    int32_t clamped_points;          /* Damage.java:391-397 */
    int32_t most_damaged_element;    /* :1778-1793 */
} nf_audit;

/* RigidWall.java:285-315 */
typedef struct {
    double plane;
    double friction;
    double impulse;
    double energy_loss;
    double friction_dissipation;
    int32_t contact_count;
    int32_t stuck_count;
    int32_t present;
    int32_t reserved;
} nf_wall_info;

/* Contact.java:366-404 */
typedef struct {
    double friction;
    double energy;
    double dissipation;
    double max_penetration;
    int32_t pair_count;
    int32_t escaped_nodes;
    int32_t segment_count;
    int32_t present;
} nf_contact_info;

/* Measurements on the deformed body: TaylorImpactCase.java:272-288 (length, mushroom). */
typedef struct {
    double z_max;
    double z_min;
    double length;                   /* z_max - z_min */
    double mushroom_diameter;        /* 2 max(r + ur) */
} nf_measure;

/* Fields readable with nf_read_field. Per-node doubles, per-point doubles (stride 4 for
 * tensors, {rr, zz, tt, rz}), per-element doubles, byte flags and int32 lists. */
typedef enum {
    NF_FIELD_UR = 0, NF_FIELD_UZ, NF_FIELD_VR, NF_FIELD_VZ, NF_FIELD_FR, NF_FIELD_FZ,
    NF_FIELD_MASS,
    NF_FIELD_STRESS,                 /* 4 doubles per point */
    NF_FIELD_BACK_STRESS,            /* 4 doubles per point */
    NF_FIELD_PLASTIC_STRAIN,         /* per point */
    NF_FIELD_PLASTIC_WORK,           /* per point, J/m^3 */
    NF_FIELD_HOURGLASS_R,            /* per element */
    NF_FIELD_HOURGLASS_Z,
    NF_FIELD_HOURGLASS_STIFFNESS,
    NF_FIELD_DAMAGE_STRENGTH,        /* per point; zero until onset */
    NF_FIELD_DAMAGE_SOFTENING,
    NF_FIELD_DAMAGE_WIDTH,
    NF_FIELD_ERODED,                 /* uint8 per element */
    NF_FIELD_ON_WALL,                /* uint8 per node */
    NF_FIELD_WALL_STATE,             /* uint8 per node, last step: NF_WALL_* bits */
    NF_FIELD_CONTACT_MASTER,         /* int32 per node: master segment or -1 */
    NF_FIELD_CONTACT_STATE,          /* uint8 per node: NF_CONTACT_* of its own pair */
    NF_FIELD_SURFACE_EDGES,          /* int32 pairs, current free surface */
    NF_FIELD_SURFACE_NODES,          /* int32, ascending */
    NF_FIELD_FIXED,                  /* uint8 per node: bit0 radial, bit1 axial */
    NF_FIELD_COUNT
} nf_field;

enum { NF_WALL_HELD = 1, NF_WALL_STUCK = 2, NF_WALL_SLID = 4, NF_WALL_ARRIVED = 8 };
enum { NF_CONTACT_PAIR = 1, NF_CONTACT_STICK = 2, NF_CONTACT_SLIP = 4 };

/* ------------------------------------------------------------------ lifecycle */

/* Number of CUDA devices visible to the library (0 when none); no reference counterpart. */
int nf_device_count(void);

/* ExplicitSolver(QuadMesh, Materials, Formulation, Integration, Kinematics, thickness,
 * cflSafety), ExplicitSolver.java:264-339 (per-element material unroll :284-300, node slots
 * :347-366, lumped mass :1559-1597, initial CFL step :333-338). element_material may be
 * NULL when material_count == 1 (Materials.uniform, core/Materials.java:36-39). */
nf_status nf_create(const nf_mesh *mesh, const nf_material *materials, int32_t material_count,
                    const int32_t *element_material, int32_t formulation, int32_t integration,
                    int32_t kinematics, double thickness, double cfl_safety, nf_solver **out);
/* ExplicitSolver.shutdown, ExplicitSolver.java:395-400 (also frees device memory). */
nf_status nf_destroy(nf_solver *h);
/* Message of the last failure on this handle, or of the calling thread when h is NULL. */
const char *nf_last_error(const nf_solver *h);
/* Bits of the status word. */
enum { NF_STATUS_NONFINITE = 1,        /* a nodal velocity or displacement stopped being finite */
       NF_STATUS_BUCKET_OVERFLOW = 4,  /* a contact bucket exceeded its bound */
       NF_STATUS_TIMEOUT = 8 };        /* a contact-pass grid barrier gave up waiting */
/* Sticky device-side status bits (NaN seen, wait timed out); 0 when healthy. */
nf_status nf_status_word(nf_solver *h, uint32_t *word);
/* Waits for the handle's work, then turns the status word into a status: NF_ETIMEOUT when a
 * contact-pass barrier gave up (that step's contact forces are incomplete; the handle refuses
 * every later nf_step, nf_advance and nf_run_until with NF_ETIMEOUT, and nf_synchronize
 * reports it too), NF_EDEVICE when a nodal velocity or displacement stopped being finite,
 * NF_OK otherwise. The reference has no counterpart: its NaNs propagate silently, and
 * nothing of it waits on another thread without end. A caller checks this on sampled
 * frames. */
nf_status nf_check(nf_solver *h);
/* Limits of the contact pass's grid-barrier wait: at most `polls` polls and `nanoseconds` of
 * the GPU's global timer per wait (0 restores the defaults, 2^27 polls and one second). For
 * tests that make a wait run out; no reference counterpart. */
nf_status nf_set_wait_limit(nf_solver *h, int64_t polls, int64_t nanoseconds);
/* Slots per cell of the contact pass's direct-indexed grid, 0..64 (default 64): a step whose
 * busiest cell holds more entries than this files through the counting sort instead; 0 sends
 * every step there. Both layouts give the same bits; for tests of the fallback and tuning. No
 * reference counterpart. */
nf_status nf_set_grid_slots(nf_solver *h, int32_t slots);

/* ------------------------------------------------------------------ setup (ExplicitSolver) */

nf_status nf_set_threads(nf_solver *h, int32_t n);                           /* :386-392, no-op */
nf_status nf_fix_radial(nf_solver *h, int32_t node);                         /* :408-410 */
nf_status nf_fix_axial(nf_solver *h, int32_t node);                          /* :413-415 */
nf_status nf_fix_all_axial(nf_solver *h);                                    /* :423-425 */
nf_status nf_set_pressure_ramp(nf_solver *h, double pascals, double ramp_seconds); /* :432-435 */
nf_status nf_set_relaxation_damping(nf_solver *h, double fraction_of_critical,
                                    double angular_frequency);              /* :450-455 */
nf_status nf_set_hourglass_coefficient(nf_solver *h, double q);              /* :466-469 */
/* setRigidWall(RigidWall.atZ(plane, friction)), :475-477 and RigidWall.java:110-136.
 * friction = +inf is the welded limit. */
nf_status nf_set_rigid_wall(nf_solver *h, double plane, double friction);
nf_status nf_clear_rigid_wall(nf_solver *h);
/* setContact(new Contact(mesh).withFriction(mu).withDamping(zeta).withStiffnessScale(s)),
 * :487-489 and Contact.java:273-364. */
nf_status nf_set_contact(nf_solver *h, double friction, double damping, double stiffness_scale);
nf_status nf_clear_contact(nf_solver *h);
nf_status nf_set_gravity(nf_solver *h, double accel_r, double accel_z);      /* :509-512 */
nf_status nf_set_erosion(nf_solver *h, double damage_threshold);             /* :549-561 */
nf_status nf_set_mass_scaling(nf_solver *h, double target_step);             /* :601-619 */
/* setDamage(double[] fractureEnergy, double[] failureStrain), :729-791; one value per
 * element each. */
nf_status nf_set_damage(nf_solver *h, const double *fracture_energy, const double *failure_strain);
nf_status nf_set_velocity(nf_solver *h, int32_t node, double vr, double vz);  /* :799-802 */
nf_status nf_set_uniform_velocity(nf_solver *h, double vr, double vz);        /* :805-808 */
/* Bulk form of setVelocity over every node, for callers that would loop :799-802. */
nf_status nf_set_velocities(nf_solver *h, const double *vr, const double *vz);

/* ------------------------------------------------------------------ run */

nf_status nf_step(nf_solver *h, int64_t steps);     /* run(int) / step(), :936-991 */
nf_status nf_advance(nf_solver *h);                 /* advance(), :1069-1075 */
/* run until time() >= t_end, the loop of TaylorImpactCase.java:250-253; steps taken are
 * returned in *taken when non-NULL. The check is made on the device, so no per-step host
 * round trip is needed. */
nf_status nf_run_until(nf_solver *h, double t_end, int64_t max_steps, int64_t *taken);
/* Blocks until the handle's stream is idle. nf_step and nf_advance only enqueue work; reads,
 * audits and nf_synchronize wait for it. Returns NF_ETIMEOUT when a contact-pass barrier of
 * the work waited for gave up (see nf_check). */
nf_status nf_synchronize(nf_solver *h);
/* Runs the handle's kernels on a caller-owned cudaStream_t (passed as void*), or on its own
 * stream again when stream is NULL. No reference counterpart: lets a host application order
 * the solver with its own device work. */
nf_status nf_set_stream(nf_solver *h, void *stream);

/* Arithmetic of the element kernels. NF_PRECISION_FP64 (the default) is the reference's
 * arithmetic, bit for bit. NF_PRECISION_MIXED runs the element constitutive, hourglass and
 * force arithmetic and keeps the element state in FP32, while nodal kinematics, the force
 * gather, contact and all audits stay FP64. Switching converts the current state. No
 * reference counterpart. */
/* NF_PRECISION_COMPENSATED (batches only) also runs the nodal update and the force gather in
 * FP32, each displacement carried as a compensated float pair (hi + lo, about 48 significant
 * bits); time, step size and the audits stay FP64. */
enum { NF_PRECISION_FP64 = 0, NF_PRECISION_MIXED = 1, NF_PRECISION_COMPENSATED = 2 };
nf_status nf_set_precision(nf_solver *h, int32_t precision);

/* ------------------------------------------------------------------ instrumentation */

/* Kernel groups of one step, for nf_profile_read. No reference counterpart. */
enum { NF_GROUP_NODAL = 0, NF_GROUP_ERODE, NF_GROUP_ELEMENT, NF_GROUP_PRESSURE, NF_GROUP_GATHER,
       NF_GROUP_CONTACT, NF_GROUP_END, NF_GROUP_COUNT };
/* When enabled, steps run without graph replay and every kernel group is bracketed by CUDA
 * events on the handle's stream. */
nf_status nf_profile(nf_solver *h, int32_t enable);
/* Accumulated device milliseconds per group since profiling was enabled, and the number of
 * steps they cover; resets the accumulation. ms must hold NF_GROUP_COUNT doubles. */
nf_status nf_profile_read(nf_solver *h, double *ms, int64_t *steps);
/* Kernel launches issued so far by this handle (a replayed graph counts its kernels). */
nf_status nf_launch_count(nf_solver *h, int64_t *launches);

/* The current device's FP64 pipe rate, measured by a kernel of independent dependent DFMA
 * chains on every SM (best of three launches): DFMA warp instructions per second and FP64
 * FLOPs per second (two per lane per DFMA). The denominator of the element pass's FP64
 * roofline; no reference counterpart. */
nf_status nf_device_fp64_rate(double *warp_instructions_per_second, double *flops_per_second);

/* ------------------------------------------------------------------ read-back */

/* Element count and element size in bytes of a field, for sizing the destination. */
nf_status nf_field_size(nf_solver *h, int32_t field, size_t *count, size_t *element_bytes);
/* Copies a field device -> host (the reference's live getters, :842-932). */
nf_status nf_read_field(nf_solver *h, int32_t field, void *dst, size_t bytes);
/* Overwrites a state field host -> device (UR..VZ, STRESS, BACK_STRESS, PLASTIC_STRAIN,
 * PLASTIC_WORK): the writes reference callers make through the live arrays. */
nf_status nf_write_field(nf_solver *h, int32_t field, const void *src, size_t bytes);
nf_status nf_get_state(nf_solver *h, nf_state *out);
nf_status nf_audits(nf_solver *h, nf_audit *out);
nf_status nf_wall_stats(nf_solver *h, nf_wall_info *out);
nf_status nf_contact_stats(nf_solver *h, nf_contact_info *out);
nf_status nf_measure_body(nf_solver *h, nf_measure *out);

/* ------------------------------------------------------------------ material point */

/* J2.update(sig, back, epsP, work, p, dRR, dZZ, dTT, dGamRZ, lambda, mu, flow, strainDt,
 * damage), solver/J2.java:163-296 with the Johnson-Cook solve :332-375 and damage onset
 * Damage.java:306-336, run once per point on the device. lambda/mu/flow come from the
 * material as the solver derives them (ExplicitSolver.java:289-299). Arrays are host memory,
 * updated in place; damage arrays may all be NULL for a material that cannot fail, else
 * geometry has 5 doubles per point (area, uR, uZ, vR, vZ). dgamma receives J2.update's
 * return value. strain holds {dRR, dZZ, dTT, dGamRZ} per point. */
typedef struct {
    const double *failure_strain;
    const double *fracture_energy;
    const double *youngs_modulus;
    const double *geometry;
    double *strength;
    double *softening;
    double *width;
} nf_damage_points;

nf_status nf_material_point_update(const nf_material *material, int32_t formulation,
                                   int32_t count, double *sig, double *back, double *eps_p,
                                   double *work, const double *strain, double strain_dt,
                                   const nf_damage_points *damage, double *dgamma);

/* No counterpart in the reference. The same update as nf_material_point_update for callers
 * that cannot allocate device memory -- cudaMalloc/cudaFree synchronise the whole device, and
 * a process whose GPU memory is owned by its own pool allocator has none to spare. It stages
 * through a fixed device array of 8192 points held by the library (1.77 MB on each GPU that
 * loads it), so it calls no allocator; count > 8192 is rejected with NF_EINVAL. The first
 * call on each device looks the array's address up and creates the library's own
 * non-blocking stream for that device (make that first call before any stream capture
 * begins); every call copies, computes and copies back on that stream and waits for it
 * alone, so it neither waits for nor holds up the caller's other streams. Calls share the
 * array, so calls made from several host threads at once race on it. */
nf_status nf_material_point_update_static(const nf_material *material, int32_t formulation,
                                          int32_t count, double *sig, double *back,
                                          double *eps_p, double *work, const double *strain,
                                          double strain_dt, const nf_damage_points *damage,
                                          double *dgamma);

/* ------------------------------------------------------------------ batched scenes */

/* Many independent scenes of one formulation, stepped together on one GPU. The reference runs
 * such sweeps one ExplicitSolver per host thread (Sweep.over, app/Sweep.java:82-105, over the
 * Taylor case TaylorImpactCase.run :214-258). Each instance is the sequence
 *   new ExplicitSolver(mesh, material, formulation, REDUCED, kinematics, thickness, cfl)
 *   setHourglassCoefficient(q); fixRadial/fixAxial(fixed nodes);
 *   setRigidWall(RigidWall.atZ(plane, friction)) unless plane is NaN;
 *   setUniformVelocity(vr, vz); then step while time < t_end,
 * plus setPressureRamp on its pressure edges, setRelaxationDamping and setDamage when given,
 * and its trajectory is bit-identical to that scene run alone through nf_create/nf_step in the
 * same precision (NF_PRECISION_FP64 or NF_PRECISION_MIXED); NF_PRECISION_COMPENSATED has no
 * single-scene form, its error is stated against FP64. Only reduced integration is
 * batched, without erosion or contact. Instances may differ in mesh, material, wall,
 * velocity, hourglass, pressure, damping, damage and t_end. */
typedef struct nf_batch nf_batch;

typedef struct {
    int32_t instance_count;
    const int32_t *node_offset;      /* [count + 1]: instance k owns nodes [k] .. [k + 1) */
    const int32_t *element_offset;   /* [count + 1]: and elements [k] .. [k + 1) */
    const double *r;                 /* [total nodes] reference coordinates */
    const double *z;
    const int32_t *conn;             /* [4 * total elements], node numbers local to the
                                        instance, CCW */
    const uint8_t *fixed;            /* [total nodes] bit 0 radial, bit 1 axial, or NULL */
    const int32_t *pressure_offset;  /* [count + 1]: instance k owns pressure edges [k] ..
                                        [k + 1) (QuadMesh pressureEdges), or NULL for none */
    const int32_t *pressure_edges;   /* [2 * total edges], node numbers local to the instance */
    const double *failure_strain;    /* [total elements] setDamage(gf, eps), or NULL for no */
    const double *fracture_energy;   /*   damage in any instance (both or neither) */
} nf_batch_mesh;

typedef struct {
    nf_material material;
    double velocity_r, velocity_z;   /* setUniformVelocity */
    double wall_plane;               /* RigidWall.atZ(plane, friction); NaN for no wall */
    double wall_friction;
    double hourglass;                /* setHourglassCoefficient */
    double t_end;                    /* the run: step while time < t_end */
    double pressure, pressure_ramp;  /* setPressureRamp(pascals, seconds) */
    double damping_fraction;         /* setRelaxationDamping(fraction, omega); omega 0: none */
    double damping_omega;
} nf_batch_instance;

/* A launch shape of the batched step; any valid shape gives the same trajectories. */
typedef struct {
    int32_t threads;                 /* threads per block: 32, 128 or 256 */
    int32_t stage_nodes;             /* mixed form: node geometry staged in shared memory */
    int32_t blocks_per_sm;           /* resident blocks per SM (1 .. occupancy limit) */
    int32_t chunk_steps;             /* steps an instance takes per launch */
} nf_batch_config;

/* Per-instance progress. */
typedef struct {
    double time;
    double timestep;
    int64_t steps;
    uint32_t status;                 /* device status bits of the instance */
    int32_t done;
} nf_batch_progress;

nf_status nf_batch_create(const nf_batch_mesh *mesh, const nf_batch_instance *instances,
                          int32_t formulation, int32_t kinematics, double thickness,
                          double cfl_safety, int32_t precision, nf_batch **out);
nf_status nf_batch_destroy(nf_batch *b);
const char *nf_batch_last_error(const nf_batch *b);
/* Autotuner: times every valid shape on trial_steps steps of the whole batch (state saved and
 * restored, so the trajectory is untouched), keeps the fastest and returns it. */
nf_status nf_batch_tune(nf_batch *b, int32_t trial_steps, nf_batch_config *chosen);
nf_status nf_batch_set_config(nf_batch *b, const nf_batch_config *config);
nf_status nf_batch_get_config(nf_batch *b, nf_batch_config *config);
/* Steps every instance until its time reaches t_end, or max_steps more steps. The chunked
 * launches are replayed as a CUDA graph; returns when all instances are done. */
nf_status nf_batch_run(nf_batch *b, int64_t max_steps);
/* Device time of the last nf_batch_run, milliseconds. */
nf_status nf_batch_elapsed(nf_batch *b, double *ms);
nf_status nf_batch_launch_count(nf_batch *b, int64_t *launches);
/* Fields over all instances, concatenated: node fields (NF_FIELD_UR .. NF_FIELD_MASS,
 * NF_FIELD_WALL_STATE, NF_FIELD_FIXED), element fields (NF_FIELD_STRESS,
 * NF_FIELD_BACK_STRESS, NF_FIELD_PLASTIC_STRAIN, NF_FIELD_PLASTIC_WORK, NF_FIELD_HOURGLASS_*)
 * as doubles (the mixed form's FP32 state widened). */
nf_status nf_batch_field_size(nf_batch *b, int32_t field, size_t *count, size_t *bytes);
nf_status nf_batch_read(nf_batch *b, int32_t field, void *dst, size_t bytes);
/* [instance_count] each. */
nf_status nf_batch_state(nf_batch *b, nf_batch_progress *out);
nf_status nf_batch_measure(nf_batch *b, nf_measure *out);
nf_status nf_batch_wall_stats(nf_batch *b, nf_wall_info *out);

/* ------------------------------------------------------------------ burst measurement */

/* BurstCase.run's measurement (validate/BurstCase.java:446-490) on every instance of a batch:
 * every sample_every steps the wall capacity (loadCapacity, :533-553), the hoop strain
 * (hoopStrain, :560-569, about mean_radius[instance]) and the applied pressure are sampled and
 * the peak kept; an instance stops once its pressure ramp has reached its target and the
 * capacity has fallen `margin` below the peak (BurstCase.PEAK_MARGIN), or at t_end tested at
 * sample points only (the reference runs whole samples). Up to trace_capacity samples per
 * instance are kept (BurstCase.Sample without the energy columns). Set before running; setting
 * again restarts the measurement. No reference counterpart as a batch (the reference runs one
 * solver per case). */
typedef struct {
    int32_t sample_every;            /* BurstCase.SAMPLE_STEPS */
    int32_t trace_capacity;
    double margin;                   /* BurstCase.PEAK_MARGIN */
} nf_batch_burst;
typedef struct {
    double peak_capacity, peak_strain, peak_applied;  /* at the capacity's maximum */
    double capacity, strain, applied;                 /* the last sample */
    int32_t samples;
    int32_t traversed;               /* the peak was passed (Result.traversed) */
} nf_burst_result;
nf_status nf_batch_set_burst(nf_batch *b, const nf_batch_burst *config, const double *mean_radius);
nf_status nf_batch_burst_results(nf_batch *b, nf_burst_result *out);
/* [instance_count * trace_capacity * 4]: time, hoop strain, capacity, applied per sample. */
nf_status nf_batch_burst_trace(nf_batch *b, double *trace);

/* ------------------------------------------------------------------ adjoint */

/* No counterpart in the reference. Gradients of a batch's final measurements with respect to
 * material and wall parameters, by a hand-written reverse sweep of the whole timestep: the
 * forward pass runs every instance to its t_end (N steps) keeping a checkpoint every
 * checkpoint_every steps; the backward pass recomputes each segment from its checkpoint and
 * runs the adjoint of every step in reverse. The elastic/plastic branch of each point, the
 * rate and temperature clamps, the wall's hold/stick/slip/arrive state of each node and the
 * element that sets each CFL step are those of the forward pass (frozen). Objectives are
 * taken after the N steps: the length ratio L/L0 (TaylorImpactCase.java:272-279) or the
 * mushroom diameter 2 max(r + ur) (:281-288); or the peak wall capacity, the largest
 * BurstCase.loadCapacity (BurstCase.java:533-553) sampled every sample_every steps of the
 * forward pass, its gradient taken at the sampled peak (the step of the peak frozen). FP64
 * batches with reduced integration (damage, pressure edges, damping and walls included). */
enum { NF_OBJECTIVE_LENGTH_RATIO = 0, NF_OBJECTIVE_MUSHROOM = 1, NF_OBJECTIVE_PEAK_CAPACITY = 2 };
/* Gradient components: Johnson-Cook A, B, n, C, m (JohnsonCook.java:66-69), the kinematic
 * hardening modulus (Material.java:20-21), the wall friction coefficient (RigidWall.atZ,
 * RigidWall.java:121-136), the fracture energy of every element (setDamage, as a common
 * value: the sum over elements of the per-element derivatives), and the yield stress and
 * isotropic hardening modulus of a material without a Johnson-Cook law (Material.java:20-21,
 * J2 flow stress sy0 + H_iso eps_p). */
enum { NF_PARAM_A = 0, NF_PARAM_B, NF_PARAM_N, NF_PARAM_C, NF_PARAM_M, NF_PARAM_KINEMATIC,
       NF_PARAM_FRICTION, NF_PARAM_FRACTURE_ENERGY, NF_PARAM_YIELD, NF_PARAM_ISOTROPIC,
       NF_PARAM_COUNT };

/* sample_every: the capacity sampling interval (0: no capacity objective). */
nf_status nf_batch_adjoint_forward(nf_batch *b, int32_t checkpoint_every, int32_t sample_every);
/* values[instance_count]; gradients[instance_count * NF_PARAM_COUNT]. May be called once per
 * objective after one forward pass. */
nf_status nf_batch_adjoint_backward(nf_batch *b, int32_t objective, double *values,
                                    double *gradients);
/* Several objectives in one backward pass (count 1 to 3, each at most once per call): the
 * segments are recomputed once and each objective's reverse sweep reads the same recomputed
 * values, so its gradients are bit-identical to a pass of its own. values[count *
 * instance_count] and gradients[count * instance_count * NF_PARAM_COUNT], objective-major. */
nf_status nf_batch_adjoint_backward_many(nf_batch *b, const int32_t *objectives, int32_t count,
                                         double *values, double *gradients);
/* Device (or, for the CPU restatement, wall) time of the last forward and backward passes. */
nf_status nf_batch_adjoint_elapsed(nf_batch *b, double *forward_ms, double *backward_ms);

/* ------------------------------------------------------------------ film (frame capture) */

/* Film.capture (render/Film.java:148-224) on the device: each capture enqueues, on the
 * solver's stream and without waiting, a frame into device memory -- the deformed node
 * positions r + ur, z + uz, the chosen element fields, the live flag of every element
 * (!isEroded), the solver's scalars and the audit partial sums -- and the frames are copied
 * back only when read. Positions and fields are kept in FP64, as the reference's frames hold
 * them. A film belongs to one solver; destroy it before the solver. */
typedef struct nf_film nf_film;
enum {
    NF_FILM_PLASTIC_STRAIN = 0,      /* elementPlasticStrain (ExplicitSolver.java:1897-1901) */
    NF_FILM_DAMAGE,                  /* elementDamage (:1764-1772) */
    NF_FILM_VON_MISES_MPA,           /* Mises of centroidStress (:1886-1894), MPa */
    NF_FILM_HOOP_STRESS_MPA,         /* centroidStress[2], MPa */
    NF_FILM_SPEED,                   /* elementSpeed (:895-902), m/s */
    NF_FILM_FIELD_KINDS
};
typedef struct {
    double time;                     /* s */
    int64_t steps;
    int32_t eroded;                  /* elements gone */
    int32_t contact_pairs;
    double pressure;                 /* the applied bore pressure (pressureAt), Pa */
} nf_film_info;
/* fields[field_count] (NF_FILM_*; up to 8); capacity: frames it can hold. */
nf_status nf_film_create(nf_solver *h, const int32_t *fields, int32_t field_count,
                         int32_t capacity, nf_film **out);
nf_status nf_film_destroy(nf_film *f);
nf_status nf_film_capture(nf_film *f);
nf_status nf_film_frames(nf_film *f, int32_t *count);
/* All frames, frame-major; any pointer may be NULL: r, z [count * nodes], values [count *
 * field_count * elements], live [count * elements], info, audits [count]. */
nf_status nf_film_read(nf_film *f, double *r, double *z, double *values, uint8_t *live,
                       nf_film_info *info, nf_audit *audits);
nf_status nf_film_clear(nf_film *f);
const char *nf_film_last_error(const nf_film *f);

#ifdef __cplusplus
}
#endif

#endif /* NEOFIZ_H */
