// api_batch.cu -- the batched handle of include/neofiz.h (nf_batch_*): many independent scenes
// set up into one set of device arrays, an autotuner over launch shapes, and runs replayed as
// CUDA graphs of chunked persistent launches (k_batch.cu).
//
// Set-up per instance follows nf_create and the setters exactly (the same helpers: lumped mass
// ExplicitSolver.java:1559-1597, node slots :347-366, initial step :333-338), so each
// instance starts from the state its single-scene twin would have.
#include "nf_internal.h"

#include <algorithm>
#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>

using namespace nf;

namespace {

thread_local std::string g_batch_err;

struct Batch {
    Dev d{};
    BatchDev b{};
    cudaStream_t stream = nullptr;
    int device = 0, sms = 1;
    bool mixed = false;                      // FP32 element state (mixed or compensated)
    bool comp = false;                       // the compensated form's FP32 nodal state
    int mode = NF_PRECISION_FP64;
    std::string err;
    std::vector<BatchInst> inst;
    int N = 0, E = 0, count = 0;
    BatchShape shape{256, 0, 1, 256};
    cudaGraphExec_t graph = nullptr;
    BatchShape graphShape{};
    int32_t *hostRemaining = nullptr;        // pinned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double lastMs = 0.0;
    long long launches = 0;
    std::vector<void *> allocs;
    // the adjoint's buffers (nf_batch_adjoint_*)
    AdjDev adj{};
    std::vector<void *> adjAllocs;
    std::vector<void *> burstAllocs;         // nf_batch_set_burst's buffers
    bool adjForward = false;
    double adjForwardMs = 0.0, adjBackwardMs = 0.0;
    long long adjTapeBytes = 0, adjBarBytes = 0, adjSeedBytes = 0;
    std::vector<long long> adjBarOff, adjSeedOff, adjFinOff, adjStateBytes;
};

constexpr int GRAPH_CHUNKS = 4;              // chunked launches per graph replay

nf_status bfail(Batch *B, nf_status st, const char *fmt, ...) {
    char buf[768];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (B) B->err = buf; else g_batch_err = buf;
    return st;
}

#define BCK(B, call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return bfail((B), NF_EDEVICE, "%s: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

template <typename T>
cudaError_t balloc(Batch &B, T **p, size_t count) {
    void *v = nullptr;
    const size_t bytes = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc(&v, bytes);
    if (e != cudaSuccess) return e;
    B.allocs.push_back(v);
    *p = (T *)v;
    return cudaMemsetAsync(v, 0, bytes, B.stream);
}

template <typename T>
cudaError_t bupload(Batch &B, T *dst, const T *src, size_t count) {
    if (!count) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, B.stream);
}

nf_status bsync(Batch &B) {
    BCK(&B, cudaStreamSynchronize(B.stream));
    BCK(&B, cudaGetLastError());
    return NF_OK;
}

void free_adjoint(Batch &B) {
    for (void *p : B.adjAllocs) cudaFree(p);
    B.adjAllocs.clear();
    B.adj = AdjDev{};
    B.adjForward = false;
}

void destroy(Batch *B) {
    if (!B) return;
    if (B->stream) cudaStreamSynchronize(B->stream);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    free_adjoint(*B);
    for (void *p : B->burstAllocs) cudaFree(p);
    for (void *p : B->allocs) cudaFree(p);
    if (B->hostRemaining) cudaFreeHost(B->hostRemaining);
    if (B->ev0) cudaEventDestroy(B->ev0);
    if (B->ev1) cudaEventDestroy(B->ev1);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
}

bool shape_valid(const Batch &B, const BatchShape &s) {
    if (s.threads != 32 && s.threads != 128 && s.threads != 256) return false;
    if (s.stage && !B.mixed) return false;
    if (s.chunk < 1 || s.blocksPerSm < 1) return false;
    return batch_max_blocks_per_sm(B.mode, s, B.b.maxNodes) >= s.blocksPerSm;
}

// The run's launches: reset the queue, launch one chunk; GRAPH_CHUNKS times.
cudaError_t enqueue_chunks(Batch &B, int chunks) {
    for (int c = 0; c < chunks; c++) {
        cudaError_t e = cudaMemsetAsync(B.b.queue, 0, sizeof(int32_t), B.stream);
        if (e != cudaSuccess) return e;
        e = launch_batch_steps(B.d, B.b, B.mode, B.shape, B.sms, B.stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

nf_status ensure_graph(Batch &B) {
    if (B.graph && memcmp(&B.graphShape, &B.shape, sizeof(BatchShape)) == 0) return NF_OK;
    if (B.graph) cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
    cudaGraph_t g = nullptr;
    BCK(&B, cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t launched = enqueue_chunks(B, GRAPH_CHUNKS);
    const cudaError_t ended = cudaStreamEndCapture(B.stream, &g);
    if (launched != cudaSuccess || ended != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return bfail(&B, NF_EDEVICE, "graph capture of the batched step: %s",
                     cudaGetErrorString(launched != cudaSuccess ? launched : ended));
    }
    const cudaError_t inst = cudaGraphInstantiate(&B.graph, g, 0);
    cudaGraphDestroy(g);
    if (inst != cudaSuccess) return bfail(&B, NF_EDEVICE, "graph instantiate: %s", cudaGetErrorString(inst));
    B.graphShape = B.shape;
    return NF_OK;
}

// The arrays a run changes, for the autotuner's save and restore.
struct Span {
    void *ptr;
    size_t bytes;
};

std::vector<Span> mutable_state(const Batch &B) {
    const Dev &d = B.d;
    const size_t N = B.N, E = B.E;
    std::vector<Span> v = {{d.U, 16 * N}, {d.V, 16 * N}, {d.F, 16 * N}, {d.flags, N},
                           {d.wallState, N}, {B.b.sc, sizeof(BatchScalars) * B.count}};
    if (B.b.burst.every > 0) {
        v.push_back({B.b.burst.state, sizeof(BurstState) * B.count});
        v.push_back({B.b.burst.trace, 32 * (size_t)B.count * B.b.burst.traceCap});
    }
    if (B.comp) {
        v.push_back({d.uC, 16 * N});
        v.push_back({d.vC, 8 * N});
        v.push_back({d.fC, 8 * N});
    }
    if (B.mixed) {
        v.push_back({d.sigF, 16 * E});
        v.push_back({d.backF, 16 * E});
        v.push_back({d.epsPF, 4 * E});
        v.push_back({d.wPF, 4 * E});
        v.push_back({d.hgF, 8 * E});
        v.push_back({d.hgKF, 4 * E});
        if (d.dStrF) {
            v.push_back({d.dStrF, 4 * E});
            v.push_back({d.dSoftF, 4 * E});
            v.push_back({d.dWidthF, 4 * E});
        }
    } else {
        v.push_back({d.sig, 32 * E});
        v.push_back({d.back, 32 * E});
        v.push_back({d.epsP, 8 * E});
        v.push_back({d.wP, 8 * E});
        v.push_back({d.hg, 16 * E});
        v.push_back({d.hgK, 8 * E});
        if (d.dStrength) {
            v.push_back({d.dStrength, 8 * E});
            v.push_back({d.dSoft, 8 * E});
            v.push_back({d.dWidth, 8 * E});
        }
    }
    return v;
}

}  // namespace

extern "C" {

const char *nf_batch_last_error(const nf_batch *h) {
    const Batch *B = reinterpret_cast<const Batch *>(h);
    return B ? B->err.c_str() : g_batch_err.c_str();
}

nf_status nf_batch_create(const nf_batch_mesh *mesh, const nf_batch_instance *instances,
                          int32_t formulation, int32_t kinematics, double thickness,
                          double cfl_safety, int32_t precision, nf_batch **out) {
    *out = nullptr;
    if (!mesh || !instances || mesh->instance_count < 1 || !mesh->node_offset ||
        !mesh->element_offset || !mesh->r || !mesh->z || !mesh->conn)
        return bfail(nullptr, NF_EINVAL, "a batch needs at least one instance and its mesh arrays");
    if (formulation < 0 || formulation > 2 || kinematics < 0 || kinematics > 1)
        return bfail(nullptr, NF_EINVAL, "unknown formulation or kinematics");
    if (precision != NF_PRECISION_FP64 && precision != NF_PRECISION_MIXED &&
        precision != NF_PRECISION_COMPENSATED)
        return bfail(nullptr, NF_EINVAL, "unknown precision %d", precision);
    const int count = mesh->instance_count;
    if (mesh->node_offset[0] != 0 || mesh->element_offset[0] != 0)
        return bfail(nullptr, NF_EINVAL, "offsets must start at 0");
    for (int k = 0; k < count; k++) {
        if (mesh->node_offset[k + 1] < mesh->node_offset[k] ||
            mesh->element_offset[k + 1] < mesh->element_offset[k])
            return bfail(nullptr, NF_EINVAL, "offsets of instance %d decrease", k);
        const nf_batch_instance &p = instances[k];
        const char *why = validate_material(p.material);
        if (why) return bfail(nullptr, NF_EINVAL, "instance %d: %s", k, why);
        if (formulation == NF_PLANE_STRESS && !std::isinf(p.material.yield_stress))
            return bfail(nullptr, NF_EINVAL,
                         "plane stress plasticity needs its own return map; not implemented");
        if (p.hourglass < 0.0)
            return bfail(nullptr, NF_EINVAL, "instance %d: hourglass coefficient must be >= 0", k);
        if (!std::isnan(p.wall_plane) && (p.wall_friction < 0.0 || p.wall_friction != p.wall_friction))
            return bfail(nullptr, NF_EINVAL, "instance %d: friction coefficient must be >= 0", k);
    }
    const long long Nl = mesh->node_offset[count], El = mesh->element_offset[count];
    const long long Kl = mesh->pressure_offset ? mesh->pressure_offset[count] : 0;
    if (Nl > INT32_MAX / 2 || El > INT32_MAX / 16 || Kl > INT32_MAX / 16)
        return bfail(nullptr, NF_EINVAL, "batch too large: %lld nodes, %lld elements", Nl, El);
    const int N = (int)Nl, E = (int)El, K = (int)Kl;
    if (mesh->pressure_offset) {
        if (mesh->pressure_offset[0] != 0 || (K > 0 && !mesh->pressure_edges))
            return bfail(nullptr, NF_EINVAL, "pressure offsets must start at 0 and have edges");
        for (int k = 0; k < count; k++) {
            if (mesh->pressure_offset[k + 1] < mesh->pressure_offset[k])
                return bfail(nullptr, NF_EINVAL, "pressure offsets of instance %d decrease", k);
            const int nn = mesh->node_offset[k + 1] - mesh->node_offset[k];
            for (long long j = 2LL * mesh->pressure_offset[k]; j < 2LL * mesh->pressure_offset[k + 1]; j++)
                if (mesh->pressure_edges[j] < 0 || mesh->pressure_edges[j] >= nn)
                    return bfail(nullptr, NF_EINVAL, "instance %d: pressure edge refers to node %d of %d",
                                 k, mesh->pressure_edges[j], nn);
        }
    }
    const bool damage = mesh->failure_strain != nullptr || mesh->fracture_energy != nullptr;
    if (damage && (!mesh->failure_strain || !mesh->fracture_energy))
        return bfail(nullptr, NF_EINVAL, "damage needs both failure strains and fracture energies");
    for (int k = 0; k < count; k++) {
        const nf_batch_instance &p = instances[k];
        if (damage) {                                           // ExplicitSolver.java:746-755
            const nf_material &m = p.material;
            const double mu = m.youngs_modulus / (2.0 * (1.0 + m.poisson_ratio));
            const double worst = 2.0 * mu + (2.0 / 3.0) * (m.kinematic_hardening - m.youngs_modulus);
            if (!(worst > 0.0))
                return bfail(nullptr, NF_EINVAL,
                             "instance %d: a fully clamped softening modulus would make the return "
                             "map singular: 2mu + (2/3)(H_kin - E) = %.17g <= 0", k, worst);
        }
        if (p.damping_omega < 0.0)
            return bfail(nullptr, NF_EINVAL, "instance %d: angular frequency must be positive", k);
    }
    if (damage)
        for (int e = 0; e < E; e++) {                           // Damage.java:232-260
            if (!(mesh->fracture_energy[e] > 0.0))
                return bfail(nullptr, NF_EINVAL, "fracture energy must be positive, was %.17g",
                             mesh->fracture_energy[e]);
            if (!(mesh->failure_strain[e] > 0.0))
                return bfail(nullptr, NF_EINVAL, "failure strain must be positive; point %d has %.17g",
                             e, mesh->failure_strain[e]);
        }
    for (int k = 0; k < count; k++) {
        const int n0 = mesh->node_offset[k], nn = mesh->node_offset[k + 1] - n0;
        for (int e = mesh->element_offset[k]; e < mesh->element_offset[k + 1]; e++) {
            for (int c = 0; c < 4; c++) {
                const int v = mesh->conn[4LL * e + c];
                if (v < 0 || v >= nn)
                    return bfail(nullptr, NF_EINVAL, "instance %d: connectivity refers to node %d of %d",
                                 k, v, nn);
            }
            const int32_t local[4] = {mesh->conn[4LL * e], mesh->conn[4LL * e + 1],
                                      mesh->conn[4LL * e + 2], mesh->conn[4LL * e + 3]};
            if (element_signed_area(mesh->r + n0, mesh->z + n0, local, 0) <= 0.0)
                return bfail(nullptr, NF_ESTATE,
                             "instance %d element %d has non-positive area; node ordering must be "
                             "counter-clockwise in (r, z)", k, e - mesh->element_offset[k]);
        }
    }
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs < 1)
        return bfail(nullptr, NF_EDEVICE, "no CUDA device is visible");

    Batch *B = new Batch();
    Dev &d = B->d;
    BatchDev &b = B->b;
    B->mixed = precision != NF_PRECISION_FP64;
    B->comp = precision == NF_PRECISION_COMPENSATED;
    B->mode = precision;
    B->N = N;
    B->E = E;
    B->count = count;
    cudaGetDevice(&B->device);
    cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, B->device);
    if (B->sms < 1) B->sms = 1;
    if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&B->ev0) != cudaSuccess || cudaEventCreate(&B->ev1) != cudaSuccess ||
        cudaMallocHost(&B->hostRemaining, sizeof(int32_t)) != cudaSuccess) {
        destroy(B);
        return bfail(nullptr, NF_EDEVICE, "stream or event creation failed");
    }

    // host set-up, instance by instance, as nf_create and the setters do it
    const bool axi = formulation == NF_AXISYMMETRIC;
    std::vector<double2> X0(N), V(N);
    std::vector<double> mass(N, 0.0), invMass(N);
    std::vector<uint8_t> flags(N, 0);
    std::vector<int4> conn(E);
    std::vector<int32_t> emat(E), slotStart(N + 1, 0), slots(4LL * E + 2LL * K);
    std::vector<int2> pedges(K);
    std::vector<double> geom(damage ? 5LL * E : 0);
    std::vector<MatDev> mats(count);
    std::vector<MatF> matsF(count);
    std::vector<BatchScalars> sc(count);
    std::vector<double> cost(count);
    B->inst.resize(count);
    int maxNodes = 1;
    for (int k = 0; k < count; k++) {
        const nf_batch_instance &p = instances[k];
        const int n0 = mesh->node_offset[k], n1 = mesh->node_offset[k + 1];
        const int e0 = mesh->element_offset[k], e1 = mesh->element_offset[k + 1];
        const int nn = n1 - n0, ne = e1 - e0;
        maxNodes = std::max(maxNodes, nn);
        const double *r = mesh->r + n0, *z = mesh->z + n0;
        const int32_t *lc = mesh->conn + 4LL * e0;
        const int k0 = mesh->pressure_offset ? mesh->pressure_offset[k] : 0;
        const int nk = mesh->pressure_offset ? mesh->pressure_offset[k + 1] - k0 : 0;
        const int32_t *lp = nk ? mesh->pressure_edges + 2LL * k0 : nullptr;
        setup_lumped_mass(r, z, lc, ne, &p.material, nullptr, axi, thickness, mass.data() + n0);
        std::vector<int32_t> ls(nn + 1, 0), lsl(4LL * ne + 2LL * nk);
        setup_node_slots(lc, nn, ne, lp, nk, ls.data(), lsl.data());
        const int slotBase = 4 * e0 + 2 * k0;
        for (int i = 0; i < nn; i++) {
            X0[n0 + i] = make_double2(r[i], z[i]);
            V[n0 + i] = make_double2(p.velocity_r, p.velocity_z);
            invMass[n0 + i] = 1.0 / mass[n0 + i];
            flags[n0 + i] = mesh->fixed ? (uint8_t)(mesh->fixed[n0 + i] & 3) : 0;
            slotStart[n0 + i + 1] = slotBase + ls[i + 1];
        }
        // local sources -> global: element slots shift by 8 e0, edge slots move past all elements
        for (long long j = 0; j < 4LL * ne + 2LL * nk; j++) {
            const int v = lsl[j];
            slots[slotBase + j] = v < 8 * ne ? v + 8 * e0 : (E + k0 + (v >> 3) - ne) * 8 + (v & 7);
        }
        for (int j = 0; j < nk; j++) pedges[k0 + j] = make_int2(lp[2 * j] + n0, lp[2 * j + 1] + n0);
        if (damage)
            for (int e = 0; e < ne; e++) {                      // ExplicitSolver.java:767-789
                const int b = 4 * e;
                const int q0 = lc[b], q1 = lc[b + 1], q2 = lc[b + 2], q3 = lc[b + 3];
                double *g = geom.data() + 5LL * (e0 + e);
                g[1] = 0.5 * (r[q1] - r[q0] + r[q2] - r[q3]);
                g[2] = 0.5 * (z[q1] - z[q0] + z[q2] - z[q3]);
                g[3] = 0.5 * (r[q3] - r[q0] + r[q2] - r[q1]);
                g[4] = 0.5 * (z[q3] - z[q0] + z[q2] - z[q1]);
                g[0] = fabs(element_signed_area(r, z, lc, e));
            }
        for (int e = 0; e < ne; e++) {
            conn[e0 + e] = make_int4(lc[4 * e] + n0, lc[4 * e + 1] + n0, lc[4 * e + 2] + n0,
                                     lc[4 * e + 3] + n0);
            emat[e0 + e] = k;
        }
        mats[k] = material_constants(p.material, formulation);
        matsF[k] = material_constants_f32(mats[k]);
        const double wave = material_wave(p.material);
        const double edge = setup_min_edge(r, z, lc, ne);
        BatchInst &in = B->inst[k];
        in.n0 = n0; in.n1 = n1; in.e0 = e0; in.e1 = e1;
        in.k0 = k0; in.k1 = k0 + nk;
        in.pressure = p.pressure;
        in.ramp = p.pressure_ramp;
        in.hasWall = std::isnan(p.wall_plane) ? 0 : 1;
        in.cfl = cfl_safety;
        in.wave = wave;
        in.massScale = 1.0;
        in.damping = p.damping_omega > 0.0 ? 2.0 * p.damping_fraction * p.damping_omega : 0.0;
        in.hourglass = p.hourglass;
        in.wallPlane = in.hasWall ? p.wall_plane : 0.0;
        in.wallFriction = in.hasWall ? p.wall_friction : 0.0;
        in.tEnd = p.t_end;
        BatchScalars &s = sc[k];
        s.minEdgeSquared = edge * edge;
        s.dt = cfl_safety * edge / wave;                      // :333-338
        s.dtPrevious = s.dt;
        s.stepLimit = 0;
        s.done = 1;
        cost[k] = (double)ne * (p.t_end > 0.0 && s.dt > 0.0 ? p.t_end / s.dt : 1.0);
    }
    std::vector<int32_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });

    d.N = N; d.E = E; d.K = K; d.ppe = 1;
    d.hasDamage = damage ? 1 : 0;
    d.axi = axi ? 1 : 0;
    d.finite = kinematics == NF_FINITE_STRAIN ? 1 : 0;
    d.full = 0;
    d.hasWall = 1;
    d.thickness = thickness;
    d.cfl = cfl_safety;
    d.massScale = 1.0;
    d.nmat = count;
    d.mixed = B->mixed ? 1 : 0;
    d.comp = B->comp ? 1 : 0;
    d.sms = B->sms;
    cudaError_t e_ = cudaSuccess;
#define A(ptr, n) if (e_ == cudaSuccess) e_ = balloc(*B, &(ptr), (n))
    A(d.X0, N); A(d.U, N); A(d.V, N); A(d.F, N); A(d.mass, N); A(d.invMass, N);
    A(d.flags, N); A(d.wallState, N);
    A(d.conn, E); A(d.emat, E); A(d.mats, count);
    A(d.contribution, 8LL * E + 8LL * K);
    A(d.nodeSlotStart, N + 1); A(d.nodeSlot, 4LL * E + 2LL * K);
    A(d.pedges, K);
    if (damage) {
        A(d.dFail, E); A(d.dGf, E); A(d.dGeom, 5LL * E);
        A(d.dStrength, E); A(d.dSoft, E); A(d.dWidth, E);
        if (B->mixed) {
            A(d.dFailF, E); A(d.dGfF, E); A(d.dGeomF, 5LL * E);
            A(d.dStrF, E); A(d.dSoftF, E); A(d.dWidthF, E);
        }
    }
    if (B->mixed) {
        A(d.matsF, count);
        A(d.sigF, 4LL * E); A(d.backF, 4LL * E); A(d.epsPF, E); A(d.wPF, E);
        A(d.hgF, E); A(d.hgKF, E); A(d.contribF, 8LL * E + 8LL * K);
        A(d.pMid, N); A(d.vdt, N);
        if (B->comp) {
            A(d.uC, N); A(d.x0C, N); A(d.vC, N); A(d.fC, N); A(d.mC, N);
        }
    } else {
        A(d.sig, 4LL * E); A(d.back, 4LL * E); A(d.epsP, E); A(d.wP, E);
        A(d.hg, E); A(d.hgK, E);
    }
    BatchInst *dInst = nullptr;
    A(dInst, count);
    A(b.sc, count);
    int32_t *dOrder = nullptr;
    A(dOrder, count);
    A(b.queue, 1); A(b.remaining, 1);
    A(b.measure, 3LL * count);
#undef A
    if (e_ != cudaSuccess) {
        destroy(B);
        return bfail(nullptr, NF_ENOMEM, "batch allocation failed: %s", cudaGetErrorString(e_));
    }
    b.inst = dInst;
    b.order = dOrder;
    b.count = count;
    b.maxNodes = maxNodes;
    e_ = cudaSuccess;
#define U(dst, src, n) if (e_ == cudaSuccess) e_ = bupload(*B, dst, src, n)
    U(d.X0, X0.data(), N); U(d.V, V.data(), N); U(d.mass, mass.data(), N);
    U(d.invMass, invMass.data(), N); U(d.flags, flags.data(), N);
    U(d.conn, conn.data(), E); U(d.emat, emat.data(), E); U(d.mats, mats.data(), count);
    U(d.nodeSlotStart, slotStart.data(), N + 1); U(d.nodeSlot, slots.data(), 4LL * E + 2LL * K);
    U(d.pedges, pedges.data(), K);
    if (damage) {
        U(d.dFail, mesh->failure_strain, E); U(d.dGf, mesh->fracture_energy, E);
        U(d.dGeom, geom.data(), 5LL * E);
        if (B->mixed) {
            std::vector<float> f(E), gf(E), g5(5LL * E);
            for (int e = 0; e < E; e++) {
                f[e] = (float)mesh->failure_strain[e];
                gf[e] = (float)mesh->fracture_energy[e];
            }
            for (size_t j = 0; j < g5.size(); j++) g5[j] = (float)geom[j];
            U(d.dFailF, f.data(), E); U(d.dGfF, gf.data(), E); U(d.dGeomF, g5.data(), 5LL * E);
            if (e_ == cudaSuccess) e_ = cudaStreamSynchronize(B->stream);   // f, gf, g5 die here
        }
    }
    if (B->mixed) U(d.matsF, matsF.data(), count);
    U(dInst, B->inst.data(), count);
    U(b.sc, sc.data(), count);
    U(dOrder, order.data(), count);
#undef U
    if (e_ != cudaSuccess) {
        destroy(B);
        return bfail(nullptr, NF_EDEVICE, "batch upload failed: %s", cudaGetErrorString(e_));
    }
    launch_batch_initial(d, b, B->mixed, B->stream);
    B->launches += 1;
    if (B->comp) {
        launch_batch_comp(d, true, B->stream);
        B->launches += 1;
    }
    // default shape: the most resident blocks of 256 threads, capped at 8 per SM
    BatchShape s{256, 0, 1, 256};
    const int occ = batch_max_blocks_per_sm(B->mode, s, maxNodes);
    s.blocksPerSm = std::max(1, std::min(occ, 8));
    B->shape = s;
    nf_status st = bsync(*B);
    if (st) {
        g_batch_err = B->err;
        destroy(B);
        return st;
    }
    *out = reinterpret_cast<nf_batch *>(B);
    return NF_OK;
}

nf_status nf_batch_destroy(nf_batch *h) {
    destroy(reinterpret_cast<Batch *>(h));
    return NF_OK;
}

nf_status nf_batch_set_config(nf_batch *h, const nf_batch_config *c) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    const BatchShape s{c->threads, c->stage_nodes ? 1 : 0, c->blocks_per_sm, c->chunk_steps};
    if (!shape_valid(B, s))
        return bfail(&B, NF_EINVAL,
                     "launch shape (threads %d, stage %d, blocks/SM %d, chunk %d) is not valid "
                     "for this batch", s.threads, s.stage, s.blocksPerSm, s.chunk);
    B.shape = s;
    return NF_OK;
}

nf_status nf_batch_get_config(nf_batch *h, nf_batch_config *c) {
    const Batch &B = *reinterpret_cast<Batch *>(h);
    c->threads = B.shape.threads;
    c->stage_nodes = B.shape.stage;
    c->blocks_per_sm = B.shape.blocksPerSm;
    c->chunk_steps = B.shape.chunk;
    return NF_OK;
}

nf_status nf_batch_run(nf_batch *h, int64_t max_steps) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    B.lastMs = 0.0;
    if (max_steps <= 0) return NF_OK;
    nf_status st = ensure_graph(B);
    if (st) return st;
    BCK(&B, cudaEventRecord(B.ev0, B.stream));
    launch_batch_arm(B.b, (long long)max_steps, B.stream);
    B.launches += 1;
    BCK(&B, cudaMemcpyAsync(B.hostRemaining, B.b.remaining, sizeof(int32_t),
                            cudaMemcpyDeviceToHost, B.stream));
    st = bsync(B);
    if (st) return st;
    while (*B.hostRemaining > 0) {
        BCK(&B, cudaGraphLaunch(B.graph, B.stream));
        B.launches += GRAPH_CHUNKS;
        BCK(&B, cudaMemcpyAsync(B.hostRemaining, B.b.remaining, sizeof(int32_t),
                                cudaMemcpyDeviceToHost, B.stream));
        st = bsync(B);
        if (st) return st;
    }
    if (B.comp) {                            // the FP64 arrays that reads see
        launch_batch_comp(B.d, false, B.stream);
        B.launches += 1;
    }
    BCK(&B, cudaEventRecord(B.ev1, B.stream));
    st = bsync(B);
    if (st) return st;
    float ms = 0.0f;
    BCK(&B, cudaEventElapsedTime(&ms, B.ev0, B.ev1));
    B.lastMs = ms;
    return NF_OK;
}

nf_status nf_batch_tune(nf_batch *h, int32_t trial_steps, nf_batch_config *chosen) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    if (trial_steps < 1) return bfail(&B, NF_EINVAL, "trial_steps must be positive");
    // save the state a trial changes
    const std::vector<Span> spans = mutable_state(B);
    size_t total = 0;
    for (const Span &s : spans) total += (s.bytes + 255) & ~(size_t)255;
    char *save = nullptr;
    BCK(&B, cudaMalloc(&save, total));
    auto copy = [&](bool toSave) {
        size_t off = 0;
        for (const Span &s : spans) {
            if (toSave) cudaMemcpyAsync(save + off, s.ptr, s.bytes, cudaMemcpyDeviceToDevice, B.stream);
            else cudaMemcpyAsync(s.ptr, save + off, s.bytes, cudaMemcpyDeviceToDevice, B.stream);
            off += (s.bytes + 255) & ~(size_t)255;
        }
    };
    copy(true);
    std::vector<BatchShape> cands;
    // one-warp blocks serve small instances (a burst slice has 16 elements): more of them
    // resident per SM instead of mostly idle 128-thread blocks
    for (int threads : {32, 128, 256})
        for (int stage = 0; stage <= (B.mixed ? 1 : 0); stage++) {
            BatchShape s{threads, stage, 1, trial_steps};
            const int occ = batch_max_blocks_per_sm(B.mode, s, B.b.maxNodes);
            bool atOcc = false;
            for (int bps : {1, 2, 4, 8, 16, 32}) {
                if (bps > occ) break;
                s.blocksPerSm = bps;
                cands.push_back(s);
                atOcc = bps == occ;
            }
            if (occ > 0 && !atOcc) {
                s.blocksPerSm = occ;
                cands.push_back(s);
            }
        }
    const BatchShape keep = B.shape;
    double bestMs = 1e300;
    BatchShape best = keep;
    nf_status st = NF_OK;
    // two rounds, each candidate kept at its faster trial: one trial of a few steps is noisy
    std::vector<float> fastest(cands.size(), 3.0e38f);
    for (int round = 0; round < 2 && !st; round++)
        for (size_t i = 0; i < cands.size(); i++) {
            B.shape = cands[i];
            cudaEventRecord(B.ev0, B.stream);
            launch_batch_arm(B.b, trial_steps, B.stream);
            cudaError_t e = enqueue_chunks(B, 1);
            cudaEventRecord(B.ev1, B.stream);
            B.launches += 2;
            if (e == cudaSuccess) e = cudaStreamSynchronize(B.stream);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, B.ev0, B.ev1);
            copy(false);
            if (e != cudaSuccess) {
                st = bfail(&B, NF_EDEVICE, "autotuner trial failed: %s", cudaGetErrorString(e));
                break;
            }
            fastest[i] = std::min(fastest[i], ms);
        }
    for (size_t i = 0; i < cands.size() && !st; i++)
        if (fastest[i] < bestMs) {
            bestMs = fastest[i];
            best = cands[i];
        }
    cudaStreamSynchronize(B.stream);
    cudaFree(save);
    best.chunk = keep.chunk;
    B.shape = st ? keep : best;
    if (chosen) nf_batch_get_config(h, chosen);
    if (st) return st;
    return bsync(B);
}

nf_status nf_batch_elapsed(nf_batch *h, double *ms) {
    *ms = reinterpret_cast<Batch *>(h)->lastMs;
    return NF_OK;
}

nf_status nf_batch_launch_count(nf_batch *h, int64_t *launches) {
    *launches = reinterpret_cast<Batch *>(h)->launches;
    return NF_OK;
}

nf_status nf_batch_field_size(nf_batch *h, int32_t field, size_t *count, size_t *bytes) {
    const Batch &B = *reinterpret_cast<Batch *>(h);
    *bytes = 8;
    switch (field) {
        case NF_FIELD_UR: case NF_FIELD_UZ: case NF_FIELD_VR: case NF_FIELD_VZ:
        case NF_FIELD_FR: case NF_FIELD_FZ: case NF_FIELD_MASS: *count = B.N; return NF_OK;
        case NF_FIELD_WALL_STATE: case NF_FIELD_FIXED: *count = B.N; *bytes = 1; return NF_OK;
        case NF_FIELD_STRESS: case NF_FIELD_BACK_STRESS: *count = 4 * (size_t)B.E; return NF_OK;
        case NF_FIELD_PLASTIC_STRAIN: case NF_FIELD_PLASTIC_WORK: case NF_FIELD_HOURGLASS_R:
        case NF_FIELD_HOURGLASS_Z: case NF_FIELD_HOURGLASS_STIFFNESS: *count = B.E; return NF_OK;
        default: return bfail(const_cast<Batch *>(&B), NF_EINVAL, "field %d is not readable from a batch", field);
    }
}

nf_status nf_batch_read(nf_batch *h, int32_t field, void *dst, size_t nbytes) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    size_t count = 0, bytes = 0;
    nf_status st = nf_batch_field_size(h, field, &count, &bytes);
    if (st) return st;
    if (nbytes < count * bytes)
        return bfail(&B, NF_EINVAL, "buffer of %zu bytes is smaller than the field (%zu)", nbytes,
                     count * bytes);
    BCK(&B, cudaStreamSynchronize(B.stream));
    const Dev &d = B.d;
    double *o = (double *)dst;
    auto pairs = [&](const double2 *src, int comp) -> nf_status {
        std::vector<double2> t(count);
        BCK(&B, cudaMemcpy(t.data(), src, 16 * count, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < count; i++) o[i] = comp ? t[i].y : t[i].x;
        return NF_OK;
    };
    auto plain = [&](const void *src, size_t elem) -> nf_status {
        BCK(&B, cudaMemcpy(dst, src, elem * count, cudaMemcpyDeviceToHost));
        return NF_OK;
    };
    auto widen = [&](const float *src) -> nf_status {
        std::vector<float> t(count);
        BCK(&B, cudaMemcpy(t.data(), src, 4 * count, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < count; i++) o[i] = t[i];
        return NF_OK;
    };
    switch (field) {
        case NF_FIELD_UR: return pairs(d.U, 0);
        case NF_FIELD_UZ: return pairs(d.U, 1);
        case NF_FIELD_VR: return pairs(d.V, 0);
        case NF_FIELD_VZ: return pairs(d.V, 1);
        case NF_FIELD_FR: return pairs(d.F, 0);
        case NF_FIELD_FZ: return pairs(d.F, 1);
        case NF_FIELD_MASS: return plain(d.mass, 8);
        case NF_FIELD_WALL_STATE: return plain(d.wallState, 1);
        case NF_FIELD_FIXED: {
            std::vector<uint8_t> f(count);
            BCK(&B, cudaMemcpy(f.data(), d.flags, count, cudaMemcpyDeviceToHost));
            uint8_t *u = (uint8_t *)dst;
            for (size_t i = 0; i < count; i++) u[i] = f[i] & 3;
            return NF_OK;
        }
        case NF_FIELD_STRESS: return B.mixed ? widen(d.sigF) : plain(d.sig, 8);
        case NF_FIELD_BACK_STRESS: return B.mixed ? widen(d.backF) : plain(d.back, 8);
        case NF_FIELD_PLASTIC_STRAIN: return B.mixed ? widen(d.epsPF) : plain(d.epsP, 8);
        case NF_FIELD_PLASTIC_WORK: return B.mixed ? widen(d.wPF) : plain(d.wP, 8);
        case NF_FIELD_HOURGLASS_STIFFNESS: return B.mixed ? widen(d.hgKF) : plain(d.hgK, 8);
        case NF_FIELD_HOURGLASS_R: case NF_FIELD_HOURGLASS_Z: {
            const int comp = field == NF_FIELD_HOURGLASS_Z;
            if (B.mixed) {
                std::vector<float2> t(count);
                BCK(&B, cudaMemcpy(t.data(), d.hgF, 8 * count, cudaMemcpyDeviceToHost));
                for (size_t i = 0; i < count; i++) o[i] = comp ? t[i].y : t[i].x;
                return NF_OK;
            }
            return pairs(d.hg, comp);
        }
        default: return bfail(&B, NF_EINVAL, "field %d is not readable from a batch", field);
    }
}

nf_status nf_batch_state(nf_batch *h, nf_batch_progress *out) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    std::vector<BatchScalars> sc(B.count);
    BCK(&B, cudaMemcpyAsync(sc.data(), B.b.sc, sizeof(BatchScalars) * B.count,
                            cudaMemcpyDeviceToHost, B.stream));
    const BurstDev &bd = B.b.burst;
    std::vector<BurstState> burst(bd.every > 0 ? B.count : 0);
    if (bd.every > 0)
        BCK(&B, cudaMemcpyAsync(burst.data(), bd.state, sizeof(BurstState) * B.count,
                                cudaMemcpyDeviceToHost, B.stream));
    nf_status st = bsync(B);
    if (st) return st;
    for (int k = 0; k < B.count; k++) {
        out[k].time = sc[k].time;
        out[k].timestep = sc[k].dt;
        out[k].steps = sc[k].steps;
        out[k].status = sc[k].status;
        out[k].done = bd.every > 0 ? (burst[k].traversed ||
                                      (sc[k].steps % bd.every == 0 &&
                                       !(sc[k].time < B.inst[k].tEnd)))
                                   : !(sc[k].time < B.inst[k].tEnd);
    }
    return NF_OK;
}

nf_status nf_batch_measure(nf_batch *h, nf_measure *out) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    launch_batch_measure(B.d, B.b, B.stream);
    B.launches += 1;
    std::vector<unsigned long long> m(3LL * B.count);
    BCK(&B, cudaMemcpyAsync(m.data(), B.b.measure, 8 * m.size(), cudaMemcpyDeviceToHost, B.stream));
    nf_status st = bsync(B);
    if (st) return st;
    auto unkey = [](unsigned long long k) {
        const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
        double v;
        memcpy(&v, &u, 8);
        return v;
    };
    for (int k = 0; k < B.count; k++) {
        const bool any = B.inst[k].n1 > B.inst[k].n0;
        out[k].z_max = any ? unkey(m[3 * k]) : -INFINITY;
        out[k].z_min = any ? unkey(m[3 * k + 1]) : INFINITY;
        out[k].length = out[k].z_max - out[k].z_min;
        const double rmax = any ? unkey(m[3 * k + 2]) : 0.0;
        out[k].mushroom_diameter = 2.0 * (rmax > 0.0 ? rmax : 0.0);
    }
    return NF_OK;
}

nf_status nf_batch_wall_stats(nf_batch *h, nf_wall_info *out) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    std::vector<BatchScalars> sc(B.count);
    BCK(&B, cudaMemcpyAsync(sc.data(), B.b.sc, sizeof(BatchScalars) * B.count,
                            cudaMemcpyDeviceToHost, B.stream));
    nf_status st = bsync(B);
    if (st) return st;
    for (int k = 0; k < B.count; k++) {
        nf_wall_info &o = out[k];
        memset(&o, 0, sizeof o);
        o.present = B.inst[k].hasWall;
        o.plane = B.inst[k].wallPlane;
        o.friction = B.inst[k].wallFriction;
        o.impulse = sc[k].wImpulse;
        o.energy_loss = sc[k].wEnergyLoss;
        o.friction_dissipation = sc[k].wFriction;
        o.contact_count = sc[k].wContact;
        o.stuck_count = sc[k].wStuck;
    }
    return NF_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------ burst

extern "C" {

nf_status nf_batch_set_burst(nf_batch *h, const nf_batch_burst *config,
                             const double *mean_radius) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    if (!config || config->sample_every < 0 || config->trace_capacity < 0 ||
        !(config->margin >= 0.0 && config->margin < 1.0))
        return bfail(&B, NF_EINVAL, "burst sampling needs sample_every >= 0, trace_capacity >= 0 "
                                    "and a margin in [0, 1)");
    if (config->sample_every > 0 && !mean_radius)
        return bfail(&B, NF_EINVAL, "burst sampling needs each instance's mean radius");
    BurstDev &bd = B.b.burst;
    for (void *p : B.burstAllocs) cudaFree(p);
    B.burstAllocs.clear();
    bd = BurstDev{};
    if (B.graph) {                           // the captured launches hold the old BatchDev
        cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
    }
    if (config->sample_every == 0) return NF_OK;
    cudaError_t e = cudaSuccess;
    auto A = [&](void **p, size_t bytes) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(p, bytes ? bytes : 1);
        if (e == cudaSuccess) {
            B.burstAllocs.push_back(*p);
            e = cudaMemsetAsync(*p, 0, bytes ? bytes : 1, B.stream);
        }
    };
    double *radius = nullptr;
    A((void **)&radius, 8 * (size_t)B.count);
    A((void **)&bd.state, sizeof(BurstState) * (size_t)B.count);
    A((void **)&bd.trace, 32 * (size_t)B.count * config->trace_capacity);
    A((void **)&bd.scratch, 8 * (size_t)B.E);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(radius, mean_radius, 8 * (size_t)B.count, cudaMemcpyHostToDevice,
                            B.stream);
    if (e != cudaSuccess) {
        for (void *p : B.burstAllocs) cudaFree(p);
        B.burstAllocs.clear();
        bd = BurstDev{};
        return bfail(&B, NF_ENOMEM, "burst allocation failed: %s", cudaGetErrorString(e));
    }
    bd.meanRadius = radius;
    bd.every = config->sample_every;
    bd.traceCap = config->trace_capacity;
    bd.margin = config->margin;
    return bsync(B);
}

nf_status nf_batch_burst_results(nf_batch *h, nf_burst_result *out) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    const BurstDev &bd = B.b.burst;
    if (bd.every == 0) return bfail(&B, NF_ESTATE, "burst sampling is not set");
    std::vector<BurstState> st(B.count);
    BCK(&B, cudaMemcpyAsync(st.data(), bd.state, sizeof(BurstState) * B.count,
                            cudaMemcpyDeviceToHost, B.stream));
    nf_status s = bsync(B);
    if (s) return s;
    for (int k = 0; k < B.count; k++) {
        nf_burst_result &o = out[k];
        o.peak_capacity = st[k].peakCapacity;
        o.peak_strain = st[k].peakStrain;
        o.peak_applied = st[k].peakApplied;
        o.capacity = st[k].capacity;
        o.strain = st[k].strain;
        o.applied = st[k].applied;
        o.samples = st[k].samples;
        o.traversed = st[k].traversed;
    }
    return NF_OK;
}

nf_status nf_batch_burst_trace(nf_batch *h, double *trace) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    const BurstDev &bd = B.b.burst;
    if (bd.every == 0) return bfail(&B, NF_ESTATE, "burst sampling is not set");
    BCK(&B, cudaMemcpyAsync(trace, bd.trace, 32 * (size_t)B.count * bd.traceCap,
                            cudaMemcpyDeviceToHost, B.stream));
    return bsync(B);
}

}  // extern "C"

// ------------------------------------------------------------------------------------ adjoint

namespace {

template <typename T>
cudaError_t aalloc(Batch &B, T **p, size_t count) {
    void *v = nullptr;
    cudaError_t e = cudaMalloc(&v, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return e;
    B.adjAllocs.push_back(v);
    *p = (T *)v;
    return cudaMemsetAsync(v, 0, sizeof(T) * (count ? count : 1), B.stream);
}

}  // namespace

extern "C" {

nf_status nf_batch_adjoint_forward(nf_batch *h, int32_t checkpoint_every, int32_t sample_every) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    if (checkpoint_every < 1) return bfail(&B, NF_EINVAL, "checkpoint interval must be positive");
    if (B.mixed) return bfail(&B, NF_EINVAL, "the adjoint runs on FP64 batches");
    if (sample_every < 0) return bfail(&B, NF_EINVAL, "sampling interval must not be negative");
    std::vector<BatchScalars> sc(B.count);
    BCK(&B, cudaMemcpyAsync(sc.data(), B.b.sc, sizeof(BatchScalars) * B.count,
                            cudaMemcpyDeviceToHost, B.stream));
    nf_status st = bsync(B);
    if (st) return st;
    for (int k = 0; k < B.count; k++)
        if (sc[k].steps != 0)
            return bfail(&B, NF_ESTATE, "the adjoint's forward pass starts from a fresh batch");
    free_adjoint(B);
    BCK(&B, adjoint_reserve_stack());
    // checkpoint capacity: 8x the step count the initial CFL step predicts, plus margin
    std::vector<long long> ckptOff(B.count), finOff(B.count), tapeOff(B.count), barOff(B.count);
    std::vector<long long> seedOff(B.count), cap(B.count), bytes(B.count);
    long long ck = 0, fi = 0, ta = 0, ba = 0, se = 0;
    for (int k = 0; k < B.count; k++) {
        const BatchInst &in = B.inst[k];
        const int n = in.n1 - in.n0, e = in.e1 - in.e0;
        bytes[k] = (long long)adj_state_bytes(n, e);
        const double est = sc[k].dt > 0.0 ? 8.0 * in.tEnd / sc[k].dt : 1.0;
        cap[k] = (long long)(est / checkpoint_every) + 4;
        ckptOff[k] = ck; ck += cap[k] * bytes[k];
        finOff[k] = fi; fi += bytes[k];
        tapeOff[k] = ta; ta += (long long)checkpoint_every * bytes[k];
        barOff[k] = ba; ba += (long long)adj_bar_bytes(n, e, in.k1 - in.k0);
        seedOff[k] = se; se += (long long)adj_seed_bytes(n, e);
    }
    AdjDev &a = B.adj;
    cudaError_t e_ = cudaSuccess;
    long long *dCkptOff = nullptr, *dFinOff = nullptr, *dTapeOff = nullptr, *dBarOff = nullptr;
    long long *dCap = nullptr, *dBytes = nullptr, *dSeedOff = nullptr, *dSeedStep = nullptr;
#define A(ptr, n) if (e_ == cudaSuccess) e_ = aalloc(B, &(ptr), (n))
    A(a.ckpt, (size_t)ck); A(a.fin, (size_t)fi); A(a.peak, (size_t)fi);
    A(a.seed, (size_t)se * NF_ADJ_MAX_WIDTH);
    A(dCkptOff, B.count); A(dFinOff, B.count); A(dTapeOff, B.count); A(dBarOff, B.count);
    A(dCap, B.count); A(dBytes, B.count); A(dSeedOff, B.count);
    A(dSeedStep, (size_t)B.count * NF_ADJ_MAX_WIDTH);
    A(a.steps, B.count); A(a.peakStep, B.count); A(a.peakValue, B.count);
    A(a.grad, (size_t)B.count * NF_PARAM_COUNT * NF_ADJ_MAX_WIDTH); A(a.overflow, 1);
#undef A
    if (e_ != cudaSuccess) {
        free_adjoint(B);
        return bfail(&B, NF_ENOMEM, "adjoint allocation failed: %s", cudaGetErrorString(e_));
    }
    BCK(&B, cudaMemcpyAsync(dCkptOff, ckptOff.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dFinOff, finOff.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dTapeOff, tapeOff.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dBarOff, barOff.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dCap, cap.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dBytes, bytes.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(dSeedOff, seedOff.data(), 8 * B.count, cudaMemcpyHostToDevice, B.stream));
    a.ckptOff = dCkptOff; a.finOff = dFinOff; a.tapeOff = dTapeOff; a.barOff = dBarOff;
    a.peakOff = dFinOff; a.seedOff = dSeedOff; a.seedStep = dSeedStep;
    a.ckptCap = dCap; a.stateBytes = dBytes;
    a.every = checkpoint_every;
    a.sampleEvery = sample_every;
    a.width = 1;
    a.seedPlane = se;
    B.adjSeedBytes = se;
    B.adjSeedOff = seedOff;
    B.adjFinOff = finOff;
    B.adjStateBytes = bytes;
    // the tape and adjoint arrays are allocated by the backward pass
    a.tape = nullptr;
    a.bar = nullptr;
    B.adjTapeBytes = ta;
    B.adjBarBytes = ba;
    a.barPlane = ba;
    B.adjBarOff = barOff;
    BCK(&B, cudaEventRecord(B.ev0, B.stream));
    launch_adjoint_forward(B.d, B.b, a, B.stream);
    B.launches += 1;
    BCK(&B, cudaEventRecord(B.ev1, B.stream));
    st = bsync(B);
    if (st) return st;
    int overflow = 0;
    BCK(&B, cudaMemcpy(&overflow, a.overflow, sizeof overflow, cudaMemcpyDeviceToHost));
    if (overflow) {
        free_adjoint(B);
        return bfail(&B, NF_ESTATE, "an instance took more steps than its checkpoint capacity");
    }
    float ms = 0.0f;
    BCK(&B, cudaEventElapsedTime(&ms, B.ev0, B.ev1));
    B.adjForwardMs = ms;
    B.adjForward = true;
    return NF_OK;
}

static bool sampled(long long peakStep) { return peakStep > 0; }

// The objective of instance k and its seed in one plane of the seed buffer: the adjoint of
// the displacements (and, for the capacity, of the hoop stress) after step *seedStep, the
// final step or the sampled peak.
static nf_status adjoint_seed(Batch &B, int32_t objective, int k,
                              const std::vector<double2> &X0, const std::vector<int32_t> &conn,
                              const std::vector<long long> &steps,
                              const std::vector<long long> &peakStep, char *plane,
                              double *value, long long *seedStep) {
    const AdjDev &a = B.adj;
    const bool finite = B.d.finite != 0;
    const BatchInst &in = B.inst[k];
    const int n = in.n1 - in.n0, e = in.e1 - in.e0;
    // the state the objective is read from: the final or the peak block (U and sig)
    const long long blk = B.adjFinOff[k];
    const char *src = objective == NF_OBJECTIVE_PEAK_CAPACITY ? a.peak : a.fin;
    std::vector<double2> U(n);
    std::vector<double> sig(4 * (size_t)e);
    BCK(&B, cudaMemcpy(U.data(), src + blk, 16 * (size_t)n, cudaMemcpyDeviceToHost));
    BCK(&B, cudaMemcpy(sig.data(), src + blk + 3 * ((16 * (size_t)n + 15) & ~(size_t)15),
                       32 * (size_t)e, cudaMemcpyDeviceToHost));
    double2 *su = reinterpret_cast<double2 *>(plane + B.adjSeedOff[k]);
    double *ss = reinterpret_cast<double *>(plane + B.adjSeedOff[k]
                                            + ((16 * (size_t)n + 15) & ~(size_t)15));
    auto R_ = [&](int i) { return finite ? X0[in.n0 + i].x + U[i].x : X0[in.n0 + i].x; };
    auto Z_ = [&](int i) { return finite ? X0[in.n0 + i].y + U[i].y : X0[in.n0 + i].y; };
    if (objective == NF_OBJECTIVE_PEAK_CAPACITY) {
        if (!(sampled(peakStep[k])))
            return bfail(&B, NF_ESTATE, "instance %d: no capacity was sampled in the forward "
                                        "pass (sample_every 0 or no sample before t_end)", k);
        *seedStep = peakStep[k];
        // BurstCase.loadCapacity (BurstCase.java:533-553) and its derivatives
        double hoop = 0.0;
        for (int j = 0; j < e; j++) {
            double sum = 0.0;
            for (int c = 0; c < 4; c++) {
                const int p = conn[4 * (size_t)(in.e0 + j) + c] - in.n0;
                const int q = conn[4 * (size_t)(in.e0 + j) + (c + 1) % 4] - in.n0;
                sum += R_(p) * Z_(q) - R_(q) * Z_(p);
            }
            hoop += sig[4 * (size_t)j + 2] * (0.5 * sum);
        }
        double bore = DBL_MAX, low = DBL_MAX, high = -DBL_MAX;
        int ib = 0, il = 0, ih = 0;
        for (int i = 0; i < n; i++) {
            if (R_(i) < bore) { bore = R_(i); ib = i; }
            if (Z_(i) < low) { low = Z_(i); il = i; }
            if (Z_(i) > high) { high = Z_(i); ih = i; }
        }
        const double den = bore * (high - low);
        const double capv = hoop / den;
        *value = capv;
        for (int j = 0; j < e; j++) {
            double r[4], z[4];
            int nn[4];
            for (int c = 0; c < 4; c++) {
                nn[c] = conn[4 * (size_t)(in.e0 + j) + c] - in.n0;
                r[c] = R_(nn[c]);
                z[c] = Z_(nn[c]);
            }
            double sum = 0.0;
            for (int c = 0; c < 4; c++) sum += r[c] * z[(c + 1) & 3] - r[(c + 1) & 3] * z[c];
            ss[4 * (size_t)j + 2] += 0.5 * sum / den;
            if (finite) {
                const double w = sig[4 * (size_t)j + 2] / den;
                for (int c = 0; c < 4; c++) {
                    su[nn[c]].x += w * 0.5 * (z[(c + 1) & 3] - z[(c + 3) & 3]);
                    su[nn[c]].y += w * 0.5 * (r[(c + 3) & 3] - r[(c + 1) & 3]);
                }
            }
        }
        if (finite) {
            su[ib].x -= capv / bore;
            su[ih].y -= capv / (high - low);
            su[il].y += capv / (high - low);
        }
        return NF_OK;
    }
    *seedStep = steps[k];
    double zmax = -DBL_MAX, zmin = DBL_MAX, z0max = -DBL_MAX, z0min = DBL_MAX, rmax = -DBL_MAX;
    int imax = 0, imin = 0, irmax = 0;
    for (int i = 0; i < n; i++) {
        const double z = X0[in.n0 + i].y + U[i].y, r = X0[in.n0 + i].x + U[i].x;
        if (z > zmax) { zmax = z; imax = i; }
        if (z < zmin) { zmin = z; imin = i; }
        if (r > rmax) { rmax = r; irmax = i; }
        if (X0[in.n0 + i].y > z0max) z0max = X0[in.n0 + i].y;
        if (X0[in.n0 + i].y < z0min) z0min = X0[in.n0 + i].y;
    }
    if (objective == NF_OBJECTIVE_LENGTH_RATIO) {
        const double L0 = z0max - z0min;
        su[imax].y += 1.0 / L0;
        su[imin].y -= 1.0 / L0;
        *value = (zmax - zmin) / L0;
    } else {
        su[irmax].x += 2.0;
        *value = 2.0 * rmax;
    }
    return NF_OK;
}

nf_status nf_batch_adjoint_backward_many(nf_batch *h, const int32_t *objectives, int32_t count,
                                         double *values, double *gradients) {
    Batch &B = *reinterpret_cast<Batch *>(h);
    if (!B.adjForward) return bfail(&B, NF_ESTATE, "run the adjoint's forward pass first");
    if (count < 1 || count > NF_ADJ_MAX_WIDTH)
        return bfail(&B, NF_EINVAL, "1 to %d objectives per backward pass, not %d",
                     NF_ADJ_MAX_WIDTH, count);
    for (int w = 0; w < count; w++)
        if (objectives[w] != NF_OBJECTIVE_LENGTH_RATIO && objectives[w] != NF_OBJECTIVE_MUSHROOM &&
            objectives[w] != NF_OBJECTIVE_PEAK_CAPACITY)
            return bfail(&B, NF_EINVAL, "unknown objective %d", objectives[w]);
    AdjDev &a = B.adj;
    cudaError_t e_ = cudaSuccess;
    if (!a.tape) {
        e_ = aalloc(B, &a.tape, (size_t)B.adjTapeBytes);
        if (e_ == cudaSuccess)
            e_ = aalloc(B, &a.bar, (size_t)B.adjBarBytes * NF_ADJ_MAX_WIDTH);
        if (e_ != cudaSuccess) return bfail(&B, NF_ENOMEM, "adjoint allocation failed: %s",
                                            cudaGetErrorString(e_));
    }
    std::vector<double2> X0(B.N);
    BCK(&B, cudaMemcpy(X0.data(), B.d.X0, 16 * (size_t)B.N, cudaMemcpyDeviceToHost));
    std::vector<long long> steps(B.count), peakStep(B.count);
    std::vector<long long> seedStep((size_t)B.count * count);
    BCK(&B, cudaMemcpy(steps.data(), a.steps, 8 * B.count, cudaMemcpyDeviceToHost));
    BCK(&B, cudaMemcpy(peakStep.data(), a.peakStep, 8 * B.count, cudaMemcpyDeviceToHost));
    std::vector<int32_t> conn(4 * (size_t)B.E);
    BCK(&B, cudaMemcpy(conn.data(), B.d.conn, 16 * (size_t)B.E, cudaMemcpyDeviceToHost));
    std::vector<char> seed((size_t)B.adjSeedBytes * count, 0);
    for (int w = 0; w < count; w++)
        for (int k = 0; k < B.count; k++) {
            const nf_status st = adjoint_seed(B, objectives[w], k, X0, conn, steps, peakStep,
                                              seed.data() + (size_t)w * B.adjSeedBytes,
                                              &values[(size_t)w * B.count + k],
                                              &seedStep[(size_t)w * B.count + k]);
            if (st) return st;
        }
    BCK(&B, cudaMemcpyAsync(a.seed, seed.data(), seed.size(), cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemcpyAsync(const_cast<long long *>(a.seedStep), seedStep.data(),
                            8 * seedStep.size(), cudaMemcpyHostToDevice, B.stream));
    BCK(&B, cudaMemsetAsync(a.bar, 0, (size_t)B.adjBarBytes * count, B.stream));
    a.width = count;
    BCK(&B, cudaEventRecord(B.ev0, B.stream));
    launch_adjoint_backward(B.d, B.b, a, B.stream);
    B.launches += 1;
    BCK(&B, cudaEventRecord(B.ev1, B.stream));
    nf_status st = bsync(B);
    if (st) return st;
    float ms = 0.0f;
    BCK(&B, cudaEventElapsedTime(&ms, B.ev0, B.ev1));
    B.adjBackwardMs = ms;
    BCK(&B, cudaMemcpy(gradients, a.grad, sizeof(double) * NF_PARAM_COUNT * B.count * count,
                       cudaMemcpyDeviceToHost));
    return NF_OK;
}

nf_status nf_batch_adjoint_backward(nf_batch *h, int32_t objective, double *values,
                                    double *gradients) {
    return nf_batch_adjoint_backward_many(h, &objective, 1, values, gradients);
}

nf_status nf_batch_adjoint_elapsed(nf_batch *h, double *forward_ms, double *backward_ms) {
    const Batch &B = *reinterpret_cast<Batch *>(h);
    *forward_ms = B.adjForwardMs;
    *backward_ms = B.adjBackwardMs;
    return NF_OK;
}

}  // extern "C"
