// api.cu -- the C ABI of include/neofiz.h: handle lifecycle, set-up, run, read-back.
//
// Set-up arithmetic that the reference performs once (per-element material constants, lumped
// mass, node slots, the initial CFL step; ExplicitSolver.java:264-366, :1559-1597) runs here on
// the host in the reference's evaluation order (this file is compiled with
// -ffp-contract=off), and everything it produces is copied to the device once. After that a
// step is a fixed sequence of kernel launches on the handle's stream.
#include "nf_internal.h"

#include <algorithm>
#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <utility>

using namespace nf;

namespace {

thread_local std::string g_err;

nf_status failv(Solver *S, nf_status st, const char *fmt, va_list ap) {
    char buf[768];
    vsnprintf(buf, sizeof buf, fmt, ap);
    if (S) S->err = buf; else g_err = buf;
    return st;
}
nf_status fail(Solver *S, nf_status st, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    nf_status r = failv(S, st, fmt, ap);
    va_end(ap);
    return r;
}

#define CK(S, call)                                                                    \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail((S), NF_EDEVICE, "%s: %s", #call, cudaGetErrorString(e_));       \
    } while (0)

struct Allocs {
    std::vector<void *> ptrs;
};

template <typename T>
cudaError_t dalloc(Solver &S, T **p, size_t count) {
    void *v = nullptr;
    const size_t bytes = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc(&v, bytes);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(v, 0, bytes, S.stream);
    *p = (T *)v;
    return e;
}

// The set-up arrays of nf_create carved from one allocation: one cudaMalloc and one memset
// instead of one each per array (the allocations dominated creating a 200k-element scene).
struct Arena {
    std::vector<std::pair<void **, size_t>> items;
    template <typename T>
    void add(T **p, size_t count) {
        items.push_back({reinterpret_cast<void **>(p), sizeof(T) * (count ? count : 1)});
    }
    cudaError_t commit(Solver &S) {
        size_t total = 0;
        for (auto &it : items) total += (it.second + 255) & ~(size_t)255;
        void *base = nullptr;
        cudaError_t e = cudaMalloc(&base, total);
        if (e != cudaSuccess) return e;
        S.arena = base;
        S.arenaBytes = total;
        char *p = static_cast<char *>(base);
        for (auto &it : items) {
            *it.first = p;
            p += (it.second + 255) & ~(size_t)255;
        }
        return cudaMemsetAsync(base, 0, total, S.stream);
    }
};

template <typename T>
cudaError_t upload(Solver &S, T *dst, const T *src, size_t count) {
    if (!count) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, S.stream);
}

double mat_lambda(const nf_material &m) {                     // Material.java:93-95
    return m.youngs_modulus * m.poisson_ratio
           / ((1.0 + m.poisson_ratio) * (1.0 - 2.0 * m.poisson_ratio));
}
double mat_mu(const nf_material &m) {                         // Material.java:98-100
    return m.youngs_modulus / (2.0 * (1.0 + m.poisson_ratio));
}
double mat_wave(const nf_material &m) {                       // Material.java:106-108
    return sqrt((mat_lambda(m) + 2.0 * mat_mu(m)) / m.density);
}

const char *material_invalid(const nf_material &m) {          // Material.java:23-39
    if (m.youngs_modulus <= 0) return "E must be positive";
    if (m.poisson_ratio <= -1.0 || m.poisson_ratio >= 0.5) return "nu must lie in (-1, 0.5)";
    if (m.density <= 0) return "density must be positive";
    if (m.yield_stress <= 0) return "yield stress must be positive";
    if (m.isotropic_hardening < 0 || m.kinematic_hardening < 0)
        return "hardening moduli must be non-negative";
    if (m.has_johnson_cook) {                                 // JohnsonCook.java:71-89
        if (m.jc_a <= 0) return "A must be positive";
        if (m.jc_b < 0) return "B must be non-negative";
        if (m.jc_n <= 0 || m.jc_n > 1) return "n must lie in (0, 1]";
        if (m.jc_c < 0) return "C must be non-negative";
        if (m.jc_m <= 0) return "m must be positive";
        if (m.jc_reference_strain_rate <= 0) return "reference strain rate must be positive";
        if (m.jc_melt_temperature <= m.jc_room_temperature)
            return "melt temperature must exceed room temperature";
        if (m.jc_specific_heat <= 0) return "specific heat must be positive";
        if (m.jc_taylor_quinney < 0 || m.jc_taylor_quinney > 1)
            return "Taylor-Quinney fraction must lie in [0, 1]";
        if (m.yield_stress != m.jc_a) return "yield stress disagrees with the Johnson-Cook A";
    }
    return nullptr;
}

MatDev mat_dev(const nf_material &m, int formulation) {       // ExplicitSolver.java:289-299
    MatDev o{};
    const double lam = formulation == NF_PLANE_STRESS
                       ? 2.0 * mat_lambda(m) * mat_mu(m) / (mat_lambda(m) + 2.0 * mat_mu(m))
                       : mat_lambda(m);
    o.lambda = lam;
    o.mu = mat_mu(m);
    o.bulk = lam + 2.0 * mat_mu(m) / 3.0;
    o.density = m.density;
    o.youngs = m.youngs_modulus;
    o.sy0 = m.yield_stress;
    o.hIso = m.isotropic_hardening;
    o.hKin = m.kinematic_hardening;
    o.jc = m.has_johnson_cook ? 1 : 0;
    if (o.jc) {
        o.a = m.jc_a; o.b = m.jc_b; o.n = m.jc_n; o.c = m.jc_c; o.m = m.jc_m;
        o.refRate = m.jc_reference_strain_rate;
        o.room = m.jc_room_temperature;
        o.melt = m.jc_melt_temperature;
        o.cp = m.jc_specific_heat;
        o.tq = m.jc_taylor_quinney;
        o.thermalCoefficient = o.tq / (m.density * o.cp);   // JohnsonCook.java:224-226
    }
    return o;
}

double signed_area(const double *r, const double *z, const int32_t *conn, int e) {
    const int b = e * 4;
    double a = 0.0;
    for (int k = 0; k < 4; k++) {
        const int i = conn[b + k], j = conn[b + (k + 1) % 4];
        a += r[i] * z[j] - r[j] * z[i];
    }
    return 0.5 * a;
}

__global__ void k_or_flag(uint8_t *flags, int node, uint8_t bit) { flags[node] |= bit; }
__global__ void k_or_all(uint8_t *flags, int n, uint8_t bit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] |= bit;
}
__global__ void k_set_velocity(double2 *V, int node, double vr, double vz) {
    V[node] = make_double2(vr, vz);
}
__global__ void k_uniform_velocity(double2 *V, int n, double vr, double vz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) V[i] = make_double2(vr, vz);
}
__global__ void k_scale_mass(double *mass, double *invMass, int n, double factor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        mass[i] *= factor;
        invMass[i] = 1.0 / mass[i];
    }
}
// The bounds of a run; the next step's run predicate follows from them (each step's end sets
// it for the step after).
__global__ void k_set_run(DevScalars *s, double tEnd, long long maxSteps) {
    s->tEnd = tEnd;
    s->maxSteps = maxSteps;
    s->stepsTaken = 0;
    s->active = s->time < tEnd && 0 < maxSteps ? 1 : 0;
}

nf_status sync_check(Solver &S) {
    CK(&S, cudaStreamSynchronize(S.stream));
    CK(&S, cudaGetLastError());
    return NF_OK;
}

nf_status read_scalars(Solver &S, DevScalars *out) {
    CK(&S, cudaMemcpyAsync(out, S.d.s, sizeof(DevScalars), cudaMemcpyDeviceToHost, S.stream));
    return sync_check(S);
}

nf_status ensure_mixed_damage(Solver &S) {
    Dev &d = S.d;
    if (d.dStrF) return NF_OK;
    const size_t P = (size_t)S.E * S.ppe;
    cudaError_t e_ = cudaSuccess;
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dStrF, P);
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dSoftF, P);
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dWidthF, P);
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dFailF, S.E);
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dGfF, S.E);
    if (e_ == cudaSuccess) e_ = dalloc(S, &d.dGeomF, 5 * (size_t)S.E);
    if (e_ != cudaSuccess)
        return fail(&S, NF_ENOMEM, "mixed-precision damage allocation failed: %s", cudaGetErrorString(e_));
    return NF_OK;
}

// lumpMass, ExplicitSolver.java:1559-1597: 2x2 Gauss lumping, in the reference's order.
// emat may be NULL (every element material 0).
void lumped_mass(const double *r, const double *z, const int32_t *conn, int E,
                 const nf_material *materials, const int32_t *emat, bool axi, double thickness,
                 double *mass) {
    const double G = 0.5773502691896258;
    const double gx[4] = {-G, G, G, -G}, ge[4] = {-G, -G, G, G};
    for (int e = 0; e < E; e++) {
        const double rho = materials[emat ? emat[e] : 0].density;
        const int b = e * 4;
        const int n0 = conn[b], n1 = conn[b + 1], n2 = conn[b + 2], n3 = conn[b + 3];
        const double r0 = r[n0], r1 = r[n1], r2 = r[n2], r3 = r[n3];
        const double z0 = z[n0], z1 = z[n1], z2 = z[n2], z3 = z[n3];
        for (int g = 0; g < 4; g++) {
            const double xi = gx[g], eta = ge[g];
            const double xm = 1.0 - xi, xp = 1.0 + xi;
            const double em = 1.0 - eta, ep = 1.0 + eta;
            const double N0 = 0.25 * xm * em, N1 = 0.25 * xp * em;
            const double N2 = 0.25 * xp * ep, N3 = 0.25 * xm * ep;
            const double dN0x = -0.25 * em, dN1x = 0.25 * em, dN2x = 0.25 * ep, dN3x = -0.25 * ep;
            const double dN0e = -0.25 * xm, dN1e = -0.25 * xp, dN2e = 0.25 * xp, dN3e = 0.25 * xm;
            const double J00 = dN0x * r0 + dN1x * r1 + dN2x * r2 + dN3x * r3;
            const double J01 = dN0x * z0 + dN1x * z1 + dN2x * z2 + dN3x * z3;
            const double J10 = dN0e * r0 + dN1e * r1 + dN2e * r2 + dN3e * r3;
            const double J11 = dN0e * z0 + dN1e * z1 + dN2e * z2 + dN3e * z3;
            const double det = J00 * J11 - J01 * J10;
            const double rg = N0 * r0 + N1 * r1 + N2 * r2 + N3 * r3;
            const double dV = axi ? 2.0 * NF_PI * rg * det : thickness * det;
            mass[n0] += rho * N0 * dV;
            mass[n1] += rho * N1 * dV;
            mass[n2] += rho * N2 * dV;
            mass[n3] += rho * N3 * dV;
        }
    }
}

// buildNodeSlots, ExplicitSolver.java:347-366: per node its sources (element 8 e + corner,
// then pressure-edge slots) in ascending order. slotStart has N + 1 entries, zeroed.
void node_slots(const int32_t *conn, int N, int E, const int32_t *pedges, int K,
                int32_t *slotStart, int32_t *slots) {
    for (long long k = 0; k < 4LL * E; k++) slotStart[conn[k] + 1]++;
    for (long long k = 0; k < 2LL * K; k++) slotStart[pedges[k] + 1]++;
    for (int i = 0; i < N; i++) slotStart[i + 1] += slotStart[i];
    std::vector<int32_t> cursor(slotStart, slotStart + N + 1);
    for (int e = 0; e < E; e++)
        for (int c = 0; c < 4; c++) slots[cursor[conn[e * 4 + c]]++] = e * 8 + c;
    for (int k = 0; k < 2 * K; k += 2) {
        const int slot = (E + k / 2) * 8;
        slots[cursor[pedges[k]]++] = slot;
        slots[cursor[pedges[k + 1]]++] = slot + 1;
    }
}

// QuadMesh.minimumEdgeLength: the shortest element edge of the reference configuration.
double min_edge_length(const double *r, const double *z, const int32_t *conn, int E) {
    double edge = DBL_MAX;
    for (int e = 0; e < E; e++)
        for (int k = 0; k < 4; k++) {
            const int i = conn[e * 4 + k], j = conn[e * 4 + (k + 1) % 4];
            const double dr = r[j] - r[i], dz = z[j] - z[i];
            const double len = sqrt(dr * dr + dz * dz);
            if (len < edge) edge = len;
        }
    return edge;
}

// The FP32 copy of a material's constants (the mixed form).
MatF mat_float(const MatDev &a) {
    MatF o{};
    o.lambda = (float)a.lambda; o.mu = (float)a.mu; o.bulk = (float)a.bulk;
    o.density = (float)a.density; o.youngs = (float)a.youngs;
    o.sy0 = (float)a.sy0; o.hIso = (float)a.hIso; o.hKin = (float)a.hKin;
    o.a = (float)a.a; o.b = (float)a.b; o.n = (float)a.n; o.c = (float)a.c;
    o.m = (float)a.m; o.refRate = (float)a.refRate; o.room = (float)a.room;
    o.melt = (float)a.melt; o.cp = (float)a.cp; o.tq = (float)a.tq;
    o.thermalCoefficient = (float)a.thermalCoefficient;
    o.jc = a.jc;
    return o;
}

// In mixed precision the FP64 element arrays are a staging copy: brought up to date before
// anything reads them (audits, field reads).
void mixed_to_double(Solver &S) {
    if (S.d.mixed) launch_convert_state(S, false, 3);
}

}  // namespace

extern "C" {

int nf_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

const char *nf_last_error(const nf_solver *h) {
    const Solver *S = reinterpret_cast<const Solver *>(h);
    return S ? S->err.c_str() : g_err.c_str();
}

nf_status nf_create(const nf_mesh *mesh, const nf_material *materials, int32_t material_count,
                    const int32_t *element_material, int32_t formulation, int32_t integration,
                    int32_t kinematics, double thickness, double cfl_safety, nf_solver **out) {
    *out = nullptr;
    if (!mesh || !materials || material_count < 1)
        return fail(nullptr, NF_EINVAL, "mesh and at least one material are required");
    if (mesh->node_count < 0 || mesh->element_count < 0 || mesh->pressure_edge_count < 0)
        return fail(nullptr, NF_EINVAL, "negative mesh size");
    if (formulation < 0 || formulation > 2 || integration < 0 || integration > 1 ||
        kinematics < 0 || kinematics > 1)
        return fail(nullptr, NF_EINVAL, "unknown formulation, integration or kinematics");
    for (int m = 0; m < material_count; m++) {
        const char *why = material_invalid(materials[m]);
        if (why) return fail(nullptr, NF_EINVAL, "%s", why);
        if (formulation == NF_PLANE_STRESS && !std::isinf(materials[m].yield_stress))
            return fail(nullptr, NF_EINVAL,
                        "plane stress plasticity needs its own return map; not implemented");
    }
    const int N = mesh->node_count, E = mesh->element_count, K = mesh->pressure_edge_count;
    for (long long k = 0; k < 4LL * E; k++)
        if (mesh->conn[k] < 0 || mesh->conn[k] >= N)
            return fail(nullptr, NF_EINVAL, "connectivity refers to node %d of %d", mesh->conn[k], N);
    for (long long k = 0; k < 2LL * K; k++)
        if (mesh->pressure_edges[k] < 0 || mesh->pressure_edges[k] >= N)
            return fail(nullptr, NF_EINVAL, "pressure edge refers to node %d of %d",
                        mesh->pressure_edges[k], N);
    if (element_material)
        for (int e = 0; e < E; e++)
            if (element_material[e] < 0 || element_material[e] >= material_count)
                return fail(nullptr, NF_EINVAL, "element %d has no material", e);
    for (int e = 0; e < E; e++)                                    // QuadMesh.java:228-237
        if (signed_area(mesh->r, mesh->z, mesh->conn, e) <= 0.0)
            return fail(nullptr, NF_ESTATE,
                        "element %d has non-positive area; node ordering must be "
                        "counter-clockwise in (r, z)", e);
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1)
        return fail(nullptr, NF_EDEVICE, "no CUDA device is visible");

    Solver *S = new Solver();
    Dev &d = S->d;
    CK(nullptr, cudaGetDevice(&S->device));
    CK(nullptr, cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    S->ownStream = S->stream;
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->device);
        S->d.sms = sms > 0 ? sms : 1;
        S->d.coopBlocks = contact_coop_blocks(S->d.sms);
    }
    S->N = N; S->E = E; S->K = K;
    S->formulation = formulation; S->integration = integration; S->kinematics = kinematics;
    S->ppe = integration == NF_FULL ? 4 : 1;
    S->materials.assign(materials, materials + material_count);
    S->emat.assign(E, 0);
    if (element_material) std::copy(element_material, element_material + E, S->emat.begin());
    S->hostR.assign(mesh->r, mesh->r + N);
    S->hostZ.assign(mesh->z, mesh->z + N);
    S->hostConn.assign(mesh->conn, mesh->conn + 4LL * E);

    d.N = N; d.E = E; d.K = K; d.ppe = S->ppe;
    d.axi = formulation == NF_AXISYMMETRIC;
    d.finite = kinematics == NF_FINITE_STRAIN;
    d.full = integration == NF_FULL;
    d.thickness = thickness;
    d.cfl = cfl_safety;
    d.massScale = 1.0;
    d.hourglass = 0.05;                                        // ExplicitSolver.java:59
    d.erosionDamage = INFINITY;
    d.cScale = 0.1;
    d.cSqrtScale = std::sqrt(0.1);
    d.nmat = material_count;

    // per-material constants and the fastest wave (Materials.java:118-127)
    std::vector<MatDev> mats(material_count);
    for (int m = 0; m < material_count; m++) mats[m] = mat_dev(materials[m], formulation);
    if (!element_material || material_count == 1) {
        d.fastestWave = mat_wave(materials[0]);
    } else {
        double fastest = 0.0;
        for (int e = 0; e < E; e++) {
            const double c = mat_wave(materials[S->emat[e]]);
            if (c > fastest) fastest = c;
        }
        d.fastestWave = fastest;
    }

    // lumped mass, ExplicitSolver.java:1559-1597
    std::vector<double> mass(N, 0.0);
    lumped_mass(mesh->r, mesh->z, mesh->conn, E, materials, S->emat.data(), d.axi != 0, thickness,
                mass.data());

    // node slots, ExplicitSolver.java:347-366
    std::vector<int32_t> slotStart(N + 1, 0), slots(4LL * E + 2LL * K);
    node_slots(mesh->conn, N, E, mesh->pressure_edges, K, slotStart.data(), slots.data());

    // initial step, QuadMesh.minimumEdgeLength + ExplicitSolver.java:333-338
    const double edge = min_edge_length(mesh->r, mesh->z, mesh->conn, E);
    DevScalars s0{};
    s0.minEdgeSquared = edge * edge;
    s0.dt = cfl_safety * edge / d.fastestWave;
    s0.dtPrevious = s0.dt;
    s0.minEdgeBits = 0x7fefffffffffffffULL;   // Double.MAX_VALUE
    s0.tEnd = INFINITY;
    d.dt0 = s0.dt;

    // edge groups for the free surface: element-edges with the same undirected node pair, in
    // (lower node, higher node, element-edge) order -- a counting sort by the lower node (stable
    // in element-edge order) and an insertion sort by the higher node within each node's few
    // edges, linear in the mesh where a comparison sort of the 4E keys is not
    std::vector<std::pair<long long, int>> keys(4LL * E);
    {
        std::vector<int32_t> start(N + 1, 0);
        for (long long q = 0; q < 4LL * E; q++) {
            const int a = mesh->conn[q], b = mesh->conn[(q & ~3LL) + ((q + 1) & 3)];
            start[std::min(a, b) + 1]++;
        }
        for (int i = 0; i < N; i++) start[i + 1] += start[i];
        std::vector<int32_t> cursor(start.begin(), start.end() - 1);
        for (long long q = 0; q < 4LL * E; q++) {
            const int a = mesh->conn[q], b = mesh->conn[(q & ~3LL) + ((q + 1) & 3)];
            const long long lo = std::min(a, b), hi = std::max(a, b);
            keys[cursor[lo]++] = std::make_pair((lo << 32) | hi, (int)q);
        }
        for (int i = 0; i < N; i++)
            for (int j = start[i] + 1; j < start[i + 1]; j++)
                for (int m = j; m > start[i] && keys[m] < keys[m - 1]; m--)
                    std::swap(keys[m], keys[m - 1]);
    }
    std::vector<int32_t> edgeGroup(4LL * E), groupStart, groupMember(4LL * E);
    for (size_t i = 0; i < keys.size();) {
        size_t j = i;
        const int g = (int)groupStart.size();
        groupStart.push_back((int)i);
        while (j < keys.size() && keys[j].first == keys[i].first) {
            edgeGroup[keys[j].second] = g;
            groupMember[j] = keys[j].second;
            j++;
        }
        i = j;
    }
    groupStart.push_back((int)keys.size());

    // device allocations
    const size_t P = (size_t)E * S->ppe;
    std::vector<double2> X0(N), zero2(N);
    for (int i = 0; i < N; i++) X0[i] = make_double2(mesh->r[i], mesh->z[i]);
    std::vector<int4> conn4(E);
    for (int e = 0; e < E; e++)
        conn4[e] = make_int4(mesh->conn[4 * e], mesh->conn[4 * e + 1], mesh->conn[4 * e + 2],
                             mesh->conn[4 * e + 3]);
    std::vector<int2> pe(K);
    for (int k = 0; k < K; k++)
        pe[k] = make_int2(mesh->pressure_edges[2 * k], mesh->pressure_edges[2 * k + 1]);
    // the Johnson-Cook work list of the FP64 one-point element pass
    bool anyJC = false;
    for (int m = 0; m < material_count; m++) anyJC = anyJC || mats[m].jc != 0;
    const bool listed = anyJC && !d.full && E > 0;
    if (listed) d.hotCap = std::max(1024, (E / 4 + 127) & ~127);
    // partial-sum slots: the per-item grids (nodes, elements, the listed element pass, which
    // also erodes) and the fixed contact grid
    d.maxBlocks = std::max(std::max(grid_for(std::max(std::max(N, E), 1), 128),
                                    listed ? grid_for((long long)E + d.hotCap, 128) : 0),
                           std::max(d.coopBlocks, 8 * d.sms)) + 1;
    d.bucketCap = std::max(1 << 14, 2 * N);
    const size_t scanInts = scan_tmp_ints(std::max(std::max(4 * E, N + 1), d.bucketCap + 1)) + 16;
    Arena arena;
#define A(ptr, n) arena.add(&(ptr), (n))
    A(d.X0, N); A(d.U, N); A(d.V, N); A(d.F, N); A(d.mass, N); A(d.invMass, N);
    A(d.flags, N); A(d.wallState, N); A(d.contactState, N);
    A(d.conn, E); A(d.emat, E); A(d.mats, material_count);
    A(d.sig, 4 * P); A(d.back, 4 * P); A(d.epsP, P); A(d.wP, P);
    A(d.hg, E); A(d.hgK, E);
    A(d.contribution, 8 * ((size_t)E + K));
    A(d.nodeSlotStart, N + 1); A(d.nodeSlot, 4LL * E + 2LL * K);
    A(d.pedges, K);
    A(d.partials, (size_t)PARTIAL_SLOTS * d.maxBlocks);
    A(d.edgeGroup, 4LL * E); A(d.groupStart, groupStart.size()); A(d.groupMember, 4LL * E);
    A(d.s, 1);
    if (listed) {
        d.hotSmem = listed_pass_smem(S->device);
        A(d.hot, 1); A(d.hotList, d.hotCap); A(d.hotNext, d.hotCap); A(d.hotStamp, E);
        A(d.jcYield, E);
    }
#undef A
    const cudaError_t e_ = arena.commit(*S);
    if (e_ != cudaSuccess) {
        nf_status st = fail(nullptr, NF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(e_));
        nf_destroy(reinterpret_cast<nf_solver *>(S));
        return st;
    }
    upload(*S, d.X0, X0.data(), N);
    upload(*S, d.mass, mass.data(), N);
    std::vector<double> invMass(N);
    for (int i = 0; i < N; i++) invMass[i] = 1.0 / mass[i];     // nodalUpdate's 1/m, once
    upload(*S, d.invMass, invMass.data(), N);
    upload(*S, d.conn, conn4.data(), E);
    upload(*S, d.emat, S->emat.data(), E);
    upload(*S, d.mats, mats.data(), material_count);
    upload(*S, d.nodeSlotStart, slotStart.data(), N + 1);
    upload(*S, d.nodeSlot, slots.data(), slots.size());
    upload(*S, d.pedges, pe.data(), K);
    upload(*S, d.edgeGroup, edgeGroup.data(), edgeGroup.size());
    upload(*S, d.groupStart, groupStart.data(), groupStart.size());
    upload(*S, d.groupMember, groupMember.data(), groupMember.size());
    upload(*S, d.s, &s0, 1);
    if (d.hot) {
        HotList h0{};                          // listing stamps start at 0: nothing listed
        h0.epoch = 1;
        upload(*S, d.hot, &h0, 1);
    }
    if (d.jcYield) launch_jc_yield(d, S->stream);
    d.scanTmpSize = (int)scanInts;
    d.scanTmp = nullptr;
    nf_status st = sync_check(*S);
    if (st) {
        g_err = S->err;
        nf_destroy(reinterpret_cast<nf_solver *>(S));
        return st;
    }
    *out = reinterpret_cast<nf_solver *>(S);
    return NF_OK;
}

nf_status nf_destroy(nf_solver *h) {
    Solver *S = reinterpret_cast<Solver *>(h);
    if (!S) return NF_OK;
    if (S->stream) cudaStreamSynchronize(S->stream);
    if (S->graph1) cudaGraphExecDestroy(S->graph1);
    if (S->graph16) cudaGraphExecDestroy(S->graph16);
    for (auto &r : S->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    Dev &d = S->d;
    void *ptrs[] = {d.X0, d.U, d.V, d.F, d.mass, d.invMass, d.flags, d.wallState, d.contactState, d.conn,
                    d.emat, d.mats, d.sig, d.back, d.epsP, d.wP, d.hg, d.hgK, d.gone, d.dead,
                    d.dFail, d.dGf, d.dGeom, d.dStrength, d.dSoft, d.dWidth, d.contribution,
                    d.nodeSlotStart, d.nodeSlot, d.pedges, d.partials, d.edgeGroup, d.groupStart,
                    d.groupMember, d.surfFlag, d.segA, d.segB, d.edgeList, d.edgePos, d.nodeList,
                    d.nodePos, d.nodeFree, d.nodeSeg, d.edgeStamp, d.nodeStamp, d.touched,
                    d.newDead, d.cr, d.cz, d.snr, d.snz, d.slen, d.pnr, d.pnz, d.lastMaster,
                    d.master, d.dropped, d.bucketCount, d.bucketStart, d.bucketCursor,
                    d.bucketEntry, d.bucketCell, d.entryCell, d.pairNodes, d.pairVal,
                    d.pairEnergy, d.pairDiss, d.incCount, d.incStart, d.incCursor, d.incEntry,
                    d.scanTmp, d.s, d.matsF, d.sigF, d.backF, d.epsPF, d.wPF, d.hgKF,
                    d.contribF, d.hgF, d.dStrF, d.dSoftF, d.dWidthF, d.dFailF, d.dGfF, d.dGeomF,
                    d.pMid, d.pCur, d.vdt, d.gaussVol, d.coopSums, d.incSlots, d.bucketF, d.bucketFL, d.bucketAB, d.bucketA, d.bucketN, d.bucketL,
                    d.fastCount, d.fastEntry, d.fastF, d.fastFL, d.fastAB, d.fastA, d.fastN,
                    d.fastL, d.nodeCell,
                    d.hot, d.hotList, d.hotNext, d.hotStamp, d.jcYield};
    const char *a0 = static_cast<const char *>(S->arena), *a1 = a0 + S->arenaBytes;
    for (void *p : ptrs) {
        const char *c = static_cast<const char *>(p);
        if (p && !(S->arena && c >= a0 && c < a1)) cudaFree(p);      // arena arrays go below
    }
    if (S->arena) cudaFree(S->arena);
    if (S->ownStream) cudaStreamDestroy(S->ownStream);
    delete S;
    return NF_OK;
}

// A contact-pass barrier that gave up (STATUS_TIMEOUT) left that step's contact forces
// incomplete, so the handle's state is no longer the reference's: the handle is marked failed,
// and this call and every later run call report NF_ETIMEOUT.
static const char *const TIMEOUT_MESSAGE =
    "a grid barrier of the contact pass waited past its limit; that step's contact forces are "
    "incomplete and this handle can no longer step";

static nf_status note_status(Solver &S, uint32_t status) {
    if (status & STATUS_TIMEOUT) S.failed = NF_ETIMEOUT;
    if (S.failed) return fail(&S, S.failed, "%s", TIMEOUT_MESSAGE);
    return NF_OK;
}

static nf_status read_status(Solver &S, uint32_t *out) {
    CK(&S, cudaMemcpyAsync(out, &S.d.s->status, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           S.stream));
    return sync_check(S);
}

nf_status nf_check(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    uint32_t w = 0;
    nf_status st = read_status(S, &w);
    if (st) return st;
    st = note_status(S, w);
    if (st) return st;
    if (w & STATUS_NONFINITE)
        return fail(&S, NF_EDEVICE, "a nodal velocity or displacement is not finite "
                                    "(status word 0x%x)", w & ~(uint32_t)STATUS_GRID_HASHED);
    if (w & STATUS_BUCKET_OVERFLOW)
        return fail(&S, NF_EDEVICE, "a contact bucket exceeded its bound (status word 0x%x)",
                    w & ~(uint32_t)STATUS_GRID_HASHED);
    return NF_OK;
}

nf_status nf_set_wait_limit(nf_solver *h, int64_t polls, int64_t nanoseconds) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (polls < 0 || nanoseconds < 0)
        return fail(&S, NF_EINVAL, "wait limits must be >= 0 (0 restores the default)");
    S.d.waitSpins = polls;
    S.d.waitNs = nanoseconds;
    return NF_OK;
}

nf_status nf_set_grid_slots(nf_solver *h, int32_t slots) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (slots < 0 || slots > NF_GRID_SLOTS)
        return fail(&S, NF_EINVAL, "grid slots must be in [0, 64]");
    S.gridSlots = slots;
    if (S.d.fastCount) S.d.fastLimit = slots;
    return NF_OK;
}

nf_status nf_status_word(nf_solver *h, uint32_t *word) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    *word = s.status & ~(uint32_t)STATUS_GRID_HASHED;
    return NF_OK;
}

nf_status nf_set_threads(nf_solver *h, int32_t n) {
    Solver *S = reinterpret_cast<Solver *>(h);
    if (n < 1) return fail(S, NF_EINVAL, "need at least one thread");
    return NF_OK;
}

nf_status nf_fix_radial(nf_solver *h, int32_t node) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (node < 0 || node >= S.N) return fail(&S, NF_EINVAL, "node %d out of range", node);
    k_or_flag<<<1, 1, 0, S.stream>>>(S.d.flags, node, 1);
    return NF_OK;
}
nf_status nf_fix_axial(nf_solver *h, int32_t node) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (node < 0 || node >= S.N) return fail(&S, NF_EINVAL, "node %d out of range", node);
    k_or_flag<<<1, 1, 0, S.stream>>>(S.d.flags, node, 2);
    return NF_OK;
}
nf_status nf_fix_all_axial(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (S.N > 0) k_or_all<<<grid_for(S.N, 256), 256, 0, S.stream>>>(S.d.flags, S.N, 2);
    return NF_OK;
}
nf_status nf_set_pressure_ramp(nf_solver *h, double pascals, double ramp) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    S.d.targetPressure = pascals;
    S.d.rampDuration = ramp;
    return NF_OK;
}
nf_status nf_set_relaxation_damping(nf_solver *h, double fraction, double omega) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (omega <= 0.0) return fail(&S, NF_EINVAL, "angular frequency must be positive");
    S.d.damping = 2.0 * fraction * omega;
    return NF_OK;
}
nf_status nf_set_hourglass_coefficient(nf_solver *h, double q) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (q < 0.0) return fail(&S, NF_EINVAL, "hourglass coefficient must be >= 0");
    S.d.hourglass = q;
    S.hourglass = q;
    return NF_OK;
}

nf_status nf_set_rigid_wall(nf_solver *h, double plane, double friction) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (friction < 0.0 || friction != friction)
        return fail(&S, NF_EINVAL, "friction coefficient must be >= 0");
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    s.wImpulse = s.wEnergyLoss = s.wFriction = 0.0;
    s.wContact = s.wStuck = 0;
    s.wContactAcc = s.wStuckAcc = 0;
    CK(&S, cudaMemcpyAsync(S.d.s, &s, sizeof s, cudaMemcpyHostToDevice, S.stream));
    S.d.hasWall = 1;
    S.d.wallPlane = plane;
    S.d.wallFriction = friction;
    if (!S.d.wallState) CK(&S, dalloc(S, &S.d.wallState, S.N));
    return sync_check(S);
}
nf_status nf_clear_rigid_wall(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    S.d.hasWall = 0;
    return NF_OK;
}

nf_status nf_set_contact(nf_solver *h, double friction, double damping, double scale) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (friction < 0.0) return fail(&S, NF_EINVAL, "friction must not be negative");
    if (damping < 0.0 || damping > 1.0)
        return fail(&S, NF_EINVAL,
                    "contact damping is a fraction of critical, so it lies in [0, 1]; was %.17g",
                    damping);
    if (!(scale > 0.0) || scale >= 2.0)
        return fail(&S, NF_EINVAL,
                    "the stiffness scale must lie in (0, 2); a pair is found from both sides, "
                    "so the effective stiffness is twice this and above 2 the contact "
                    "frequency exceeds what central difference can integrate, was %.17g", scale);
    Dev &d = S.d;
    const int N = S.N, E = S.E;
    // a node's free edges are at most two per element around it
    std::vector<int32_t> valence(N, 0);
    for (long long k = 0; k < 4LL * E; k++) valence[S.hostConn[k]]++;
    int segCap = 2;
    for (int n = 0; n < N; n++) segCap = std::max(segCap, 2 * valence[n]);
    if (!d.dead) {
        cudaError_t e_ = cudaSuccess;
#define A(ptr, n) if (e_ == cudaSuccess) e_ = dalloc(S, &(ptr), (n))
        A(d.dead, E);
        A(d.surfFlag, 4LL * E);
        A(d.segA, 4LL * E); A(d.segB, 4LL * E);
        A(d.edgeList, 4LL * E); A(d.edgePos, 4LL * E);
        A(d.nodeList, N); A(d.nodePos, N);
        A(d.nodeFree, N);
        A(d.nodeSeg, (size_t)N * (size_t)segCap);
        A(d.edgeStamp, 4LL * E); A(d.nodeStamp, N); A(d.touched, N);
        A(d.newDead, E);
        A(d.cr, N); A(d.cz, N);
        A(d.snr, 4LL * E); A(d.snz, 4LL * E); A(d.slen, 4LL * E);
        A(d.pnr, N); A(d.pnz, N);
        A(d.lastMaster, N); A(d.master, N); A(d.dropped, N);
        A(d.bucketCount, d.bucketCap + 1); A(d.bucketStart, d.bucketCap + 1);
        A(d.bucketCursor, d.bucketCap + 1);
        A(d.bucketEntry, 8LL * E); A(d.bucketF, 8LL * E); A(d.bucketFL, 8LL * E);
        A(d.bucketAB, 8LL * E); A(d.bucketA, 8LL * E); A(d.bucketN, 8LL * E); A(d.bucketL, 8LL * E);
        A(d.bucketCell, 8LL * E); A(d.entryCell, 8LL * E);
        d.fastCells = std::min(d.bucketCap + 1, 1 << 16);
        d.fastCap = NF_GRID_SLOTS;
        d.fastLimit = S.gridSlots;
        A(d.fastCount, d.fastCells);
        A(d.fastEntry, (size_t)d.fastCells * d.fastCap);
        A(d.fastF, (size_t)d.fastCells * d.fastCap); A(d.fastFL, (size_t)d.fastCells * d.fastCap);
        A(d.fastAB, (size_t)d.fastCells * d.fastCap);
        A(d.fastA, (size_t)d.fastCells * d.fastCap); A(d.fastN, (size_t)d.fastCells * d.fastCap);
        A(d.fastL, (size_t)d.fastCells * d.fastCap);
        A(d.nodeCell, N);
        A(d.pairNodes, N); A(d.pairVal, 12LL * N); A(d.pairEnergy, N); A(d.pairDiss, N);
        A(d.incCount, N + 1); A(d.incStart, N + 1); A(d.incCursor, N + 1); A(d.incEntry, 3LL * N);
        A(d.incSlots, (size_t)NF_INC_CAP * N);
        A(d.scanTmp, (size_t)d.scanTmpSize);
        A(d.coopSums, (size_t)d.coopBlocks);
#undef A
        if (e_ != cudaSuccess)
            return fail(&S, NF_ENOMEM, "contact allocation failed: %s", cudaGetErrorString(e_));
        d.segCap = segCap;
        // the end nodes of every element edge (QuadMesh.surface's edge k of element e runs
        // from corner k to corner k + 1)
        std::vector<int32_t> a(4LL * E), b(4LL * E);
        for (long long q = 0; q < 4LL * E; q++) {
            a[q] = S.hostConn[q];
            b[q] = S.hostConn[(q & ~3LL) + ((q + 1) & 3)];
        }
        CK(&S, upload(S, d.segA, a.data(), a.size()));
        CK(&S, upload(S, d.segB, b.data(), b.size()));
        const nf_status up = sync_check(S);             // a and b are about to go
        if (up) return up;
    } else {
        CK(&S, cudaMemsetAsync(d.dead, 0, E, S.stream));
    }
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    s.stale = 1;                       // new Contact(mesh): adopt() on the first begin
    s.fullRebuild = 1;
    s.newDeadCount = 0;
    s.nTouched = 0;
    s.edgeListLen = s.nodeListLen = 0;
    s.pairs = 0;
    s.escaped = 0;
    s.cEnergy = 0.0;
    s.cDissipation = 0.0;
    s.maxPenBits = 0;
    s.surfEdges = 0;
    s.surfNodes = 0;
    CK(&S, cudaMemcpyAsync(d.s, &s, sizeof s, cudaMemcpyHostToDevice, S.stream));
    d.hasContact = 1;
    d.cFriction = friction;
    d.cDamping = damping;
    d.cScale = scale;
    d.cSqrtScale = std::sqrt(scale);
    S.contactSet = true;
    return sync_check(S);
}
nf_status nf_clear_contact(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    S.d.hasContact = 0;
    S.contactSet = false;
    return NF_OK;
}

nf_status nf_set_gravity(nf_solver *h, double ar, double az) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    S.d.gravR = ar;
    S.d.gravZ = az;
    return NF_OK;
}

nf_status nf_set_erosion(nf_solver *h, double threshold) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (!S.damageSet)
        return fail(&S, NF_ESTATE, "erosion needs a failure model; call setDamage first");
    if (!(threshold > 0.0) || threshold > 1.0)
        return fail(&S, NF_EINVAL,
                    "the erosion threshold is a damage, so it lies in (0, 1]; was %.17g", threshold);
    S.d.erosionDamage = threshold;
    if (!S.d.gone) CK(&S, dalloc(S, &S.d.gone, S.E));
    S.d.hasErosion = 1;
    return sync_check(S);
}

nf_status nf_set_mass_scaling(nf_solver *h, double target) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (!(target > 0.0)) return fail(&S, NF_EINVAL, "the target step must be positive");
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    if (target < s.dt)
        return fail(&S, NF_EINVAL,
                    "the step is already %.17g s, longer than the target %.17g; mass scaling adds "
                    "mass and cannot shorten a step", s.dt, target);
    const double factor = (target / s.dt) * (target / s.dt);
    if (S.N > 0) k_scale_mass<<<grid_for(S.N, 256), 256, 0, S.stream>>>(S.d.mass, S.d.invMass, S.N, factor);
    S.d.massScale *= factor;
    s.dt = target;
    s.dtPrevious = s.dt;
    S.d.dt0 = s.dt;
    CK(&S, cudaMemcpyAsync(S.d.s, &s, sizeof s, cudaMemcpyHostToDevice, S.stream));
    return sync_check(S);
}

nf_status nf_set_damage(nf_solver *h, const double *gf, const double *eps) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    for (const nf_material &m : S.materials) {                 // ExplicitSolver.java:746-755
        const double worst = 2.0 * mat_mu(m) + (2.0 / 3.0) * (m.kinematic_hardening - m.youngs_modulus);
        if (!(worst > 0.0))
            return fail(&S, NF_EINVAL,
                        "a fully clamped softening modulus would make the return map singular: "
                        "2mu + (2/3)(H_kin - E) = %.17g <= 0", worst);
    }
    const int E = S.E, ppe = S.ppe;
    std::vector<double> geom(5LL * E);
    for (int e = 0; e < E; e++) {                              // ExplicitSolver.java:767-789
        const int b = e * 4;
        const double *r = S.hostR.data(), *z = S.hostZ.data();
        const int32_t *c = S.hostConn.data();
        const int n0 = c[b], n1 = c[b + 1], n2 = c[b + 2], n3 = c[b + 3];
        geom[5 * e + 1] = 0.5 * (r[n1] - r[n0] + r[n2] - r[n3]);
        geom[5 * e + 2] = 0.5 * (z[n1] - z[n0] + z[n2] - z[n3]);
        geom[5 * e + 3] = 0.5 * (r[n3] - r[n0] + r[n2] - r[n1]);
        geom[5 * e + 4] = 0.5 * (z[n3] - z[n0] + z[n2] - z[n1]);
        geom[5 * e] = fabs(signed_area(r, z, c, e));
    }
    for (int e = 0; e < E; e++)                                // Damage.java:232-243
        for (int g = 0; g < ppe; g++) {
            if (!(gf[e] > 0.0)) return fail(&S, NF_EINVAL, "fracture energy must be positive, was %.17g", gf[e]);
            const double youngs = S.materials[S.emat[e]].youngs_modulus;
            if (!(youngs > 0.0)) return fail(&S, NF_EINVAL, "Young's modulus must be positive, was %.17g", youngs);
        }
    for (int e = 0; e < E; e++)                                // Damage.java:249-260
        for (int g = 0; g < ppe; g++) {
            const int p = e * ppe + g;
            if (!(eps[e] > 0.0))
                return fail(&S, NF_EINVAL, "failure strain must be positive; point %d has %.17g", p, eps[e]);
            if (!(geom[5 * e] > 0.0))
                return fail(&S, NF_EINVAL, "area must be positive; point %d has %.17g", p, geom[5 * e]);
        }
    Dev &d = S.d;
    const size_t P = (size_t)E * ppe;
    if (!d.dFail) {
        cudaError_t e_ = cudaSuccess;
#define A(ptr, n) if (e_ == cudaSuccess) e_ = dalloc(S, &(ptr), (n))
        A(d.dFail, E); A(d.dGf, E); A(d.dGeom, 5LL * E);
        A(d.dStrength, P); A(d.dSoft, P); A(d.dWidth, P);
#undef A
        if (e_ != cudaSuccess)
            return fail(&S, NF_ENOMEM, "damage allocation failed: %s", cudaGetErrorString(e_));
    } else {
        CK(&S, cudaMemsetAsync(d.dStrength, 0, sizeof(double) * P, S.stream));
        CK(&S, cudaMemsetAsync(d.dSoft, 0, sizeof(double) * P, S.stream));
        CK(&S, cudaMemsetAsync(d.dWidth, 0, sizeof(double) * P, S.stream));
    }
    CK(&S, upload(S, d.dFail, eps, E));
    CK(&S, upload(S, d.dGf, gf, E));
    CK(&S, upload(S, d.dGeom, geom.data(), geom.size()));
    d.hasDamage = 1;
    S.damageSet = true;
    if (d.mixed) {
        nf_status st = ensure_mixed_damage(S);
        if (st) return st;
        launch_convert_state(S, true, 2);
    }
    return sync_check(S);
}

nf_status nf_set_velocity(nf_solver *h, int32_t node, double vr, double vz) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (node < 0 || node >= S.N) return fail(&S, NF_EINVAL, "node %d out of range", node);
    k_set_velocity<<<1, 1, 0, S.stream>>>(S.d.V, node, vr, vz);
    return NF_OK;
}
nf_status nf_set_uniform_velocity(nf_solver *h, double vr, double vz) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (S.N > 0) k_uniform_velocity<<<grid_for(S.N, 256), 256, 0, S.stream>>>(S.d.V, S.N, vr, vz);
    return NF_OK;
}
nf_status nf_set_velocities(nf_solver *h, const double *vr, const double *vz) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    std::vector<double2> v(S.N);
    for (int i = 0; i < S.N; i++) v[i] = make_double2(vr[i], vz[i]);
    CK(&S, upload(S, S.d.V, v.data(), S.N));
    return sync_check(S);
}

// Captures `steps` whole steps into an executable graph (kernel nodes only).
static nf_status capture_steps(Solver &S, int steps, cudaGraphExec_t *out, int *kernels) {
    cudaGraph_t g = nullptr;
    CK(&S, cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
    int n = 0;
    for (int k = 0; k < steps; k++) n += launch_step(S, true);
    cudaError_t e = cudaStreamEndCapture(S.stream, &g);
    if (e != cudaSuccess) return fail(&S, NF_EDEVICE, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(&S, NF_EDEVICE, "graph instantiate: %s", cudaGetErrorString(e));
    *kernels = n;
    return NF_OK;
}

// Graphs are captured for the current configuration (the Dev record the kernels receive by
// value); any setter that changes it invalidates them.
static nf_status ensure_graphs(Solver &S) {
    if (S.graphValid && memcmp(&S.graphDev, &S.d, sizeof(Dev)) == 0) return NF_OK;
    if (S.graph1) cudaGraphExecDestroy(S.graph1);
    if (S.graph16) cudaGraphExecDestroy(S.graph16);
    S.graph1 = S.graph16 = nullptr;
    S.graphValid = false;
    nf_status st = capture_steps(S, 1, &S.graph1, &S.graphKernels1);
    if (st) return st;
    st = capture_steps(S, 16, &S.graph16, &S.graphKernels16);
    if (st) return st;
    memcpy(&S.graphDev, &S.d, sizeof(Dev));
    S.graphValid = true;
    return NF_OK;
}

static nf_status enqueue_steps(Solver &S, int64_t steps) {
    if (S.profiling) {
        for (int64_t k = 0; k < steps; k++) S.launches += launch_step(S, true);
        S.profSteps += steps;
        return NF_OK;
    }
    if (!S.noGraphs && ensure_graphs(S) != NF_OK) {
        // a stream that cannot capture (a cooperative kernel node the runtime refuses): the
        // same launches, enqueued one step at a time
        (void)cudaGetLastError();
        S.noGraphs = true;
        S.err.clear();
    }
    if (S.noGraphs) {
        for (int64_t k = 0; k < steps; k++) S.launches += launch_step(S, true);
        return NF_OK;
    }
    while (steps >= 16) {
        CK(&S, cudaGraphLaunch(S.graph16, S.stream));
        S.launches += S.graphKernels16;
        steps -= 16;
    }
    for (; steps > 0; steps--) {
        CK(&S, cudaGraphLaunch(S.graph1, S.stream));
        S.launches += S.graphKernels1;
    }
    return NF_OK;
}

// run(int), ExplicitSolver.java:936-938. Enqueues the steps and returns; reads wait for them.
nf_status nf_step(nf_solver *h, int64_t steps) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (S.failed) return note_status(S, 0);
    if (steps <= 0) return NF_OK;
    if (!S.unbounded) {
        k_set_run<<<1, 1, 0, S.stream>>>(S.d.s, INFINITY, (long long)9.0e18);
        S.launches++;
        S.unbounded = true;
    }
    if (S.hostSteps == 0) {
        S.launches += launch_initial_assembly(S);
        S.profSteps += 0;
    }
    nf_status st = enqueue_steps(S, steps);
    if (st) return st;
    S.hostSteps += steps;
    CK(&S, cudaGetLastError());
    return NF_OK;
}

nf_status nf_advance(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (S.failed) return note_status(S, 0);
    S.launches += launch_advance(S);
    return sync_check(S);
}

// The loop of TaylorImpactCase.java:250-253: steps while time < t_end. The predicate is
// evaluated on the device; chunks of sixteen predicated steps are replayed between checks.
nf_status nf_run_until(nf_solver *h, double t_end, int64_t max_steps, int64_t *taken) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (taken) *taken = 0;
    if (S.failed) return note_status(S, 0);
    if (max_steps <= 0) return NF_OK;
    k_set_run<<<1, 1, 0, S.stream>>>(S.d.s, t_end, max_steps);
    S.launches++;
    S.unbounded = false;
    if (S.hostSteps == 0) S.launches += launch_initial_assembly(S);
    DevScalars s{};
    for (;;) {
        nf_status st = enqueue_steps(S, 16);
        if (st) return st;
        st = read_scalars(S, &s);
        if (st) return st;
        if (s.status & STATUS_TIMEOUT) {
            S.hostSteps += s.stepsTaken;
            if (taken) *taken = s.stepsTaken;
            return note_status(S, s.status);
        }
        if (!s.active || s.stepsTaken >= max_steps || !(s.time < t_end)) break;
    }
    S.hostSteps += s.stepsTaken;
    if (taken) *taken = s.stepsTaken;
    return NF_OK;
}

nf_status nf_synchronize(nf_solver *h) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    uint32_t w = 0;
    nf_status st = read_status(S, &w);
    if (st) return st;
    return note_status(S, w);
}

nf_status nf_set_stream(nf_solver *h, void *stream) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    nf_status st = sync_check(S);
    if (st) return st;
    S.stream = stream ? reinterpret_cast<cudaStream_t>(stream) : S.ownStream;
    return NF_OK;
}

nf_status nf_profile(nf_solver *h, int32_t enable) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    S.profiling = enable != 0;
    return NF_OK;
}

nf_status nf_profile_read(nf_solver *h, double *ms, int64_t *steps) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    nf_status st = sync_check(S);
    if (st) return st;
    for (auto &r : S.recs) {
        float t = 0.0f;
        CK(&S, cudaEventElapsedTime(&t, r.a, r.b));
        S.profMs[r.group] += t;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    S.recs.clear();
    for (int g = 0; g < NF_GROUP_COUNT; g++) {
        ms[g] = S.profMs[g];
        S.profMs[g] = 0.0;
    }
    if (steps) *steps = S.profSteps;
    S.profSteps = 0;
    return NF_OK;
}

nf_status nf_set_precision(nf_solver *h, int32_t precision) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (precision == NF_PRECISION_COMPENSATED)
        return fail(&S, NF_EINVAL, "the compensated form runs in batches (nf_batch_create)");
    if (precision != NF_PRECISION_FP64 && precision != NF_PRECISION_MIXED)
        return fail(&S, NF_EINVAL, "unknown precision %d", precision);
    nf_status st = sync_check(S);
    if (st) return st;
    Dev &d = S.d;
    if (precision == NF_PRECISION_MIXED && !d.mixed) {
        const size_t P = (size_t)S.E * S.ppe;
        if (!d.sigF) {
            cudaError_t e_ = cudaSuccess;
#define A(ptr, n) if (e_ == cudaSuccess) e_ = dalloc(S, &(ptr), (n))
            A(d.matsF, S.materials.size());
            A(d.sigF, 4 * P); A(d.backF, 4 * P); A(d.epsPF, P); A(d.wPF, P);
            A(d.hgF, S.E); A(d.hgKF, S.E); A(d.contribF, 8 * ((size_t)S.E + S.K));
            A(d.pMid, S.N); A(d.pCur, S.N); A(d.vdt, S.N); A(d.gaussVol, P);
#undef A
            if (e_ != cudaSuccess)
                return fail(&S, NF_ENOMEM, "mixed-precision allocation failed: %s", cudaGetErrorString(e_));
            std::vector<MatF> mf(S.materials.size());
            for (size_t m = 0; m < S.materials.size(); m++)
                mf[m] = mat_float(mat_dev(S.materials[m], S.formulation));
            CK(&S, upload(S, d.matsF, mf.data(), mf.size()));
            launch_point_volumes(S, d.gaussVol);
        }
        if (S.damageSet) {
            st = ensure_mixed_damage(S);
            if (st) return st;
        }
        launch_convert_state(S, true, 3);
        d.mixed = 1;
    } else if (precision == NF_PRECISION_FP64 && d.mixed) {
        launch_convert_state(S, false, 3);
        d.mixed = 0;
    }
    return sync_check(S);
}

nf_status nf_launch_count(nf_solver *h, int64_t *launches) {
    *launches = reinterpret_cast<Solver *>(h)->launches;
    return NF_OK;
}

nf_status nf_field_size(nf_solver *h, int32_t field, size_t *count, size_t *bytes) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    const size_t N = S.N, E = S.E, P = (size_t)S.E * S.ppe;
    *bytes = 8;
    switch (field) {
        case NF_FIELD_UR: case NF_FIELD_UZ: case NF_FIELD_VR: case NF_FIELD_VZ:
        case NF_FIELD_FR: case NF_FIELD_FZ: case NF_FIELD_MASS: *count = N; break;
        case NF_FIELD_STRESS: case NF_FIELD_BACK_STRESS: *count = 4 * P; break;
        case NF_FIELD_PLASTIC_STRAIN: case NF_FIELD_PLASTIC_WORK: *count = P; break;
        case NF_FIELD_HOURGLASS_R: case NF_FIELD_HOURGLASS_Z: case NF_FIELD_HOURGLASS_STIFFNESS:
            *count = E; break;
        case NF_FIELD_DAMAGE_STRENGTH: case NF_FIELD_DAMAGE_SOFTENING: case NF_FIELD_DAMAGE_WIDTH:
            *count = S.damageSet ? P : 0; break;
        case NF_FIELD_ERODED: *count = S.d.gone ? E : 0; *bytes = 1; break;
        case NF_FIELD_ON_WALL: case NF_FIELD_WALL_STATE: case NF_FIELD_CONTACT_STATE:
        case NF_FIELD_FIXED: *count = N; *bytes = 1; break;
        case NF_FIELD_CONTACT_MASTER: *count = N; *bytes = 4; break;
        case NF_FIELD_SURFACE_EDGES: case NF_FIELD_SURFACE_NODES: {
            *bytes = 4;
            if (!S.contactSet) { *count = 0; break; }
            DevScalars s;
            nf_status st = read_scalars(S, &s);
            if (st) return st;
            *count = field == NF_FIELD_SURFACE_EDGES ? 2 * (size_t)s.surfEdges : (size_t)s.surfNodes;
            break;
        }
        default: return fail(&S, NF_EINVAL, "unknown field %d", field);
    }
    return NF_OK;
}

nf_status nf_read_field(nf_solver *h, int32_t field, void *dst, size_t nbytes) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    size_t count, eb;
    nf_status st = nf_field_size(h, field, &count, &eb);
    if (st) return st;
    if (nbytes != count * eb)
        return fail(&S, NF_EINVAL, "field %d holds %zu bytes, caller passed %zu", field, count * eb, nbytes);
    if (count == 0) return NF_OK;
    Dev &d = S.d;
    mixed_to_double(S);
    st = sync_check(S);
    if (st) return st;
    auto pair = [&](const double2 *src, int comp) -> nf_status {
        std::vector<double2> tmp(count);
        CK(&S, cudaMemcpy(tmp.data(), src, sizeof(double2) * count, cudaMemcpyDeviceToHost));
        double *o = (double *)dst;
        for (size_t i = 0; i < count; i++) o[i] = comp ? tmp[i].y : tmp[i].x;
        return NF_OK;
    };
    auto copy = [&](const void *src) -> nf_status {
        CK(&S, cudaMemcpy(dst, src, nbytes, cudaMemcpyDeviceToHost));
        return NF_OK;
    };
    switch (field) {
        case NF_FIELD_UR: return pair(d.U, 0);
        case NF_FIELD_UZ: return pair(d.U, 1);
        case NF_FIELD_VR: return pair(d.V, 0);
        case NF_FIELD_VZ: return pair(d.V, 1);
        case NF_FIELD_FR: return pair(d.F, 0);
        case NF_FIELD_FZ: return pair(d.F, 1);
        case NF_FIELD_MASS: return copy(d.mass);
        case NF_FIELD_STRESS: return copy(d.sig);
        case NF_FIELD_BACK_STRESS: return copy(d.back);
        case NF_FIELD_PLASTIC_STRAIN: return copy(d.epsP);
        case NF_FIELD_PLASTIC_WORK: return copy(d.wP);
        case NF_FIELD_HOURGLASS_R: return pair(d.hg, 0);
        case NF_FIELD_HOURGLASS_Z: return pair(d.hg, 1);
        case NF_FIELD_HOURGLASS_STIFFNESS: return copy(d.hgK);
        case NF_FIELD_DAMAGE_STRENGTH: return copy(d.dStrength);
        case NF_FIELD_DAMAGE_SOFTENING: return copy(d.dSoft);
        case NF_FIELD_DAMAGE_WIDTH: return copy(d.dWidth);
        case NF_FIELD_ERODED: return copy(d.gone);
        case NF_FIELD_WALL_STATE: return copy(d.wallState);
        case NF_FIELD_CONTACT_STATE: return copy(d.contactState);
        case NF_FIELD_ON_WALL: case NF_FIELD_FIXED: {
            std::vector<uint8_t> f(count);
            CK(&S, cudaMemcpy(f.data(), d.flags, count, cudaMemcpyDeviceToHost));
            uint8_t *o = (uint8_t *)dst;
            for (size_t i = 0; i < count; i++)
                o[i] = field == NF_FIELD_ON_WALL ? ((f[i] >> 2) & 1) : (f[i] & 3);
            return NF_OK;
        }
        case NF_FIELD_CONTACT_MASTER: {
            // the device keeps masters as element edges; the reference numbers a segment by
            // its rank among the free edges in element order (QuadMesh.surface)
            int32_t *o = (int32_t *)dst;
            for (size_t i = 0; i < count; i++) o[i] = -1;
            if (!S.contactSet) return NF_OK;
            std::vector<int32_t> flag(4LL * S.E), pos(S.N), master(S.N);
            CK(&S, cudaMemcpy(flag.data(), d.surfFlag, 4 * flag.size(), cudaMemcpyDeviceToHost));
            CK(&S, cudaMemcpy(pos.data(), d.nodePos, 4 * pos.size(), cudaMemcpyDeviceToHost));
            CK(&S, cudaMemcpy(master.data(), d.master, 4 * master.size(), cudaMemcpyDeviceToHost));
            std::vector<int32_t> rank(flag.size());
            int32_t r = 0;
            for (size_t q = 0; q < flag.size(); q++) {
                rank[q] = r;
                r += flag[q] ? 1 : 0;
            }
            for (int n = 0; n < S.N; n++)
                if (pos[n] >= 0 && master[n] >= 0) o[n] = rank[master[n]];
            return NF_OK;
        }
        case NF_FIELD_SURFACE_NODES: {              // the surface nodes, ascending
            std::vector<int32_t> free(S.N);
            CK(&S, cudaMemcpy(free.data(), d.nodeFree, 4 * free.size(), cudaMemcpyDeviceToHost));
            int32_t *o = (int32_t *)dst;
            size_t k = 0;
            for (int n = 0; n < S.N && k < count; n++)
                if (free[n] > 0) o[k++] = n;
            return NF_OK;
        }
        case NF_FIELD_SURFACE_EDGES: {              // the free edges in element order
            std::vector<int32_t> flag(4LL * S.E);
            CK(&S, cudaMemcpy(flag.data(), d.surfFlag, 4 * flag.size(), cudaMemcpyDeviceToHost));
            int32_t *o = (int32_t *)dst;
            size_t k = 0;
            for (size_t q = 0; q < flag.size() && k + 1 < count + 1; q++) {
                if (!flag[q]) continue;
                o[k++] = S.hostConn[q];
                o[k++] = S.hostConn[(q & ~(size_t)3) + ((q + 1) & 3)];
            }
            return NF_OK;
        }
        default: return fail(&S, NF_EINVAL, "unknown field %d", field);
    }
}

nf_status nf_write_field(nf_solver *h, int32_t field, const void *src, size_t nbytes) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    Dev &d = S.d;
    size_t count, eb;
    switch (field) {
        case NF_FIELD_UR: case NF_FIELD_UZ: case NF_FIELD_VR: case NF_FIELD_VZ:
        case NF_FIELD_STRESS: case NF_FIELD_BACK_STRESS: case NF_FIELD_PLASTIC_STRAIN:
        case NF_FIELD_PLASTIC_WORK: break;
        default: return fail(&S, NF_EINVAL, "field %d is not writable", field);
    }
    nf_status st = nf_field_size(h, field, &count, &eb);
    if (st) return st;
    if (nbytes != count * eb)
        return fail(&S, NF_EINVAL, "field %d holds %zu bytes, caller passed %zu", field, count * eb, nbytes);
    mixed_to_double(S);
    st = sync_check(S);
    if (st) return st;
    struct Refloat {
        Solver &S;
        ~Refloat() {
            if (S.d.mixed) {
                launch_convert_state(S, true, 1);
                cudaStreamSynchronize(S.stream);
            }
        }
    } refloat{S};
    auto pair = [&](double2 *dstp, int comp) -> nf_status {
        std::vector<double2> tmp(count);
        CK(&S, cudaMemcpy(tmp.data(), dstp, sizeof(double2) * count, cudaMemcpyDeviceToHost));
        const double *in = (const double *)src;
        for (size_t i = 0; i < count; i++) (comp ? tmp[i].y : tmp[i].x) = in[i];
        CK(&S, cudaMemcpy(dstp, tmp.data(), sizeof(double2) * count, cudaMemcpyHostToDevice));
        return NF_OK;
    };
    switch (field) {
        case NF_FIELD_UR: return pair(d.U, 0);
        case NF_FIELD_UZ: return pair(d.U, 1);
        case NF_FIELD_VR: return pair(d.V, 0);
        case NF_FIELD_VZ: return pair(d.V, 1);
        case NF_FIELD_STRESS: CK(&S, cudaMemcpy(d.sig, src, nbytes, cudaMemcpyHostToDevice)); return NF_OK;
        case NF_FIELD_BACK_STRESS: CK(&S, cudaMemcpy(d.back, src, nbytes, cudaMemcpyHostToDevice)); return NF_OK;
        case NF_FIELD_PLASTIC_STRAIN: case NF_FIELD_PLASTIC_WORK:
            CK(&S, cudaMemcpy(field == NF_FIELD_PLASTIC_STRAIN ? d.epsP : d.wP, src, nbytes,
                              cudaMemcpyHostToDevice));
            if (d.jcYield) {                   // the kept yield radii follow the new state
                launch_jc_yield(d, S.stream);
                return sync_check(S);
            }
            return NF_OK;
        default: return NF_EINVAL;
    }
}

nf_status nf_get_state(nf_solver *h, nf_state *o) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    memset(o, 0, sizeof *o);
    o->time = s.time;
    o->timestep = s.dt;
    o->timestep_previous = s.dtPrevious;
    o->reference_timestep = S.d.dt0;
    o->mass_scale = S.d.massScale;
    o->min_edge_squared = s.minEdgeSquared;
    o->fastest_wave = S.d.fastestWave;
    o->eroded_energy = s.erodedEnergy;
    if (S.d.rampDuration <= 0.0) {
        o->bore_pressure = S.d.targetPressure;
    } else {
        const double q = std::min(1.0, s.time / S.d.rampDuration);
        o->bore_pressure = S.d.targetPressure * q * q * (3.0 - 2.0 * q);
    }
    o->steps = s.steps;
    o->eroded_elements = s.erodedCount;
    o->inverted_elements = s.invertedCount;
    o->node_count = S.N;
    o->element_count = S.E;
    o->points_per_element = S.ppe;
    o->pressure_edge_count = S.K;
    return NF_OK;
}

nf_status nf_audits(nf_solver *h, nf_audit *o) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    mixed_to_double(S);
    nf_status st = sync_check(S);
    if (st) return st;
    launch_audits(S, o);
    return sync_check(S);
}

nf_status nf_wall_stats(nf_solver *h, nf_wall_info *o) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    memset(o, 0, sizeof *o);
    o->present = S.d.hasWall;
    o->plane = S.d.wallPlane;
    o->friction = S.d.wallFriction;
    o->impulse = s.wImpulse;
    o->energy_loss = s.wEnergyLoss;
    o->friction_dissipation = s.wFriction;
    o->contact_count = s.wContact;
    o->stuck_count = s.wStuck;
    return NF_OK;
}

nf_status nf_contact_stats(nf_solver *h, nf_contact_info *o) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    memset(o, 0, sizeof *o);
    if (!S.contactSet) return NF_OK;
    DevScalars s;
    nf_status st = read_scalars(S, &s);
    if (st) return st;
    o->present = 1;
    o->friction = S.d.cFriction;
    o->energy = s.cEnergy;
    o->dissipation = s.cDissipation;
    double mp;
    memcpy(&mp, &s.maxPenBits, 8);
    o->max_penetration = mp;
    o->pair_count = s.pairs;
    o->escaped_nodes = s.escaped;
    o->segment_count = s.surfEdges;
    return NF_OK;
}

nf_status nf_measure_body(nf_solver *h, nf_measure *o) {
    Solver &S = *reinterpret_cast<Solver *>(h);
    nf_status st = sync_check(S);
    if (st) return st;
    launch_measure(S, o);
    return sync_check(S);
}

nf_status nf_material_point_update(const nf_material *material, int32_t formulation, int32_t count,
                                   double *sig, double *back, double *eps_p, double *work,
                                   const double *strain, double strain_dt,
                                   const nf_damage_points *damage, double *dgamma) {
    const char *why = material_invalid(*material);
    if (why) return fail(nullptr, NF_EINVAL, "%s", why);
    if (count <= 0) return NF_OK;
    const MatDev m = mat_dev(*material, formulation);
    const size_t n = count;
    const bool dm = damage && damage->failure_strain;
    double *buf = nullptr;
    const size_t total = 4 * n + 4 * n + n + n + 4 * n + n + (dm ? (n * 3 + 5 * n + 3 * n) : 0);
    if (cudaMalloc(&buf, sizeof(double) * total) != cudaSuccess)
        return fail(nullptr, NF_ENOMEM, "device allocation failed");
    double *dsig = buf, *dback = dsig + 4 * n, *deps = dback + 4 * n, *dwork = deps + n;
    double *dstrain = dwork + n, *dg = dstrain + 4 * n, *rest = dg + n;
    cudaMemcpy(dsig, sig, 8 * 4 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dback, back, 8 * 4 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(deps, eps_p, 8 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dwork, work, 8 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dstrain, strain, 8 * 4 * n, cudaMemcpyHostToDevice);
    double *fail_ = nullptr, *gf = nullptr, *yo = nullptr, *geom = nullptr, *str = nullptr,
           *soft = nullptr, *wid = nullptr;
    if (dm) {
        fail_ = rest; gf = fail_ + n; yo = gf + n; geom = yo + n; str = geom + 5 * n;
        soft = str + n; wid = soft + n;
        cudaMemcpy(fail_, damage->failure_strain, 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(gf, damage->fracture_energy, 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(yo, damage->youngs_modulus, 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(geom, damage->geometry, 8 * 5 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(str, damage->strength, 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(soft, damage->softening, 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(wid, damage->width, 8 * n, cudaMemcpyHostToDevice);
    }
    launch_material_points(m, count, dsig, dback, deps, dwork, dstrain, strain_dt, fail_, gf, yo,
                           geom, str, soft, wid, dg, 0);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaFree(buf);
        return fail(nullptr, NF_EDEVICE, "material point kernel: %s", cudaGetErrorString(e));
    }
    cudaMemcpy(sig, dsig, 8 * 4 * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(back, dback, 8 * 4 * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(eps_p, deps, 8 * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(work, dwork, 8 * n, cudaMemcpyDeviceToHost);
    if (dgamma) cudaMemcpy(dgamma, dg, 8 * n, cudaMemcpyDeviceToHost);
    if (dm) {
        cudaMemcpy(damage->strength, str, 8 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(damage->softening, soft, 8 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(damage->width, wid, 8 * n, cudaMemcpyDeviceToHost);
    }
    cudaFree(buf);
    return NF_OK;
}

}  // extern "C"

// Helpers shared with the allocation-free entry point (noalloc.cu).
namespace nf {
const char *validate_material(const nf_material &m) { return material_invalid(m); }
MatDev material_constants(const nf_material &m, int formulation) { return mat_dev(m, formulation); }
void set_thread_error(const char *message) { g_err = message; }
// Set-up helpers shared with the batched handle (api_batch.cu).
double material_wave(const nf_material &m) { return mat_wave(m); }
MatF material_constants_f32(const MatDev &m) { return mat_float(m); }
double element_signed_area(const double *r, const double *z, const int32_t *conn, int e) {
    return signed_area(r, z, conn, e);
}
void setup_lumped_mass(const double *r, const double *z, const int32_t *conn, int E,
                       const nf_material *materials, const int32_t *emat, bool axi,
                       double thickness, double *mass) {
    lumped_mass(r, z, conn, E, materials, emat, axi, thickness, mass);
}
void setup_node_slots(const int32_t *conn, int N, int E, const int32_t *pedges, int K,
                      int32_t *slotStart, int32_t *slots) {
    node_slots(conn, N, E, pedges, K, slotStart, slots);
}
double setup_min_edge(const double *r, const double *z, const int32_t *conn, int E) {
    return min_edge_length(r, z, conn, E);
}
// Helpers shared with the device film (k_film.cu).
void solver_state_to_double(Solver &S) { mixed_to_double(S); }
nf_status solver_fail(Solver &S, nf_status st, const char *message) {
    return fail(&S, st, "%s", message);
}
nf_status solver_sync(Solver &S) { return sync_check(S); }
}  // namespace nf
