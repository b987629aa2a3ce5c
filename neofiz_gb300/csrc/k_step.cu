// k_step.cu -- the kernels of one explicit central-difference timestep
// (ExplicitSolver.step, src/main/java/org/neofiz/solver/ExplicitSolver.java:940-991):
//
//   k_nodal            dtAvg, decay, gain; velocity/position update, fixed DOFs,   :947-956,
//                      rigid wall                                                  :998-1062
//   k_erode            deletion of failed or inverted elements                      :663-691
//   k_element_reduced  one-point quadrature + Flanagan-Belytschko hourglass        :1373-1504
//   k_element_full     2x2 Gauss quadrature                                         :1219-1339
//   k_pressure         follower pressure on the bore edges                          :1511-1556
//   k_gather           per-node sum of its sources in CSR order, plus m g           :1147-1165
//                      (its first blocks sort the next step's work list)
//   (contact kernels, k_contact.cu)                                                :1099-1109
//   k_end              running totals, adaptive CFL step, the next step's run      :985-990
//                      predicate
//   (k_begin starts the initial assembly only)
//
// Every kernel reads the solver's scalars (dt, time, ...) from device memory, so a sequence
// of steps is a fixed sequence of launches with no host decision between them.
#include "nf_bodies.cuh"
#include "nf_surface.cuh"

namespace nf {

constexpr int BLOCK = 128;

__device__ __forceinline__ unsigned long long dbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long u) {
    return __longlong_as_double((long long)u);
}

// Fixed-shape block sum: the same inputs in the same threads always add in the same order.
// A warp whose 32 values are all +0 skips its tree (its sum is +0 either way), which most warps
// of the per-step totals are (wall terms, eroded energy): an FP64 warp instruction costs the
// same with any number of lanes, so the tree is not free.
__device__ double block_sum(double v, double *sh) {
    if (__any_sync(0xffffffffu, __double_as_longlong(v) != 0))
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0) {
        const int warps = (blockDim.x + 31) >> 5;
        for (int w = 0; w < warps; w++) t += sh[w];
    }
    return t;   // valid in thread 0
}

// ------------------------------------------------------------------------------------ begin

// The initial assembly's start: the run predicate and the contact pass's per-step scalars.
// A step proper starts inside k_nodal.
__global__ void k_begin(Dev d) {
    DevScalars *s = d.s;
    s->active = s->time < s->tEnd && s->stepsTaken < s->maxSteps ? 1 : 0;
    contact_step_reset(s);
}

// ------------------------------------------------------------------------------------ nodal

// nodalUpdate, ExplicitSolver.java:998-1062, with RigidWall.hold/crosses/arrive/slide
// (RigidWall.java:163-259). A fixed grid strides over the nodes; each thread adds its nodes'
// wall terms in node order and the block adds its threads in a fixed tree, so the totals are
// deterministic. 1/m comes from the invMass array (the same division, done once). In the
// mixed form the kernel also writes the FP32 geometry the element kernel reads.
//
// The step starts here (ExplicitSolver.java:944-952): the run predicate was set by the last
// step's end (or by the run's bounds); each block's first thread forms the damping
// coefficients from dt and dtPrevious, which nothing in this kernel writes (the same values in
// every block; one thread, as FP64 costs a whole warp's issue whatever the lanes), and block 0
// resets the contact pass's per-step scalars, which nothing in this kernel reads. The wall
// counts add into their own accumulators, which the step's end publishes and clears
// (RigidWall.beginStep, RigidWall.java:153-156).
__global__ void __launch_bounds__(BLOCK) k_nodal(Dev d) {
    __shared__ double sh[BLOCK / 32];
    __shared__ double coef[3];
    DevScalars *s = d.s;
    if (!s->active) return;
    const double dt = s->dt;
    {
        // the thread's first node is fetched into L1 while the coefficients are formed
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < d.N) {
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.U + i));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.V + i));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.F + i));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.X0 + i));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.mass + i));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(d.invMass + i));
        }
    }
    if (threadIdx.x == 0) {
        const double avg = 0.5 * (s->dtPrevious + dt);
        const double half = 0.5 * d.damping * avg;
        coef[0] = (1.0 - half) / (1.0 + half);
        coef[1] = avg / (1.0 + half);
        coef[2] = avg;
        if (blockIdx.x == 0) {
            s->decay = coef[0];
            s->gain = coef[1];
            s->dtAvg = avg;
            contact_step_reset(s);
        }
    }
    __syncthreads();
    const double decay = coef[0], gain = coef[1], dtAvg = coef[2];
    double impulse = 0.0, loss = 0.0, fric = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.N; i += gridDim.x * blockDim.x) {
        nodal_node(d, i, NodalCoef{decay, gain, dtAvg, dt},
                   WallRef{d.hasWall, d.wallPlane, d.wallFriction, &d.s->wContactAcc,
                           &d.s->wStuckAcc},
                   d.mixed ? MixedGeo{d.pMid, d.pCur, d.vdt, 0} : MixedGeo{nullptr, nullptr, nullptr, 0},
                   &d.s->status, impulse, loss, fric);
    }
    if (d.hasWall) {
        // a block whose terms are all +0 (no node on the wall) has sums of +0: one vote
        // instead of three trees
        const bool any = (__double_as_longlong(impulse) | __double_as_longlong(loss) |
                          __double_as_longlong(fric)) != 0;
        double a = 0.0, b = 0.0, c = 0.0;
        if (__syncthreads_or(any)) {
            a = block_sum(impulse, sh);
            b = block_sum(loss, sh);
            c = block_sum(fric, sh);
        }
        if (threadIdx.x == 0) {
            d.partials[(PARTIAL_WALL + 0) * d.maxBlocks + blockIdx.x] = a;
            d.partials[(PARTIAL_WALL + 1) * d.maxBlocks + blockIdx.x] = b;
            d.partials[(PARTIAL_WALL + 2) * d.maxBlocks + blockIdx.x] = c;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {               // ExplicitSolver.java:973-974
        d.s->time += dt;
        d.s->steps += 1;
    }
}

// ------------------------------------------------------------------------------------ geometry helpers

// gaussVolume, ExplicitSolver.java:1939-1965 (reference configuration)
__device__ double gauss_volume(const Dev &d, int e, int g) {
    const int4 c = d.conn[e];
    const double2 p0 = d.X0[c.x], p1 = d.X0[c.y], p2 = d.X0[c.z], p3 = d.X0[c.w];
    const double r0 = p0.x, r1 = p1.x, r2 = p2.x, r3 = p3.x;
    const double z0 = p0.y, z1 = p1.y, z2 = p2.y, z3 = p3.y;
    const double G = 0.5773502691896258;
    const double gx[4] = {-G, G, G, -G}, ge[4] = {-G, -G, G, G};
    const double xi = d.ppe == 1 ? 0.0 : gx[g];
    const double eta = d.ppe == 1 ? 0.0 : ge[g];
    const double weight = d.ppe == 1 ? 4.0 : 1.0;
    const double xm = 1.0 - xi, xp = 1.0 + xi, em = 1.0 - eta, ep = 1.0 + eta;
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
    return weight * (d.axi ? 2.0 * NF_PI * rg * det : d.thickness * det);
}

// pointStrainEnergy, ExplicitSolver.java:1666-1675
__device__ double point_strain_energy(const Dev &d, int e, int g) {
    const int p = e * d.ppe + g;
    const double *sg = d.sig + 4 * (size_t)p;
    const MatDev &m = d.mats[d.emat[e]];
    const double press = (sg[0] + sg[1] + sg[2]) / 3.0;
    const double a = sg[0] - press, bb = sg[1] - press, c = sg[2] - press;
    const double dd = sg[3];
    const double density = (a * a + bb * bb + c * c + 2.0 * dd * dd) / (4.0 * m.mu)
                           + press * press / (2.0 * m.bulk);
    return density * gauss_volume(d, e, g);
}

__global__ void k_point_volumes(Dev d, double *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.E * d.ppe) return;
    out[p] = gauss_volume(d, p / d.ppe, p % d.ppe);
}

int launch_point_volumes(Solver &S, double *out) {
    const int P = S.d.E * S.d.ppe;
    if (P > 0) k_point_volumes<<<grid_for(P, BLOCK), BLOCK, 0, S.stream>>>(S.d, out);
    return 1;
}

// ------------------------------------------------------------------------------------ erosion

// erode, ExplicitSolver.java:663-691, for element e: its damage and signed current area
// decide whether it goes; the strain energy it held is added to energy.
// cur (when given) holds element_current(d, e).
__device__ __forceinline__ void erode_element(const Dev &d, int e, double &energy,
                                              const double2 *cur = nullptr) {
    if (d.gone[e]) return;
    {
        bool failed = false;
        if (d.hasDamage) {                                  // elementDamage, :1764-1772
            double sum = 0.0;
            for (int g = 0; g < d.ppe; g++) {
                const int p = e * d.ppe + g;
                sum += damage_at(d.dStrength[p], d.dSoft[p], d.dFail[e], d.epsP[p]);
            }
            failed = (d.ppe == 1 ? sum : sum / d.ppe) >= d.erosionDamage;   // x / 1 is x
        }
        double2 p[4];                                        // currentArea, :681-691
        if (cur) {
            for (int k = 0; k < 4; k++) p[k] = cur[k];
        } else {
            element_current(d, e, p);
        }
        double a = 0.0;
        for (int k = 0; k < 4; k++) {
            const double2 pi = p[k], pj = p[(k + 1) & 3];
            a += pi.x * pj.y - pj.x * pi.y;
        }
        // 0.5 a <= 0 by a's bits: a <= 0 (either zero, a negative number or -inf), or a the
        // least subnormal, whose half rounds to +0; NaN is neither
        const uint64_t ua = (uint64_t)__double_as_longlong(a);
        const bool inverted = (ua << 1) <= 2u || ((ua >> 63) && (ua << 1) <= 0xffe0000000000000ULL);
        if (failed || inverted) {
            d.gone[e] = 1;
            atomicAdd(&d.s->erodedCount, 1);
            if (inverted && !failed) atomicAdd(&d.s->invertedCount, 1);
            for (int g = 0; g < d.ppe; g++) energy += point_strain_energy(d, e, g);
            if (d.hasContact) {                              // Contact.forget, :329-332
                d.dead[e] = 1;
                d.s->stale = 1;
                d.newDead[atomicAdd(&d.s->newDeadCount, 1)] = e;   // at most E, ever
            }
        }
    }
}

__global__ void __launch_bounds__(BLOCK) k_erode(Dev d) {
    __shared__ double sh[BLOCK / 32];
    if (!d.s->active) return;
    double energy = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d.E; e += gridDim.x * blockDim.x)
        erode_element(d, e, energy);
    const double t = block_sum(energy, sh);
    if (threadIdx.x == 0) d.partials[PARTIAL_ERODE * d.maxBlocks + blockIdx.x] = t;
}

// ------------------------------------------------------------------------------------ element kernels

__device__ __forceinline__ void min_edge_commit(Dev &d, double minEdge) {
    for (int o = 16; o > 0; o >>= 1)
        minEdge = jmin_nonneg(minEdge, __shfl_down_sync(0xffffffffu, minEdge, o));
    if ((threadIdx.x & 31) == 0) atomicMin(&d.s->minEdgeBits, dbits(minEdge));
}

// reducedIntegration, ExplicitSolver.java:1373-1504
__global__ void __launch_bounds__(BLOCK) k_element_reduced(Dev d, int zeroStrain) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double minEdge = DMAX;
    if (e < d.E) {
        element_reduced(d, e, zeroStrain ? 0.0 : d.s->dt, d.hourglass, minEdge);
    }
    min_edge_commit(d, minEdge);
}

// reducedIntegration over the Johnson-Cook work list: threads [0, count) take the listed
// elements in list order (most expensive cost class first, so warps hold points of equal solve
// length and the longest start first), threads [count, count + E) take every element not
// listed; each element is computed once, by the same code as k_element_reduced. Each warp
// appends its points' cost classes for the next step's list. With `erode` the pass first
// decides each element's erosion (erode_element): an element's erosion reads only its own point
// and nodes, which no other element's update writes, so deciding it just before the element's
// own update is the same as a pass over all elements before any update.
__global__ void __launch_bounds__(BLOCK) k_element_reduced_listed(Dev d, int zeroStrain, int erode) {
    __shared__ double sh[BLOCK / 32];
    if (!d.s->active) return;
    const HotList *h = d.hot;
    const int listed = h->count;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    int e = -1;
    if (g < listed) {
        e = d.hotList[g];
    } else if (g - listed < d.E) {
        const int c = g - listed;
        if (d.hotStamp[c] != h->epoch) e = c;
    }
    double minEdge = DMAX, energy = 0.0;
    int cost = 0;
    if (e >= 0) {
        double2 cur[4];                  // x + u of the nodes, for the erosion test and cr/cz
        element_current(d, e, cur);
        if (erode) erode_element(d, e, energy, cur);
        element_reduced(d, e, zeroStrain ? 0.0 : d.s->dt, d.hourglass, minEdge, &cost, cur);
    }
    const unsigned want = __ballot_sync(0xffffffffu, cost > 0);
    if (want) {
        const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&d.hot->nextCount, __popc(want));
        base = __shfl_sync(0xffffffffu, base, leader);
        const int cls = min(cost, HOT_CLASSES - 1);
        const int pos = base + __popc(want & ((1u << lane) - 1u));
        const bool kept = cost > 0 && pos < d.hotCap;
        if (kept) d.hotNext[pos] = make_int2(e, cls);
        // the kept entries per class, one atomic per class present in the warp
        const int key = kept ? cls : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (kept && lane == __ffs(peers) - 1) atomicAdd(&d.hot->classCount[cls], __popc(peers));
    }
    min_edge_commit(d, minEdge);
    if (erode) {
        const double t = block_sum(energy, sh);
        if (threadIdx.x == 0) d.partials[PARTIAL_ERODE * d.maxBlocks + blockIdx.x] = t;
    }
}

// Dynamic shared memory (unused) that the listed pass requests so that at most two of its
// blocks share an SM: eight warps per SM keep the FP64 pipe busy, and a listed warp with a long
// Johnson-Cook solve competes with seven others for it instead of eleven. Needs the device
// current; sets the kernel's attribute.
__global__ void k_jc_yield(Dev d) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d.E; e += gridDim.x * blockDim.x) {
        const MatDev &f = d.mats[d.emat[e]];
        if (f.jc) d.jcYield[e] = jc_yield(f, d.epsP[e], d.wP[e]);
    }
}

void launch_jc_yield(const Dev &d, cudaStream_t st) {
    if (d.jcYield && d.E > 0) k_jc_yield<<<grid_for(d.E, BLOCK), BLOCK, 0, st>>>(d);
}

int listed_pass_smem(int device) {
    int perSm = 0, optin = 0;
    if (cudaDeviceGetAttribute(&perSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess)
        return 0;
    const int smem = perSm / 3 + 2048;
    if (smem > optin || 2 * (smem + 1024) > perSm) return 0;
    if (cudaFuncSetAttribute(k_element_reduced_listed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return 0;
    return smem;
}

constexpr int HOT_BATCH = 8;

// Blocks that build the work list: HOT_BATCH entries per thread of the longest list, at most
// two per SM.
static int hot_build_blocks(const Dev &d) {
    const int per = BLOCK * HOT_BATCH;
    const int want = (d.hotCap + per - 1) / per;
    return want < 1 ? 1 : want > 2 * d.sms ? 2 * d.sms : want;
}

// The next step's work list from the entries the pass appended: a counting sort by cost class,
// most expensive first; listed elements are stamped with the new epoch. Run by `blocks` blocks
// of the launch, this one being `block` of them.
__device__ void hot_build(const Dev &d, int block, int blocks) {
    __shared__ int start[HOT_CLASSES];
    __shared__ int last;
    HotList *h = d.hot;
    const int n = min(h->nextCount, d.hotCap);
    const int epoch = h->epoch + 1;
    if (threadIdx.x == 0) {                  // the pass counted the classes as it appended
        int acc = 0;
        for (int k = HOT_CLASSES - 1; k >= 0; k--) {
            start[k] = acc;
            acc += h->classCount[k];
        }
    }
    __syncthreads();
    // every block takes a run of entries; lanes of a warp holding the same class take their
    // positions in that class with one atomic on its global fill count (few classes, many
    // entries); each thread loads HOT_BATCH entries before using them, so their loads overlap
    const int lane = threadIdx.x & 31;
    const int stride = blocks * blockDim.x, span = HOT_BATCH * stride;
    for (int base = block * blockDim.x + threadIdx.x - lane; base < n; base += span) {
        int2 it[HOT_BATCH];
#pragma unroll
        for (int k = 0; k < HOT_BATCH; k++) {
            const int i = base + k * stride + lane;
            it[k] = i < n ? d.hotNext[i] : make_int2(-1, -1);
        }
#pragma unroll
        for (int k = 0; k < HOT_BATCH; k++) {
            const unsigned peers = __match_any_sync(0xffffffffu, it[k].y);
            const int leader = __ffs(peers) - 1;
            int first = 0;
            if (it[k].y >= 0 && lane == leader)
                first = start[it[k].y] + atomicAdd(&h->fill[it[k].y], __popc(peers));
            first = __shfl_sync(0xffffffffu, first, leader);
            if (it[k].y >= 0) {
                const int pos = first + __popc(peers & ((1u << lane) - 1u));
                d.hotList[pos] = it[k].x;
                d.hotStamp[it[k].x] = epoch;
            }
        }
    }
    // the last block to finish clears the counts for the pass that appends next
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&h->done, 1) == blocks - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int k = threadIdx.x; k < HOT_CLASSES; k += blockDim.x) {
        h->classCount[k] = 0;
        h->fill[k] = 0;
    }
    if (threadIdx.x == 0) {
        h->count = n;
        h->epoch = epoch;
        h->nextCount = 0;
        h->done = 0;
    }
}

// fullIntegration, ExplicitSolver.java:1219-1339
__global__ void __launch_bounds__(BLOCK) k_element_full(Dev d, int zeroStrain) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double minEdge = DMAX;
    if (e < d.E) {
        double *ef = d.contribution + 8 * (size_t)e;
        if (d.gone != nullptr && d.gone[e]) {
            for (int k = 0; k < 8; k++) ef[k] = 0.0;
        } else {
            const double strainDt = zeroStrain ? 0.0 : d.s->dt;
            const MatDev &fl = d.mats[d.emat[e]];
            const double lambda = fl.lambda, mu = fl.mu;
            const int4 c = d.conn[e];
            const double mid = -0.5 * strainDt;
            const double2 x0 = d.X0[c.x], x1 = d.X0[c.y], x2 = d.X0[c.z], x3 = d.X0[c.w];
            const double2 u0 = d.U[c.x], u1 = d.U[c.y], u2 = d.U[c.z], u3 = d.U[c.w];
            const double2 v0 = d.V[c.x], v1 = d.V[c.y], v2 = d.V[c.z], v3 = d.V[c.w];
            double r0, r1, r2, r3, z0, z1, z2, z3;
            if (d.finite) {
                r0 = x0.x + u0.x + mid * v0.x; r1 = x1.x + u1.x + mid * v1.x;
                r2 = x2.x + u2.x + mid * v2.x; r3 = x3.x + u3.x + mid * v3.x;
                z0 = x0.y + u0.y + mid * v0.y; z1 = x1.y + u1.y + mid * v1.y;
                z2 = x2.y + u2.y + mid * v2.y; z3 = x3.y + u3.y + mid * v3.y;
            } else {
                r0 = x0.x; r1 = x1.x; r2 = x2.x; r3 = x3.x;
                z0 = x0.y; z1 = x1.y; z2 = x2.y; z3 = x3.y;
            }
            const double a0 = v0.x * strainDt, a1 = v1.x * strainDt;
            const double a2 = v2.x * strainDt, a3 = v3.x * strainDt;
            const double c0 = v0.y * strainDt, c1 = v1.y * strainDt;
            const double c2 = v2.y * strainDt, c3 = v3.y * strainDt;

            if (d.finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);

            double g0r = 0, g1r = 0, g2r = 0, g3r = 0;
            double g0z = 0, g1z = 0, g2z = 0, g3z = 0;
            const double G = 0.5773502691896258;
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const double xi = (g == 0 || g == 3) ? -G : G;
                const double eta = (g < 2) ? -G : G;
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
                const double inv = 1.0 / det;

                const double d0r = (J11 * dN0x - J01 * dN0e) * inv;
                const double d1r = (J11 * dN1x - J01 * dN1e) * inv;
                const double d2r = (J11 * dN2x - J01 * dN2e) * inv;
                const double d3r = (J11 * dN3x - J01 * dN3e) * inv;
                const double d0z = (-J10 * dN0x + J00 * dN0e) * inv;
                const double d1z = (-J10 * dN1x + J00 * dN1e) * inv;
                const double d2z = (-J10 * dN2x + J00 * dN2e) * inv;
                const double d3z = (-J10 * dN3x + J00 * dN3e) * inv;

                const double dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
                const double dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
                const double dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
                const double dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
                const double dGamRZ = dRdZ + dZdR;

                double rg = 0.0, dEpsT = 0.0;
                if (d.axi) {
                    rg = N0 * r0 + N1 * r1 + N2 * r2 + N3 * r3;
                    dEpsT = (N0 * a0 + N1 * a1 + N2 * a2 + N3 * a3) / rg;
                }
                const int p = e * 4 + g;
                double sg[4], bk[4];
                {
                    const double2 *ps = reinterpret_cast<const double2 *>(d.sig + 4 * (size_t)p);
                    const double2 *pb = reinterpret_cast<const double2 *>(d.back + 4 * (size_t)p);
                    const double2 s01 = ps[0], s23 = ps[1], b01 = pb[0], b23 = pb[1];
                    sg[0] = s01.x; sg[1] = s01.y; sg[2] = s23.x; sg[3] = s23.y;
                    bk[0] = b01.x; bk[1] = b01.y; bk[2] = b23.x; bk[3] = b23.y;
                }
                if (d.finite) {
                    const double spinDt = 0.5 * (dZdR - dRdZ);
                    if (!is_zero(spinDt)) {
                        const double cs = corot_cos(spinDt), sn = corot_sin(spinDt);
                        corot_rotate(sg, cs, sn);
                        corot_rotate(bk, cs, sn);
                    }
                }
                double epsP = d.epsP[p], work = d.wP[p];
                if (d.hasDamage) {
                    DamageRef dr;
                    dr.failureStrain = d.dFail[e];
                    dr.strength = d.dStrength + p;
                    dr.softening = d.dSoft + p;
                    dr.width = d.dWidth + p;
                    dr.geometry = d.dGeom + 5 * (size_t)e;
                    dr.fractureEnergy = d.dGf[e];
                    dr.youngs = fl.youngs;
                    j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, lambda, mu, fl,
                              strainDt, &dr, d.dStrength[p], d.dSoft[p]);
                } else {
                    j2_update(sg, bk, epsP, work, dEpsR, dEpsZ, dEpsT, dGamRZ, lambda, mu, fl,
                              strainDt, (const DamageRef *)nullptr, 0.0, 0.0);
                }
                {
                    double2 *ps = reinterpret_cast<double2 *>(d.sig + 4 * (size_t)p);
                    double2 *pb = reinterpret_cast<double2 *>(d.back + 4 * (size_t)p);
                    ps[0] = make_double2(sg[0], sg[1]); ps[1] = make_double2(sg[2], sg[3]);
                    pb[0] = make_double2(bk[0], bk[1]); pb[1] = make_double2(bk[2], bk[3]);
                    d.epsP[p] = epsP;
                    d.wP[p] = work;
                }
                const double sR = sg[0], sZ = sg[1], sT = sg[2], sRZ = sg[3];
                const double dV = d.axi ? 2.0 * NF_PI * rg * det : d.thickness * det;
                if (d.axi) {
                    const double hh = sT / rg * dV;
                    g0r -= (d0r * sR + d0z * sRZ) * dV + N0 * hh;
                    g1r -= (d1r * sR + d1z * sRZ) * dV + N1 * hh;
                    g2r -= (d2r * sR + d2z * sRZ) * dV + N2 * hh;
                    g3r -= (d3r * sR + d3z * sRZ) * dV + N3 * hh;
                } else {
                    g0r -= (d0r * sR + d0z * sRZ) * dV;
                    g1r -= (d1r * sR + d1z * sRZ) * dV;
                    g2r -= (d2r * sR + d2z * sRZ) * dV;
                    g3r -= (d3r * sR + d3z * sRZ) * dV;
                }
                g0z -= (d0z * sZ + d0r * sRZ) * dV;
                g1z -= (d1z * sZ + d1r * sRZ) * dV;
                g2z -= (d2z * sZ + d2r * sRZ) * dV;
                g3z -= (d3z * sZ + d3r * sRZ) * dV;
            }
            double2 *ef2 = reinterpret_cast<double2 *>(ef);
            ef2[0] = make_double2(g0r, g1r);
            ef2[1] = make_double2(g2r, g3r);
            ef2[2] = make_double2(g0z, g1z);
            ef2[3] = make_double2(g2z, g3z);
        }
    }
    min_edge_commit(d, minEdge);
}

// ------------------------------------------------------------------------------------ pressure

// applyPressure + pressureAt, ExplicitSolver.java:1203-1207, :1511-1556
__global__ void k_pressure(Dev d) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.K) return;
    pressure_edge(d, e, d.s->time, d.targetPressure, d.rampDuration);
}

// ------------------------------------------------------------------------------------ gather

// gather, ExplicitSolver.java:1147-1165: ascending source order, then gravity. With a work
// list, the launch's first listBlocks blocks build the next step's list instead, and with
// contact the next block rebuilds the surface after this step's erosion when few elements
// eroded (the three read and write disjoint data; the contact pass, next on the stream, reads
// the surface). One launch saves kernel boundaries, and the rebuild runs beside the gather
// instead of as two barrier-separated phases of the contact pass.
__global__ void __launch_bounds__(BLOCK) k_gather(Dev d, int listBlocks, int surfaceBlock) {
    DevScalars *s = d.s;
    if (!s->active) return;
    if ((int)blockIdx.x < listBlocks) {
        hot_build(d, blockIdx.x, listBlocks);
        return;
    }
    if (surfaceBlock && (int)blockIdx.x == listBlocks) {
        if (s->stale && !s->fullRebuild && s->newDeadCount <= SURFACE_BLOCK_DEAD)
            surface_rebuild_block(d);
        return;
    }
    const int n = (blockIdx.x - listBlocks - surfaceBlock) * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    d.F[n] = gather_node(d, n);
    if (d.hasContact) d.contactState[n] = 0;
}

// ------------------------------------------------------------------------------------ end of step

// Deterministic sums of the per-block partials: lane l of a warp adds partials l, l + 32, ...
// in that order, then the warp's fixed tree adds the lanes. Same inputs, same result.

// Folds the block partials, then the adaptive CFL step (:985-990).
constexpr int END_WARPS_PER_LIST = 5;         // k_end: 6 lists x 5 warps of its 32
__global__ void __launch_bounds__(1024) k_end(Dev d, int nodeBlocks, int elemBlocks,
                                             int slotBlocks, int updateDt) {
    __shared__ double part[6][END_WARPS_PER_LIST];
    __shared__ double folded[6];
    DevScalars *s = d.s;
    if (!s->active) return;
    // the six per-block partial lists, five warps each: warp w of a list takes the w-th of five
    // contiguous runs of it, each lane adds its terms lane-strided in order, the warp's fixed
    // tree adds the lanes, and the five runs are added in order -- a fixed order, so the totals
    // are deterministic
    {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int list = warp / END_WARPS_PER_LIST, run = warp % END_WARPS_PER_LIST;
        const double *src = nullptr;
        int count = 0;
        if (list < 3 && updateDt && d.hasWall) {
            src = d.partials + (PARTIAL_WALL + list) * d.maxBlocks;
            count = nodeBlocks;
        } else if (list == 3 && updateDt && d.hasErosion) {
            src = d.partials + PARTIAL_ERODE * d.maxBlocks;
            count = elemBlocks;
        } else if ((list == 4 || list == 5) && d.hasContact) {
            src = d.partials + (PARTIAL_CONTACT + list - 4) * d.maxBlocks;
            count = slotBlocks;
        }
        const int chunk = (count + END_WARPS_PER_LIST - 1) / END_WARPS_PER_LIST;
        const int lo = min(count, run * chunk), hi = min(count, lo + chunk);
        // each lane adds the terms lo + lane, + 32, + 64, ... in that order, eight loads at a
        // time. The loop runs the same number of times in every lane of the warp (positions at
        // or past hi read as +0), so the warp vote inside it is taken by all 32 lanes. A batch
        // of +0s in every lane is skipped: v starts at +0 and a sum of doubles only reaches -0
        // from -0 terms, so adding +0 never changes it (most blocks' wall and erosion terms
        // are +0)
        double v = 0.0;
        for (int base = lo; base < hi; base += 8 * 32) {
            double x[8];
            long long any = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int k = base + lane + 32 * j;
                x[j] = k < hi ? src[k] : 0.0;
                any |= __double_as_longlong(x[j]);
            }
            if (__any_sync(0xffffffffu, any != 0)) {
#pragma unroll
                for (int j = 0; j < 8; j++) v += x[j];
            }
        }
        if (__any_sync(0xffffffffu, __double_as_longlong(v) != 0))
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && list < 6) part[list][run] = v;
        __syncthreads();
        if (threadIdx.x < 6) {
            double t = 0.0;
            for (int r = 0; r < END_WARPS_PER_LIST; r++) t += part[threadIdx.x][r];
            folded[threadIdx.x] = t;
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double w0 = folded[0], w1 = folded[1], w2 = folded[2], er = folded[3];
    const double c0 = folded[4], c1 = folded[5];
    if (updateDt && d.hasWall) {
        s->wImpulse += w0;
        s->wEnergyLoss += w1;
        s->wFriction += w2;
        s->wContact = s->wContactAcc;
        s->wStuck = s->wStuckAcc;
        s->wContactAcc = 0;
        s->wStuckAcc = 0;
    }
    if (updateDt && d.hasErosion) s->erodedEnergy += er;
    if (d.hasContact) {
        s->cEnergy = c0;
        s->cDissipation += c1;
    }
    const double minEdge = bitsd(s->minEdgeBits);
    s->minEdgeSquared = minEdge;
    s->minEdgeBits = dbits(DMAX);
    if (updateDt) {
        if (d.finite) {
            s->dtPrevious = s->dt;
            s->dt = d.cfl * sqrt(minEdge * d.massScale) / d.fastestWave;
        }
        s->stepsTaken += 1;
    }
    // the next step's run predicate (its kernels all read it)
    s->active = s->time < s->tEnd && s->stepsTaken < s->maxSteps ? 1 : 0;
}

// advance(), ExplicitSolver.java:1069-1075: displacement from the current velocity, no
// velocity update.
__global__ void k_advance_nodes(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const uint8_t fl = d.flags[i];
    const double dt = d.s->dt;
    double2 u = d.U[i];
    const double2 v = d.V[i];
    if (!(fl & 1)) u.x += v.x * dt;
    if (!(fl & 2)) u.y += v.y * dt;
    d.U[i] = u;
}

__global__ void k_set_active(Dev d) {
    d.s->active = 1;
    contact_step_reset(d.s);
}

// ------------------------------------------------------------------------------------ launch

// The one-point element pass erodes too (one pass instead of two over the elements) when the
// step erodes and the pass is the FP64 listed one or the mixed one; its blocks then hold the
// eroded-energy partials.
static bool erosion_fused(const Dev &d) {
    return d.hasErosion && d.E > 0 && !d.full && (d.mixed || d.hot);
}
static int eroding_blocks(const Solver &S) {
    if (!erosion_fused(S.d)) return element_grid(S);
    return S.d.mixed ? grid_for(S.d.E, 128) : grid_for((long long)S.d.E + S.d.hotCap, BLOCK);
}

static int assemble(Solver &S, int zeroStrain, bool prepared = false, bool erode = false) {
    Dev &d = S.d;
    const cudaStream_t st = S.stream;
    int n = 0;
    S.mark(NF_GROUP_ELEMENT, true);
    if (d.mixed) {
        if (!prepared) n += launch_prepare_mixed(S, zeroStrain);
        n += launch_element_mixed(S, zeroStrain, erode);
    } else if (d.E > 0) {
        if (d.full) {
            k_element_full<<<grid_for(d.E, BLOCK), BLOCK, 0, st>>>(d, zeroStrain);
            n++;
        } else if (d.hot) {
            k_element_reduced_listed<<<grid_for((long long)d.E + d.hotCap, BLOCK), BLOCK,
                                       d.hotSmem, st>>>(d, zeroStrain, erode ? 1 : 0);
            n++;
        } else {
            k_element_reduced<<<grid_for(d.E, BLOCK), BLOCK, 0, st>>>(d, zeroStrain);
            n++;
        }
    }
    S.mark(NF_GROUP_ELEMENT, false);
    if (d.K > 0) {
        S.mark(NF_GROUP_PRESSURE, true);
        if (d.mixed) n += launch_pressure_mixed(S);
        else {
            k_pressure<<<grid_for(d.K, BLOCK), BLOCK, 0, st>>>(d);
            n++;
        }
        S.mark(NF_GROUP_PRESSURE, false);
    }
    S.mark(NF_GROUP_GATHER, true);
    // the listed element pass's work list is built by the gather's launch (or alone)
    const int listBlocks = !d.mixed && d.E > 0 && !d.full && d.hot ? hot_build_blocks(d) : 0;
    if (d.N > 0 && !d.mixed) {
        const int surfaceBlock = d.hasContact ? 1 : 0;
        k_gather<<<listBlocks + surfaceBlock + grid_for(d.N, BLOCK), BLOCK, 0, st>>>(
            d, listBlocks, surfaceBlock);
        n++;
    } else {
        if (d.N > 0) n += launch_gather_mixed(S);
        if (listBlocks) {
            k_gather<<<listBlocks, BLOCK, 0, st>>>(d, listBlocks, 0);
            n++;
        }
    }
    S.mark(NF_GROUP_GATHER, false);
    if (d.hasContact) {
        S.mark(NF_GROUP_CONTACT, true);
        n += launch_contact(S, true);
        S.mark(NF_GROUP_CONTACT, false);
    }
    return n;
}

int launch_initial_assembly(Solver &S) {
    Dev &d = S.d;
    k_begin<<<1, 1, 0, S.stream>>>(d);
    int n = 1 + assemble(S, 1);
    k_end<<<1, 1024, 0, S.stream>>>(d, nodal_grid(S), element_grid(S), d.coopBlocks, 0);
    return n + 1;
}

int launch_step(Solver &S, bool) {
    Dev &d = S.d;
    const cudaStream_t st = S.stream;
    int n = 0;
    S.mark(NF_GROUP_NODAL, true);
    if (d.N > 0) {
        k_nodal<<<nodal_grid(S), BLOCK, 0, st>>>(d);    // in the mixed form it also prepares
        n++;
    }
    S.mark(NF_GROUP_NODAL, false);
    const bool fused = erosion_fused(d);
    if (d.hasErosion && d.E > 0 && !fused) {
        S.mark(NF_GROUP_ERODE, true);
        if (d.mixed) n += launch_erode_mixed(S);
        else {
            k_erode<<<element_grid(S), BLOCK, 0, st>>>(d);
            n++;
        }
        S.mark(NF_GROUP_ERODE, false);
    }
    n += assemble(S, 0, d.N > 0 && d.mixed, fused);
    S.mark(NF_GROUP_END, true);
    k_end<<<1, 1024, 0, st>>>(d, nodal_grid(S), eroding_blocks(S), d.coopBlocks, 1);
    n++;
    S.mark(NF_GROUP_END, false);
    return n;
}

int launch_advance(Solver &S) {
    Dev &d = S.d;
    k_set_active<<<1, 1, 0, S.stream>>>(d);
    int n = 1;
    if (d.N > 0) {
        k_advance_nodes<<<grid_for(d.N, BLOCK), BLOCK, 0, S.stream>>>(d);
        n++;
    }
    n += assemble(S, 0);
    k_end<<<1, 1024, 0, S.stream>>>(d, nodal_grid(S), element_grid(S), d.coopBlocks, 0);
    return n + 1;
}

// Event bracketing of kernel groups while profiling (nf_profile).
void Solver::mark(int group, bool begin) {
    if (!profiling) return;
    if (begin) {
        Rec r{group, nullptr, nullptr};
        cudaEventCreate(&r.a);
        cudaEventCreate(&r.b);
        cudaEventRecord(r.a, stream);
        recs.push_back(r);
    } else {
        cudaEventRecord(recs.back().b, stream);
    }
}

// ------------------------------------------------------------------------------------ audits

enum {
    A_KE, A_CKE, A_PZ, A_PR, A_SE, A_WP, A_FD, A_HG, A_COUNT
};

// Node audits (ExplicitSolver.java:875-886, :1610-1640), reduced per block.
__global__ void __launch_bounds__(BLOCK) k_audit_nodes(Dev d, double *out) {
    __shared__ double sh[BLOCK / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0, cke = 0, pz = 0, pr = 0;
    if (i < d.N) {
        const double hh = 0.5 * d.s->dt;
        const double m = d.mass[i];
        const double invM = 1.0 / m;
        const uint8_t fl = d.flags[i];
        const double2 v = d.V[i], f = d.F[i];
        const bool held = d.hasWall && (fl & 4) && f.y <= 0.0;
        const double cvr = (fl & 1) ? v.x : v.x + hh * f.x * invM;
        const double cvz = ((fl & 2) || held) ? v.y : v.y + hh * f.y * invM;
        cke = 0.5 * m * (cvr * cvr + cvz * cvz);
        ke = m * (v.x * v.x + v.y * v.y);
        pz = m * v.y;
        pr = m * v.x;
    }
    const double a = block_sum(ke, sh), b = block_sum(cke, sh);
    const double c = block_sum(pz, sh), e = block_sum(pr, sh);
    if (threadIdx.x == 0) {
        out[4 * blockIdx.x + 0] = a;
        out[4 * blockIdx.x + 1] = b;
        out[4 * blockIdx.x + 2] = c;
        out[4 * blockIdx.x + 3] = e;
    }
}

// Point audits (:1654-1860), reduced per block: SE, Wp V, fracture, hourglass, max eps,
// yielded, max damage, begun, failed, clamped, max temperature (-1 marks no thermal model).
__global__ void __launch_bounds__(BLOCK) k_audit_points(Dev d, double *out) {
    __shared__ double sh[BLOCK / 32];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double se = 0, wp = 0, fd = 0, hg = 0, mx = 0, yielded = 0, md = 0, begun = 0, failed = 0,
           clamped = 0, tmax = -INFINITY;
    if (e < d.E) {
        const MatDev &m = d.mats[d.emat[e]];
        for (int g = 0; g < d.ppe; g++) {
            const int p = e * d.ppe + g;
            const double vol = gauss_volume(d, e, g);
            if (!(d.gone != nullptr && d.gone[e])) se += point_strain_energy(d, e, g);
            wp += d.wP[p] * vol;
            const double ep = d.epsP[p];
            if (ep > mx) mx = ep;
            if (ep > 0.0) yielded += 1.0;
            if (d.hasDamage) {
                const double sf = d.dStrength[p], slope = d.dSoft[p];
                if (sf > 0.0) {
                    const double full = -sf / slope;
                    double excess = ep - d.dFail[e];
                    double diss = 0.0;
                    if (excess > 0.0) {
                        if (excess > full) excess = full;
                        diss = excess * (sf + 0.5 * slope * excess);
                    }
                    fd += diss * vol;
                    begun += 1.0;
                }
                const double dm = damage_at(sf, slope, d.dFail[e], ep);
                if (dm > md) md = dm;
                if (dm >= 1.0) failed += 1.0;
                if (slope == -m.youngs) clamped += 1.0;
            }
            if (m.jc) {
                const double t = m.room + m.tq * d.wP[p] / (m.density * m.cp);
                tmax = jmax(tmax, t);
            } else {
                tmax = NAN;
            }
        }
        if (!d.full && d.hourglass != 0.0) {
            const double k = d.hgK[e];
            const double2 q = d.hg[e];
            if (k > 0.0) hg = 0.5 * (q.x * q.x + q.y * q.y) / k;
        }
    }
    const double r0 = block_sum(se, sh), r1 = block_sum(wp, sh), r2 = block_sum(fd, sh);
    const double r3 = block_sum(hg, sh), r4 = block_sum(yielded, sh), r5 = block_sum(begun, sh);
    const double r6 = block_sum(failed, sh), r7 = block_sum(clamped, sh);
    // maxima: exact, any order
    __shared__ double smx[BLOCK], smd[BLOCK], stm[BLOCK];
    smx[threadIdx.x] = mx; smd[threadIdx.x] = md; stm[threadIdx.x] = tmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0, c = -INFINITY;
        for (int k = 0; k < blockDim.x; k++) {
            if (smx[k] > a) a = smx[k];
            if (smd[k] > b) b = smd[k];
            c = jmax(c, stm[k]);
        }
        double *o = out + 12 * blockIdx.x;
        o[0] = r0; o[1] = r1; o[2] = r2; o[3] = r3; o[4] = r4; o[5] = r5; o[6] = r6; o[7] = r7;
        o[8] = a; o[9] = b; o[10] = c;
        // most damaged element: first element (lowest index) holding this block's max damage
        int worst = -1;
        double wv = 0.0;
        for (int k = 0; k < blockDim.x; k++) {
            const int el = blockIdx.x * blockDim.x + k;
            if (el >= d.E || !d.hasDamage) break;
            for (int g = 0; g < d.ppe; g++) {
                const int p = el * d.ppe + g;
                const double dm = damage_at(d.dStrength[p], d.dSoft[p], d.dFail[el], d.epsP[p]);
                if (dm > wv) { wv = dm; worst = el; }
            }
        }
        o[11] = (double)worst;
    }
}

size_t audit_partial_doubles(const Dev &d) {
    return 4 * (size_t)grid_for(d.N, BLOCK) + 12 * (size_t)grid_for(d.E, BLOCK);
}

void launch_audit_partials(Solver &S, double *buf) {
    Dev &d = S.d;
    const int nb = grid_for(d.N, BLOCK), eb = grid_for(d.E, BLOCK);
    k_audit_nodes<<<nb, BLOCK, 0, S.stream>>>(d, buf);
    k_audit_points<<<eb, BLOCK, 0, S.stream>>>(d, buf + 4 * (size_t)nb);
}

void reduce_audit_partials(const Solver &S, const double *h, nf_audit *o) {
    const Dev &d = S.d;
    const int nb = grid_for(d.N, BLOCK), eb = grid_for(d.E, BLOCK);
    memset(o, 0, sizeof *o);
    for (int b = 0; b < nb; b++) {
        o->kinetic_energy += h[4 * b + 0];
        o->centred_kinetic_energy += h[4 * b + 1];
        o->axial_momentum += h[4 * b + 2];
        o->radial_momentum += h[4 * b + 3];
    }
    o->kinetic_energy *= 0.5;
    double yielded = 0, begun = 0, failed = 0, clamped = 0, tmax = -INFINITY;
    double worstVal = 0.0;
    int worst = -1;
    const double *p = h + 4 * (size_t)nb;
    for (int b = 0; b < eb; b++) {
        const double *q = p + 12 * (size_t)b;
        o->strain_energy += q[0];
        o->plastic_dissipation += q[1];
        o->fracture_dissipation += q[2];
        o->hourglass_energy += q[3];
        yielded += q[4]; begun += q[5]; failed += q[6]; clamped += q[7];
        if (q[8] > o->max_plastic_strain) o->max_plastic_strain = q[8];
        if (q[9] > worstVal) { worstVal = q[9]; worst = (int)q[11]; }
        if (q[9] > o->max_damage) o->max_damage = q[9];
        if (std::isnan(q[10]) || std::isnan(tmax)) tmax = NAN;
        else if (q[10] > tmax) tmax = q[10];
    }
    const double P = (double)d.E * d.ppe;
    o->yielded_fraction = yielded / P;
    o->damaged_fraction = d.hasDamage ? begun / P : 0.0;
    o->failed_fraction = d.hasDamage ? failed / P : 0.0;
    o->clamped_points = (int32_t)clamped;
    o->max_temperature = tmax;
    o->most_damaged_element = d.hasDamage ? worst : -1;
    if (S.integration == NF_FULL || S.hourglass == 0.0) o->hourglass_energy = 0.0;
}

void launch_audits(Solver &S, nf_audit *o) {
    const size_t n = audit_partial_doubles(S.d);
    double *buf = nullptr;
    cudaMalloc(&buf, sizeof(double) * n);
    launch_audit_partials(S, buf);
    std::vector<double> h(n);
    cudaMemcpyAsync(h.data(), buf, sizeof(double) * n, cudaMemcpyDeviceToHost, S.stream);
    cudaStreamSynchronize(S.stream);
    cudaFree(buf);
    reduce_audit_partials(S, h.data(), o);
}

// Body measurements (TaylorImpactCase.java:272-288): exact extrema, any order.
__global__ void k_measure(Dev d, unsigned long long *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const double2 x = d.X0[i], u = d.U[i];
    const double zc = x.y + u.y;
    const double rc = x.x + u.x;
    // order-preserving integer images of doubles
    auto key = [](double v) -> unsigned long long {
        const unsigned long long b = dbits(v);
        return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
    };
    atomicMax(&out[0], key(zc));
    atomicMin(&out[1], key(zc));
    atomicMax(&out[2], key(rc));
}

static double unkey(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    double v;
    memcpy(&v, &b, 8);
    return v;
}

void launch_measure(Solver &S, nf_measure *o) {
    Dev &d = S.d;
    unsigned long long *buf = nullptr;
    cudaMalloc(&buf, 3 * sizeof(unsigned long long));
    unsigned long long init[3] = {0ULL, ~0ULL, 0ULL};
    cudaMemcpyAsync(buf, init, sizeof init, cudaMemcpyHostToDevice, S.stream);
    if (d.N > 0) k_measure<<<grid_for(d.N, BLOCK), BLOCK, 0, S.stream>>>(d, buf);
    unsigned long long h[3];
    cudaMemcpyAsync(h, buf, sizeof h, cudaMemcpyDeviceToHost, S.stream);
    cudaStreamSynchronize(S.stream);
    cudaFree(buf);
    o->z_max = d.N ? unkey(h[0]) : -INFINITY;
    o->z_min = d.N ? unkey(h[1]) : INFINITY;
    o->length = o->z_max - o->z_min;
    const double rmax = d.N ? unkey(h[2]) : 0.0;
    o->mushroom_diameter = 2.0 * (rmax > 0.0 ? rmax : 0.0);
}

// ------------------------------------------------------------------------------------ material points

__global__ void k_material_points(MatDev m, int count, double *sig, double *back, double *epsP,
                                  double *work, const double *strain, double strainDt,
                                  const double *fail, const double *gf, const double *youngs,
                                  const double *geom, double *strength, double *soft,
                                  double *width, double *dgamma) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    double sg[4] = {sig[4 * p], sig[4 * p + 1], sig[4 * p + 2], sig[4 * p + 3]};
    double bk[4] = {back[4 * p], back[4 * p + 1], back[4 * p + 2], back[4 * p + 3]};
    double ep = epsP[p], w = work[p];
    double g;
    if (fail != nullptr) {
        DamageRef dr;
        dr.failureStrain = fail[p];
        dr.strength = strength + p;
        dr.softening = soft + p;
        dr.width = width + p;
        dr.geometry = geom + 5 * (size_t)p;
        dr.fractureEnergy = gf[p];
        dr.youngs = youngs[p];
        g = j2_update(sg, bk, ep, w, strain[4 * p], strain[4 * p + 1], strain[4 * p + 2],
                      strain[4 * p + 3], m.lambda, m.mu, m, strainDt, &dr, strength[p], soft[p]);
    } else {
        g = j2_update(sg, bk, ep, w, strain[4 * p], strain[4 * p + 1], strain[4 * p + 2],
                      strain[4 * p + 3], m.lambda, m.mu, m, strainDt, (const DamageRef *)nullptr, 0.0, 0.0);
    }
    for (int k = 0; k < 4; k++) { sig[4 * p + k] = sg[k]; back[4 * p + k] = bk[k]; }
    epsP[p] = ep;
    work[p] = w;
    dgamma[p] = g;
}

void launch_material_points(const MatDev &m, int count, double *sig, double *back, double *epsP,
                            double *work, const double *strain, double strainDt,
                            const double *fail, const double *gf, const double *youngs,
                            const double *geom, double *strength, double *soft, double *width,
                            double *dgamma, cudaStream_t stream) {
    if (count <= 0) return;
    k_material_points<<<grid_for(count, BLOCK), BLOCK, 0, stream>>>(
        m, count, sig, back, epsP, work, strain, strainDt, fail, gf, youngs, geom, strength,
        soft, width, dgamma);
}

}  // namespace nf
