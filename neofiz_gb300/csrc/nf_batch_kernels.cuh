// nf_batch_kernels.cuh -- the persistent batched kernel (k_batch.cu), as templates: the FP64
// and mixed forms are instantiated in k_batch.cu, the compensated form in k_batch_comp.cu,
// which is compiled with float contraction and fast float division and square root.
#pragma once

#include "nf_batch_step.cuh"

namespace nf {

// Up to `chunk` steps of instance k by the whole block: ExplicitSolver.step, :940-991, with the
// loop condition of TaylorImpactCase.java:250-253 (step while time < t_end).
// An instance's displacement and centroid hoop stress in the batch's precision.
template <bool MIXED, bool COMP>
__device__ __forceinline__ double2 inst_u(const Dev &d, int i) {
    if (COMP) {
        const float4 u = d.uC[i];
        return make_double2((double)u.x + (double)u.y, (double)u.z + (double)u.w);
    }
    return d.U[i];
}
template <bool MIXED>
__device__ __forceinline__ double inst_hoop(const Dev &d, int e) {
    // centroidStress(e)[2] (ExplicitSolver.java:1886-1894) of a one-point element
    return MIXED ? (double)d.sigF[4 * (size_t)e + 2] : d.sig[4 * (size_t)e + 2];
}

// One sample of BurstCase.run (BurstCase.java:449-490) for instance k by the whole block:
// loadCapacity (:533-553, the hoop stress times the element area summed in element order by
// thread 0), hoopStrain (:560-569), the applied pressure (borePressure, pressureAt
// :1203-1207), the running peak and the turnover test. Returns whether the peak was
// traversed (the same answer in every thread).
template <bool MIXED, bool COMP, int T>
__device__ bool burst_sample(const Dev &d, const BatchDev &b, const BatchInst &in, int k,
                             double time, double *sh) {
    __shared__ double ext[5][T / 32];
    __shared__ int verdict;
    const BurstDev &bd = b.burst;
    const bool finite = d.finite != 0;
    for (int e = in.e0 + threadIdx.x; e < in.e1; e += T) {
        const int4 c = d.conn[e];
        const int nn[4] = {c.x, c.y, c.z, c.w};
        double sum = 0.0;
        for (int q = 0; q < 4; q++) {
            const int i = nn[q], j = nn[(q + 1) & 3];
            const double2 xi = d.X0[i], xj = d.X0[j];
            double ri = xi.x, rj = xj.x, zi = xi.y, zj = xj.y;
            if (finite) {
                const double2 ui = inst_u<MIXED, COMP>(d, i), uj = inst_u<MIXED, COMP>(d, j);
                ri = xi.x + ui.x; rj = xj.x + uj.x; zi = xi.y + ui.y; zj = xj.y + uj.y;
            }
            sum += ri * zj - rj * zi;
        }
        bd.scratch[e] = inst_hoop<MIXED>(d, e) * (0.5 * sum);
    }
    // extrema, exact in any order: loadCapacity's bore, low, high; hoopStrain's bore, rim
    double bore = DMAX, low = DMAX, high = -DMAX, boreH = DMAX, rimH = -DMAX;
    for (int i = in.n0 + threadIdx.x; i < in.n1; i += T) {
        const double2 x = d.X0[i], u = inst_u<MIXED, COMP>(d, i);
        const double r = finite ? x.x + u.x : x.x, z = finite ? x.y + u.y : x.y;
        bore = fmin(bore, r);
        low = fmin(low, z);
        high = fmax(high, z);
        boreH = fmin(boreH, x.x + u.x);
        rimH = fmax(rimH, x.x + u.x);
    }
    for (int o = 16; o > 0; o >>= 1) {
        bore = fmin(bore, __shfl_down_sync(0xffffffffu, bore, o));
        low = fmin(low, __shfl_down_sync(0xffffffffu, low, o));
        high = fmax(high, __shfl_down_sync(0xffffffffu, high, o));
        boreH = fmin(boreH, __shfl_down_sync(0xffffffffu, boreH, o));
        rimH = fmax(rimH, __shfl_down_sync(0xffffffffu, rimH, o));
    }
    if ((threadIdx.x & 31) == 0) {
        const int w = threadIdx.x >> 5;
        ext[0][w] = bore; ext[1][w] = low; ext[2][w] = high; ext[3][w] = boreH; ext[4][w] = rimH;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < T / 32; w++) {
            bore = fmin(bore, ext[0][w]);
            low = fmin(low, ext[1][w]);
            high = fmax(high, ext[2][w]);
            boreH = fmin(boreH, ext[3][w]);
            rimH = fmax(rimH, ext[4][w]);
        }
        double hoopArea = 0.0;
        for (int e = in.e0; e < in.e1; e++) hoopArea += bd.scratch[e];
        const double capacity = hoopArea / (bore * (high - low));
        const double strain = nf_log(0.5 * (boreH + rimH) / bd.meanRadius[k]);
        double applied = in.pressure;
        if (in.ramp > 0.0) {
            const double s = jmin(1.0, time / in.ramp);
            applied = in.pressure * s * s * (3.0 - 2.0 * s);
        }
        BurstState &st = bd.state[k];
        if (bd.traceCap > 0 && st.samples < bd.traceCap) {
            double *t = bd.trace + 4 * ((size_t)k * bd.traceCap + st.samples);
            t[0] = time; t[1] = strain; t[2] = capacity; t[3] = applied;
        }
        st.samples += 1;
        st.capacity = capacity;
        st.strain = strain;
        st.applied = applied;
        if (capacity > st.peakCapacity) {
            st.peakCapacity = capacity;
            st.peakStrain = strain;
            st.peakApplied = applied;
        } else if (applied >= in.pressure && capacity < st.peakCapacity * (1.0 - bd.margin)) {
            st.traversed = 1;                  // past the peak, and past the end of the ramp
        }
        verdict = st.traversed;
    }
    __syncthreads();
    const bool out = verdict != 0;
    __syncthreads();
    return out;
}

template <bool MIXED, bool STAGE, int T, bool COMP>
__device__ void run_instance(const Dev &d, const BatchDev &b, int k, int chunk, float4 *sPMid,
                             float2 *sVdt, double *shMin, int (*wallCount)[2], BlockStep *bs) {
    const BatchInst in = b.inst[k];
    BatchScalars *scp = b.sc + k;
    if (scp->done) return;
    const int tid = threadIdx.x;
    double dt = scp->dt, dtPrev = scp->dtPrevious, time = scp->time;
    double minEdge = scp->minEdgeSquared;
    long long steps = scp->steps;
    const long long limit = scp->stepLimit;
    double impulse = 0.0, loss = 0.0, fric = 0.0;
    if (tid == 0) {
        wallCount[0][0] = wallCount[0][1] = 0;
        wallCount[1][0] = wallCount[1][1] = 0;
        block_step_init(*bs, d, in, dt, dtPrev);
    }
    __syncthreads();
    float4 *pMid = STAGE ? sPMid : d.pMid;
    float2 *vdt = STAGE ? sVdt : d.vdt;
    const int base = STAGE ? in.n0 : 0;
    const MixedGeo geo = MIXED ? MixedGeo{pMid, nullptr, vdt, -base}
                               : MixedGeo{nullptr, nullptr, nullptr, 0};
    // burst mode: the run stops only at sample points (BurstCase.java:446-449: run a whole
    // sample's steps, then test the deadline) or once the peak is traversed
    const int every = b.burst.every;
    bool traversed = every > 0 && b.burst.state[k].traversed;
    int taken = 0;
    for (; taken < chunk; taken++) {
        if (traversed || steps >= limit) break;
        if ((every == 0 || steps % every == 0) && !(time < in.tEnd)) break;
        // RigidWall.beginStep: this step's counts go to buffer `par`; the other is cleared for
        // the next step (its last users passed this step's first barrier already)
        const int par = taken & 1;
        if (tid == 0) {
            wallCount[par ^ 1][0] = 0;
            wallCount[par ^ 1][1] = 0;
        }
        minEdge = batch_step<MIXED, T, COMP>(d, in, dt, dtPrev, time, steps, geo, pMid, vdt,
                                             base, &scp->status, &wallCount[par][0],
                                             &wallCount[par][1], impulse, loss, fric, shMin,
                                             bs);
        if (every > 0 && steps % every == 0)
            traversed = burst_sample<MIXED, COMP, T>(d, b, in, k, time, shMin);
    }
    const double ti = block_total<T>(impulse, shMin);
    const double tl = block_total<T>(loss, shMin);
    const double tf = block_total<T>(fric, shMin);
    if (tid == 0) {
        scp->dt = dt;
        scp->dtPrevious = dtPrev;
        scp->time = time;
        scp->steps = steps;
        scp->minEdgeSquared = minEdge;
        if (taken > 0) {
            scp->wContact = wallCount[(taken - 1) & 1][0];
            scp->wStuck = wallCount[(taken - 1) & 1][1];
        }
        scp->wImpulse += ti;
        scp->wEnergyLoss += tl;
        scp->wFriction += tf;
        const bool ended = every > 0 ? (steps % every == 0 && !(time < in.tEnd))
                                     : !(time < in.tEnd);
        if (ended || traversed || steps >= limit) {
            scp->done = 1;
            atomicSub(b.remaining, 1);
        }
    }
    __syncthreads();
}

// The queue loop of the persistent kernel: each block takes the next instance (most
// expensive first) for a chunk of steps until none is left.
template <bool MIXED, bool STAGE, int T, bool COMP>
__device__ __forceinline__ void batch_queue(const Dev &d, const BatchDev &b, int chunk) {
    extern __shared__ __align__(16) unsigned char dyn[];
    __shared__ double shMin[T / 32 + 1];
    __shared__ int wallCount[2][2];
    __shared__ int next;
    __shared__ BlockStep bs;
    float4 *sPMid = reinterpret_cast<float4 *>(dyn);
    float2 *sVdt = reinterpret_cast<float2 *>(dyn + sizeof(float4) * (size_t)b.maxNodes);
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(b.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= b.count) return;
        run_instance<MIXED, STAGE, T, COMP>(d, b, b.order[q], chunk, sPMid, sVdt, shMin,
                                            wallCount, &bs);
    }
}

// The FP64 and mixed forms (the compiler's register choice).
template <bool MIXED, bool STAGE, int T>
__global__ void __launch_bounds__(T) k_batch_steps(Dev d, BatchDev b, int chunk) {
    batch_queue<MIXED, STAGE, T, false>(d, b, chunk);
}

// The compensated form keeps few values live across its FP32 phases: capped at 64 registers
// (1024 resident threads per SM) it hides more memory latency than with the compiler's choice.
template <bool STAGE, int T>
__global__ void __launch_bounds__(T, 1024 / T) k_batch_steps_comp(Dev d, BatchDev b, int chunk) {
    batch_queue<true, STAGE, T, true>(d, b, chunk);
}

}  // namespace nf
