// nf_batch_kernels.cuh -- the persistent batched kernel (k_batch.cu), as templates: the FP64
// and mixed forms are instantiated in k_batch.cu, the compensated form in k_batch_comp.cu,
// which is compiled with float contraction and fast float division and square root.
#pragma once

#include "nf_batch_step.cuh"

namespace nf {

// Up to `chunk` steps of instance k by the whole block: ExplicitSolver.step, :940-991, with the
// loop condition of TaylorImpactCase.java:250-253 (step while time < t_end).
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
    int taken = 0;
    for (; taken < chunk; taken++) {
        if (!(time < in.tEnd) || steps >= limit) break;
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
        if (!(time < in.tEnd) || steps >= limit) {
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
