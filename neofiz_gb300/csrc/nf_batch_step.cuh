// nf_batch_step.cuh -- one step of one batched instance by a whole block, shared by the
// batched kernel (k_batch.cu) and the adjoint kernels (k_adjoint.cu).
#pragma once

#include "nf_bodies.cuh"

namespace nf {

__device__ __forceinline__ unsigned long long bbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bdouble(unsigned long long u) {
    return __longlong_as_double((long long)u);
}

// Exact block minimum of the per-thread shortest squared edges, returned to every thread. The
// warps combine with jmin and the warps' results by the integer order of their bits, as the
// single-scene kernels do with shuffles and atomicMin.
template <int T>
__device__ double block_min_edge(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v = jmin(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = bbits(sh[0]);
        for (int w = 1; w < T / 32; w++) m = min(m, bbits(sh[w]));
        sh[T / 32] = bdouble(m);
    }
    __syncthreads();
    return sh[T / 32];
}

template <int T>
__device__ double block_min_edge_f(float v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    return block_min_edge<T>((double)v, sh);
}

// Fixed-tree block sum; valid in thread 0.
template <int T>
__device__ double block_total(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < T / 32; w++) t += sh[w];
    __syncthreads();
    return t;
}

// The coming step's size and nodal coefficients (:947-956, :985-990), computed once per block
// by thread 0 and read by every thread: the same formulas as each thread would evaluate, so
// the same bits, without every thread spending FP64 divisions and a square root on them.
struct BlockStep {
    double dt, decay, gain, dtAvg;
    float fdt, fdecay, fgain, fdtAvg;               // the same in FP32 (the FP32 forms)
    float plane, friction, gravR, gravZ, hourglass; // the instance's constants in FP32
};

__device__ __forceinline__ void block_step_coef(BlockStep &bs, const BatchInst &in, double dt,
                                                double dtPrev) {
    const double dtAvg = 0.5 * (dtPrev + dt);
    const double half = 0.5 * in.damping * dtAvg;
    bs.dt = dt;
    bs.decay = (1.0 - half) / (1.0 + half);
    bs.gain = dtAvg / (1.0 + half);
    bs.dtAvg = dtAvg;
    bs.fdt = (float)bs.dt;
    bs.fdecay = (float)bs.decay;
    bs.fgain = (float)bs.gain;
    bs.fdtAvg = (float)bs.dtAvg;
}

// At the start of a chunk (thread 0): the coefficients and the FP32 constants.
__device__ __forceinline__ void block_step_init(BlockStep &bs, const Dev &d, const BatchInst &in,
                                                double dt, double dtPrev) {
    block_step_coef(bs, in, dt, dtPrev);
    bs.plane = (float)in.wallPlane;
    bs.friction = (float)in.wallFriction;
    bs.gravR = (float)d.gravR;
    bs.gravZ = (float)d.gravZ;
    bs.hourglass = (float)in.hourglass;
}

// Thread 0's part of a step's end: the block minimum of the warps' minima (exact, by the order
// of the bits), the CFL step (:985-990) and the next step's coefficients. Out of line: one
// thread runs it once a step, and its FP64 division and square root stay out of the
// registers of the element and node loops.
static __device__ __noinline__ void block_step_advance(double *sh, int warps, BlockStep *bs,
                                                const BatchInst &in, double dt, double dtPrev,
                                                int finite) {
    unsigned long long m = bbits(sh[0]);
    for (int w = 1; w < warps; w++) m = min(m, bbits(sh[w]));
    const double me = bdouble(m);
    sh[warps] = me;
    if (finite) block_step_coef(*bs, in, in.cfl * sqrt(me * in.massScale) / in.wave, dt);
    else block_step_coef(*bs, in, dt, dtPrev);
}

// The common end of block_min_edge_next(_f): each warp's minimum is in sh[warp].
template <int T>
__device__ __forceinline__ double block_min_tail(double *sh, BlockStep *bs, const BatchInst &in,
                                                 double dt, double dtPrev, int finite) {
    __syncthreads();
    if (threadIdx.x == 0) block_step_advance(sh, T / 32, bs, in, dt, dtPrev, finite);
    __syncthreads();
    return sh[T / 32];
}

// block_min_edge, with thread 0 also preparing the next step in bs between the barriers.
template <int T>
__device__ double block_min_edge_next(double v, double *sh, BlockStep *bs, const BatchInst &in,
                                      double dt, double dtPrev, int finite) {
    for (int o = 16; o > 0; o >>= 1) v = jmin(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    return block_min_tail<T>(sh, bs, in, dt, dtPrev, finite);
}

// The same for FP32 edges: the warps reduce in FP32 (exact), lane 0 widens its minimum.
template <int T>
__device__ double block_min_edge_next_f(float v, double *sh, BlockStep *bs, const BatchInst &in,
                                        double dt, double dtPrev, int finite) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)v;
    return block_min_tail<T>(sh, bs, in, dt, dtPrev, finite);
}

// One step of instance `in` by the whole block, ExplicitSolver.step :940-991: the nodal update
// (with the mixed form's float geometry when geo.pMid is set), the assembly with the block's
// exact shortest squared edge, the per-node gather, the next CFL step. dt, dtPrev, time and
// steps advance in place; returns the shortest squared edge. COMP (with MIXED): the
// compensated form's FP32 nodal update and gather (nf_bodies.cuh). With bs (a block-shared
// BlockStep prepared for this step), the step's coefficients and the next step size come from
// thread 0 through it; without, every thread evaluates them.
template <bool MIXED, int T, bool COMP = false>
__device__ __forceinline__ double batch_step(const Dev &d, const BatchInst &in, double &dt,
                                             double &dtPrev, double &time, long long &steps,
                                             const MixedGeo &geo, const float4 *pMid,
                                             const float2 *vdt, int base, uint32_t *status,
                                             int *wallContact, int *wallStuck, double &impulse,
                                             double &loss, double &fric, double *shMin,
                                             BlockStep *bs = nullptr) {
    static_assert(!COMP || MIXED, "the compensated form assembles in FP32");
    NodalCoef co;
    if (bs) {
        co = NodalCoef{bs->decay, bs->gain, bs->dtAvg, dt};
    } else {
        const double dtAvg = 0.5 * (dtPrev + dt);                   // :947-956
        const double half = 0.5 * in.damping * dtAvg;
        co = NodalCoef{(1.0 - half) / (1.0 + half), dtAvg / (1.0 + half), dtAvg, dt};
    }
    const WallRef w{in.hasWall, in.wallPlane, in.wallFriction, wallContact, wallStuck};
    if (COMP) {                                                  // requires bs
        for (int i = in.n0 + threadIdx.x; i < in.n1; i += T)
            nodal_node_comp(d, i, bs->fdecay, bs->fgain, bs->fdtAvg, bs->fdt, bs->plane,
                            bs->friction, w, geo, status, impulse, loss, fric);
    } else {
        for (int i = in.n0 + threadIdx.x; i < in.n1; i += T)
            nodal_node(d, i, co, w, geo, status, impulse, loss, fric);
    }
    __syncthreads();
    time += dt;                                                       // :973-974
    steps += 1;
    double me;
    if (MIXED) {
        float m = 3.4028235e38f;
        const float sdt = bs ? bs->fdt : (float)dt, qhg = bs ? bs->hourglass : (float)in.hourglass;
        for (int e = in.e0 + threadIdx.x; e < in.e1; e += T)
            element_reduced_f32(d, e, sdt, qhg, pMid, vdt, base, m);
        for (int k = in.k0 + threadIdx.x; k < in.k1; k += T) {   // applyPressure, :1203-1207
            if (COMP) pressure_edge_comp(d, k, time, in.pressure, in.ramp);
            else pressure_edge_f32(d, k, time, in.pressure, in.ramp);
        }
        if (bs) {
            me = block_min_edge_next_f<T>(m, shMin, bs, in, dt, dtPrev, d.finite);
        } else {
            me = block_min_edge_f<T>(m, shMin);
        }
    } else {
        double m = DMAX;
        for (int e = in.e0 + threadIdx.x; e < in.e1; e += T) element_reduced(d, e, dt, in.hourglass, m);
        for (int k = in.k0 + threadIdx.x; k < in.k1; k += T)
            pressure_edge(d, k, time, in.pressure, in.ramp);
        me = bs ? block_min_edge_next<T>(m, shMin, bs, in, dt, dtPrev, d.finite)
                : block_min_edge<T>(m, shMin);
    }
    // the gather keeps the nodal loop's node-to-thread map, so the next nodal update reads
    // only forces its own thread wrote
    for (int i = in.n0 + threadIdx.x; i < in.n1; i += T) {
        if (COMP) d.fC[i] = gather_node_comp(d, i, bs->gravR, bs->gravZ);
        else d.F[i] = MIXED ? gather_node_f32(d, i) : gather_node(d, i);
    }
    if (d.finite) {                                                   // :985-990
        dtPrev = dt;
        dt = bs ? bs->dt : in.cfl * sqrt(me * in.massScale) / in.wave;
    }
    return me;
}

}  // namespace nf
