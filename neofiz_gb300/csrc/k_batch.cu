// k_batch.cu -- many independent scenes (a parameter sweep: the reference runs one solver per
// thread through Sweep.over, src/main/java/org/neofiz/app/Sweep.java:82-105) stepped by one
// persistent kernel.
//
// One block owns one instance at a time and runs its whole step with block barriers between
// the phases: nodal update, element assembly with the block's exact minimum edge, the
// per-node gather, the next CFL step. Blocks take instances from a queue (most expensive
// first), each for a chunk of steps, so uneven meshes and uneven step counts balance. Every
// phase calls the same per-node and per-element bodies as the single-scene kernels
// (nf_bodies.cuh), in the same order per node and per element, so an instance's trajectory is
// bit-identical to the same scene run alone in the same precision. The audit totals (wall
// impulse, energy loss, friction work) are summed per block in a fixed order: deterministic
// for a given launch shape, but not in the single-scene kernels' association.
//
// Launch shape: block size (128, 256), whether the mixed form stages each instance's float
// node geometry in shared memory, blocks per SM and the chunk length are chosen by the
// autotuner (api_batch.cu); none of them changes the trajectory.
#include "nf_batch_kernels.cuh"

namespace nf {

constexpr int MEASURE_BLOCK = 256;

// The first assembly of every instance (zero strain increment), in the batch's precision, as
// the single-scene path runs it before its first step; records the shortest edge.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_batch_initial(Dev d, BatchDev b) {
    __shared__ double shMin[256 / 32 + 1];
    const BatchInst in = b.inst[blockIdx.x];
    double me;
    if (MIXED) {
        for (int i = in.n0 + threadIdx.x; i < in.n1; i += 256)
            prepare_node(d, i, 0.0, MixedGeo{d.pMid, nullptr, d.vdt, 0});
        __syncthreads();
        float m = 3.4028235e38f;
        for (int e = in.e0 + threadIdx.x; e < in.e1; e += 256)
            element_reduced_f32(d, e, 0.0f, (float)in.hourglass, d.pMid, d.vdt, 0, m);
        me = block_min_edge_f<256>(m, shMin);
    } else {
        double m = DMAX;
        for (int e = in.e0 + threadIdx.x; e < in.e1; e += 256)
            element_reduced(d, e, 0.0, in.hourglass, m);
        me = block_min_edge<256>(m, shMin);
    }
    const double t0 = b.sc[blockIdx.x].time;
    for (int k = in.k0 + threadIdx.x; k < in.k1; k += 256) {
        if (MIXED) pressure_edge_f32(d, k, t0, in.pressure, in.ramp);
        else pressure_edge(d, k, t0, in.pressure, in.ramp);
    }
    __syncthreads();
    for (int i = in.n0 + threadIdx.x; i < in.n1; i += 256)
        d.F[i] = MIXED ? gather_node_f32(d, i) : gather_node(d, i);
    if (threadIdx.x == 0) b.sc[blockIdx.x].minEdgeSquared = me;
}

// Arms a run: every instance may take maxSteps more steps; counts the instances left to run.
__global__ void k_batch_arm(BatchDev b, long long maxSteps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) *b.queue = 0;
    if (k >= b.count) return;
    BatchScalars &s = b.sc[k];
    s.stepLimit = s.steps + maxSteps;
    const int every = b.burst.every;
    const bool ended = every > 0 ? (s.steps % every == 0 && !(s.time < b.inst[k].tEnd)) ||
                                       b.burst.state[k].traversed
                                 : !(s.time < b.inst[k].tEnd);
    const bool done = ended || maxSteps <= 0;
    s.done = done ? 1 : 0;
    if (!done) atomicAdd(b.remaining, 1);
}

// TaylorImpactCase.java:272-288 per instance: max z, min z, max r of the current
// configuration, as order-preserving integer images (exact in any order).
__device__ __forceinline__ unsigned long long okey_b(double v) {
    const unsigned long long u = bbits(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

__global__ void __launch_bounds__(MEASURE_BLOCK) k_batch_measure(Dev d, BatchDev b) {
    __shared__ unsigned long long sh[3][MEASURE_BLOCK / 32];
    const BatchInst in = b.inst[blockIdx.x];
    unsigned long long zmax = 0ULL, zmin = ~0ULL, rmax = 0ULL;
    for (int i = in.n0 + threadIdx.x; i < in.n1; i += MEASURE_BLOCK) {
        const double2 x = d.X0[i], u = d.U[i];
        const unsigned long long kz = okey_b(x.y + u.y), kr = okey_b(x.x + u.x);
        zmax = max(zmax, kz);
        zmin = min(zmin, kz);
        rmax = max(rmax, kr);
    }
    for (int o = 16; o > 0; o >>= 1) {
        zmax = max(zmax, __shfl_down_sync(0xffffffffu, zmax, o));
        zmin = min(zmin, __shfl_down_sync(0xffffffffu, zmin, o));
        rmax = max(rmax, __shfl_down_sync(0xffffffffu, rmax, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][warp] = zmax;
        sh[1][warp] = zmin;
        sh[2][warp] = rmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < MEASURE_BLOCK / 32; w++) {
            zmax = max(zmax, sh[0][w]);
            zmin = min(zmin, sh[1][w]);
            rmax = max(rmax, sh[2][w]);
        }
        b.measure[3 * blockIdx.x + 0] = zmax;
        b.measure[3 * blockIdx.x + 1] = zmin;
        b.measure[3 * blockIdx.x + 2] = rmax;
    }
}

// ------------------------------------------------------------------------------------ launch

template <bool MIXED, bool STAGE, int T, bool COMP>
static const void *steps_kernel() {
    return (const void *)k_batch_steps<MIXED, STAGE, T>;
}

template <bool MIXED, bool STAGE, bool COMP>
static const void *by_threads(int threads) {
    if (threads == 32) return steps_kernel<MIXED, STAGE, 32, COMP>();
    return threads == 128 ? steps_kernel<MIXED, STAGE, 128, COMP>()
                          : steps_kernel<MIXED, STAGE, 256, COMP>();
}

template <bool MIXED, bool COMP>
static const void *by_shape(const BatchShape &s) {
    if (MIXED && s.stage) return by_threads<MIXED, true, COMP>(s.threads);
    return by_threads<MIXED, false, COMP>(s.threads);
}

static const void *select_kernel(int mode, const BatchShape &s) {
    if (mode == NF_PRECISION_COMPENSATED) return comp_steps_kernel(s);
    if (mode == NF_PRECISION_MIXED) return by_shape<true, false>(s);
    return by_shape<false, false>(s);
}

size_t batch_shared_bytes(int mode, const BatchShape &s, int maxNodes) {
    return mode != NF_PRECISION_FP64 && s.stage ? (sizeof(float4) + sizeof(float2)) * (size_t)maxNodes
                                                : 0;
}

// Resident blocks per SM of a shape (0 when it cannot launch, e.g. too much shared memory).
int batch_max_blocks_per_sm(int mode, const BatchShape &s, int maxNodes) {
    const void *k = select_kernel(mode, s);
    const size_t smem = batch_shared_bytes(mode, s, maxNodes);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, s.threads, smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t launch_batch_steps(const Dev &d, const BatchDev &b, int mode, const BatchShape &s,
                               int sms, cudaStream_t st) {
    const void *k = select_kernel(mode, s);
    const size_t smem = batch_shared_bytes(mode, s, b.maxNodes);
    int blocks = sms * s.blocksPerSm;
    if (blocks > b.count) blocks = b.count;
    if (blocks < 1) blocks = 1;
    Dev dd = d;
    BatchDev bb = b;
    int chunk = s.chunk;
    void *args[] = {&dd, &bb, &chunk};
    return cudaLaunchKernel(k, dim3(blocks), dim3(s.threads), args, smem, st);
}

void launch_batch_initial(const Dev &d, const BatchDev &b, bool mixed, cudaStream_t st) {
    if (b.count <= 0) return;
    if (mixed) k_batch_initial<true><<<b.count, 256, 0, st>>>(d, b);
    else k_batch_initial<false><<<b.count, 256, 0, st>>>(d, b);
}

void launch_batch_arm(const BatchDev &b, long long maxSteps, cudaStream_t st) {
    cudaMemsetAsync(b.remaining, 0, sizeof(int32_t), st);
    k_batch_arm<<<grid_for(b.count > 0 ? b.count : 1, 256), 256, 0, st>>>(b, maxSteps);
}

void launch_batch_measure(const Dev &d, const BatchDev &b, cudaStream_t st) {
    if (b.count > 0) k_batch_measure<<<b.count, MEASURE_BLOCK, 0, st>>>(d, b);
}

}  // namespace nf
