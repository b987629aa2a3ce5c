// k_scan.cu -- exclusive prefix sum over int32 on the device, used to compact the free
// surface, the surface nodes, the contact grid buckets and the contact incidence lists.
// Three passes: per-tile scan (1024 items per 256-thread block), scan of the tile totals
// (recursively), add-back. Integer addition is exact, so the order of the tree is immaterial.
#include "nf_internal.h"

namespace nf {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    return (int)(g < 1 ? 1 : g);
}

__global__ void k_scan_tiles(const int32_t *in, int32_t *out, int nMax, int32_t *tileSums,
                             const int *pred, const int *nDev) {
    if (pred && !*pred) return;
    const int n = nDev ? min(*nDev, nMax) : nMax;
    if (blockIdx.x * SCAN_TILE >= n) {          // a tile past the live length contributes 0
        if (threadIdx.x == 0) tileSums[blockIdx.x] = 0;
        return;
    }
    __shared__ int32_t warpSums[SCAN_BLOCK / 32];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS];
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = base + k;
        v[k] = i < n ? in[i] : 0;
        local += v[k];
    }
    // inclusive scan of thread totals within the warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t inc = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < SCAN_BLOCK / 32 ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < SCAN_BLOCK / 32) warpSums[lane] = w;
    }
    __syncthreads();
    int32_t run = inc - local + (warp > 0 ? warpSums[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_BLOCK - 1) tileSums[blockIdx.x] = run;
}

__global__ void k_scan_add(int32_t *out, int nMax, const int32_t *tileOffsets, const int *pred,
                           const int *nDev) {
    if (pred && !*pred) return;
    const int n = nDev ? min(*nDev, nMax) : nMax;
    const int tile = blockIdx.x;
    const int32_t add = tileOffsets[tile];
    const int base = tile * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x) {
        const int i = base + k;
        if (i < n) out[i] += add;
    }
}

__global__ void k_scan_copy_total(const int32_t *src, int32_t *dst, const int *pred) {
    if (pred && !*pred) return;
    *dst = *src;
}

__global__ void k_scan_zero_total(int32_t *dst, const int *pred) {
    if (pred && !*pred) return;
    *dst = 0;
}

size_t scan_tmp_ints(int n) {
    size_t total = 0;
    long long m = n;
    while (m > 1) {
        m = (m + SCAN_TILE - 1) / SCAN_TILE;
        total += 2 * (size_t)m + 2;
    }
    return total + 4;
}

// tmp must hold scan_tmp_ints(n) ints. totalOut (device) receives the sum when non-null.
// in and out may alias.
// When pred is non-null every kernel of the scan does nothing unless *pred is non-zero, so
// the scan can sit in a fixed launch sequence and only run on the steps that need it.
// nDev, when given, is a device-side live length (at most n): only that prefix is scanned.
int scan_exclusive(const int32_t *in, int32_t *out, int n, int32_t *totalOut, int32_t *tmp,
                   cudaStream_t stream, const int *pred, const int *nDev) {
    if (n <= 0) {
        if (totalOut) {
            k_scan_zero_total<<<1, 1, 0, stream>>>(totalOut, pred);
            return 1;
        }
        return 0;
    }
    const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    int32_t *tileSums = tmp;
    int32_t *tileOffsets = tmp + tiles + 1;
    int launched = 1;
    k_scan_tiles<<<tiles, SCAN_BLOCK, 0, stream>>>(in, out, n, tileSums, pred, nDev);
    if (tiles > 1) {
        launched += scan_exclusive(tileSums, tileOffsets, tiles, totalOut, tmp + 2 * tiles + 2,
                                   stream, pred, nullptr);
        k_scan_add<<<tiles, SCAN_BLOCK, 0, stream>>>(out, n, tileOffsets, pred, nDev);
        launched++;
    } else if (totalOut) {
        k_scan_copy_total<<<1, 1, 0, stream>>>(tileSums, totalOut, pred);
        launched++;
    }
    return launched;
}

}  // namespace nf
