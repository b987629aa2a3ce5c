// k_contact.cu -- penalty node-to-segment contact with a Coulomb cone
// (src/main/java/org/neofiz/solver/Contact.java), and the free-surface rebuild it needs after
// erosion (mesh/QuadMesh.java:188-226 via Contact.adopt, Contact.java:290-322).
//
// The reference's result depends on three orders, and each is reproduced exactly:
//   * the surface is listed in element order and its nodes ascending (a stream compaction
//     of per-edge and per-node flags, i.e. an ordered scan);
//   * the search visits the nine cells in (dj, di) order and, within a cell, the segments in
//     the order the counting sort filed them -- ascending segment, first endpoint before the
//     second (Contact.java:530-545, :578-603). Buckets are filled with atomics and then
//     sorted by (cell, 2 s + endpoint), which restores exactly that order;
//   * every node's force receives its contact terms in slave order, normal before tangent
//     (Contact.java:446-462, :717-754). Each pair's twelve terms are computed in parallel,
//     each node then sorts its incident pairs and adds them in that order.
// The running totals (spring energy, dissipation) are audits; they are reduced in a fixed
// order per block, so they are deterministic but not summed in the reference's serial order.
#include "nf_internal.h"

namespace nf {

constexpr int CB = 128;
constexpr int STEP_GRID = 256;       // blocks of the per-step kernels (grid-stride over counts)
constexpr int REBUILD_GRID = 1024;   // blocks of the surface-rebuild kernels
constexpr int SEARCH_GRID = 512;     // blocks of 4 warps, one warp per slave at a time
constexpr int RESOLVE_BLOCKS = 256;  // fixed, so the partial sums have a fixed order
constexpr double MAX_DEPTH = 0.5;
constexpr double STICK_RELAXATION = 0.5;
constexpr double FACING = 0.25;

__device__ __forceinline__ unsigned long long okey(double v) {     // order-preserving image
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double unokey(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    return __longlong_as_double((long long)b);
}

__device__ double block_sum_c(double v, double *sh) {
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
    return t;
}

// ---------------------------------------------------------------------------- begin

#define GRID_STRIDE(i, count) \
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (count); i += gridDim.x * blockDim.x)

// Contact.begin, Contact.java:424-436: per-step totals, and whether the surface is stale.
__global__ void k_contact_begin(Dev d) {
    DevScalars *s = d.s;
    s->rebuild = s->active && s->stale;
    if (!s->active) return;
    s->pairs = 0;
    s->maxPenBits = 0ULL;
    s->bbox[0] = ~0ULL;   // min r
    s->bbox[1] = ~0ULL;   // min z
    s->bbox[2] = 0ULL;    // max r
    s->bbox[3] = 0ULL;    // max z
    s->longestBits = 0ULL;
}

// ---------------------------------------------------------------------------- surface rebuild

__global__ void k_surf_flags(Dev d) {
    if (!d.s->rebuild) return;
    GRID_STRIDE(q, 4 * d.E) {
        const int e = q >> 2;
        int flag = 0;
        if (!d.dead[e]) {
            const int g = d.edgeGroup[q];
            int live = 0;
            for (int m = d.groupStart[g]; m < d.groupStart[g + 1]; m++)
                if (!d.dead[d.groupMember[m] >> 2]) live++;
            flag = live == 1;
        }
        d.surfFlag[q] = flag;
    }
}

// a[0 .. n) = 0, with n = min(*nDev, nMax) when nDev is given
__global__ void k_zero_int(int32_t *a, int nMax, const int *pred, const int *nDev) {
    if (pred && !*pred) return;
    const int n = nDev ? min(*nDev, nMax) : nMax;
    GRID_STRIDE(i, n) a[i] = 0;
}

__global__ void k_copy_int(const int32_t *src, int32_t *dst, int nMax, const int *pred,
                           const int *nDev) {
    if (pred && !*pred) return;
    const int n = nDev ? min(*nDev, nMax) : nMax;
    GRID_STRIDE(i, n) dst[i] = src[i];
}

__global__ void k_surf_emit(Dev d) {
    if (!d.s->rebuild) return;
    GRID_STRIDE(q, 4 * d.E) {
        if (!d.surfFlag[q]) continue;
        const int e = q >> 2, k = q & 3;
        const int4 c = d.conn[e];
        const int nn[4] = {c.x, c.y, c.z, c.w};
        const int a = nn[k], b = nn[(k + 1) & 3];
        const int p = d.surfPos[q];
        d.segA[p] = a;
        d.segB[p] = b;
        d.segOwner[p] = e;
        d.nodeFlag[a] = 1;
        d.nodeFlag[b] = 1;
    }
}

__global__ void k_surf_nodes(Dev d) {
    if (!d.s->rebuild) return;
    GRID_STRIDE(n, d.N) {
        if (d.nodeFlag[n]) {
            const int slot = d.nodePos[n];
            d.surfNodes[slot] = n;
            d.slotOf[n] = slot;
            d.lastMaster[slot] = -1;         // Contact.adopt, :319-321
            d.master[slot] = -1;
            d.dropped[slot] = 0;
            d.segCount[slot] = 0;
        } else {
            d.slotOf[n] = -1;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d.s->slotScanN = 0;   // set by k_seg_scan_n
}

__global__ void k_seg_scan_n(Dev d) {
    if (!d.s->rebuild) return;
    d.s->slotScanN = d.s->surfNodes + 1;
    d.segCount[d.s->surfNodes] = 0;
}

__global__ void k_seg_count(Dev d) {
    if (!d.s->rebuild) return;
    GRID_STRIDE(s, d.s->surfEdges) {
        atomicAdd(&d.segCount[d.slotOf[d.segA[s]]], 1);
        atomicAdd(&d.segCount[d.slotOf[d.segB[s]]], 1);
    }
}

__global__ void k_seg_fill(Dev d) {
    if (!d.s->rebuild) return;
    GRID_STRIDE(s, d.s->surfEdges) {
        d.segOf[atomicAdd(&d.segCursor[d.slotOf[d.segA[s]]], 1)] = s;
        d.segOf[atomicAdd(&d.segCursor[d.slotOf[d.segB[s]]], 1)] = s;
    }
}

// Restores ascending segment order in each node's list (Contact.java:306-313), then retires
// the rebuild.
__global__ void k_seg_sort(Dev d) {
    if (!d.s->rebuild) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) d.s->stale = 0;
    GRID_STRIDE(i, d.s->surfNodes) {
        const int lo = d.segStart[i], hi = d.segStart[i + 1];
        for (int k = lo + 1; k < hi; k++) {
            const int v = d.segOf[k];
            int j = k - 1;
            while (j >= lo && d.segOf[j] > v) {
                d.segOf[j + 1] = d.segOf[j];
                j--;
            }
            d.segOf[j + 1] = v;
        }
    }
}

// ---------------------------------------------------------------------------- geometry

// Contact.geometry, Contact.java:467-500 (coordinates and the bounding box of the grid)
__global__ void k_contact_nodes(Dev d) {
    if (!d.s->active) return;
    unsigned long long kr0 = ~0ULL, kz0 = ~0ULL, kr1 = 0ULL, kz1 = 0ULL;
    GRID_STRIDE(i, d.s->surfNodes) {
        const int n = d.surfNodes[i];
        const double2 x = d.X0[n], u = d.U[n];
        const double cr = x.x + u.x, cz = x.y + u.y;
        d.cr[n] = cr;
        d.cz[n] = cz;
        d.incCount[i] = 0;
        d.pairNodes[i] = make_int4(-1, -1, -1, 0);
        const unsigned long long kr = okey(cr), kz = okey(cz);
        kr0 = min(kr0, kr); kr1 = max(kr1, kr);
        kz0 = min(kz0, kz); kz1 = max(kz1, kz);
    }
    // extrema are exact in any order: reduce in the warp, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        kr0 = min(kr0, __shfl_down_sync(0xffffffffu, kr0, o));
        kz0 = min(kz0, __shfl_down_sync(0xffffffffu, kz0, o));
        kr1 = max(kr1, __shfl_down_sync(0xffffffffu, kr1, o));
        kz1 = max(kz1, __shfl_down_sync(0xffffffffu, kz1, o));
    }
    if ((threadIdx.x & 31) == 0 && kr1 != 0ULL) {
        atomicMin(&d.s->bbox[0], kr0);
        atomicMin(&d.s->bbox[1], kz0);
        atomicMax(&d.s->bbox[2], kr1);
        atomicMax(&d.s->bbox[3], kz1);
    }
}

__global__ void k_contact_segs(Dev d) {
    if (!d.s->active) return;
    unsigned long long lb = 0ULL;
    GRID_STRIDE(s, d.s->surfEdges) {
        const int a = d.segA[s], b = d.segB[s];
        const double dr = d.cr[b] - d.cr[a], dz = d.cz[b] - d.cz[a];
        const double len = sqrt(dr * dr + dz * dz);
        d.slen[s] = len;
        if (len > 0.0) {
            d.snr[s] = dz / len;
            d.snz[s] = -dr / len;
        } else {
            d.snr[s] = 0.0;
            d.snz[s] = 0.0;
        }
        lb = max(lb, (unsigned long long)__double_as_longlong(len));
    }
    for (int o = 16; o > 0; o >>= 1) lb = max(lb, __shfl_down_sync(0xffffffffu, lb, o));
    if ((threadIdx.x & 31) == 0 && lb != 0ULL) atomicMax(&d.s->longestBits, lb);
}

__global__ void k_contact_pnorm(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(i, d.s->surfNodes) {
        double sr = 0.0, sz = 0.0;
        for (int k = d.segStart[i]; k < d.segStart[i + 1]; k++) {
            sr += d.snr[d.segOf[k]];
            sz += d.snz[d.segOf[k]];
        }
        const double len = sqrt(sr * sr + sz * sz);
        d.pnr[i] = len > 0.0 ? sr / len : 0.0;
        d.pnz[i] = len > 0.0 ? sz / len : 0.0;
    }
}

// Contact.grid, Contact.java:515-545 (the grid's extent and cell size)
__global__ void k_grid_setup(Dev d) {
    DevScalars *s = d.s;
    if (!s->active) return;
    s->slotScanN = s->surfNodes + 1;
    d.incCount[s->surfNodes] = 0;
    if (s->surfNodes == 0) {
        s->cols = s->rows = 1;
        s->cells = 1;
        s->hashed = 0;
        s->bucketScanN = 2;
        return;
    }
    const double rlo = unokey(s->bbox[0]), zlo = unokey(s->bbox[1]);
    const double rhi = unokey(s->bbox[2]), zhi = unokey(s->bbox[3]);
    const double longest = __longlong_as_double((long long)s->longestBits);
    const double cellSize = longest > 0.0 ? 1.5 * longest : 1.0;
    s->cellSize = cellSize;
    s->gridR0 = rlo;
    s->gridZ0 = zlo;
    const int a = jd2i((rhi - rlo) / cellSize) + 1;
    const int b = jd2i((zhi - zlo) / cellSize) + 1;
    s->cols = a > 1 ? a : 1;
    s->rows = b > 1 ? b : 1;
    s->cells = (long long)s->cols * (long long)s->rows;
    s->hashed = s->cells > d.bucketCap;
    s->bucketScanN = (int)((s->hashed ? (long long)d.bucketCap : s->cells) + 1);
    if (s->hashed) atomicOr(&s->status, STATUS_GRID_HASHED);
}

__device__ __forceinline__ int iclamp(int v, int n) { return v < 0 ? 0 : v >= n ? n - 1 : v; }

__device__ __forceinline__ long long cell_of(const DevScalars *s, double r, double z) {
    const int i = iclamp(jd2i((r - s->gridR0) / s->cellSize), s->cols);
    const int j = iclamp(jd2i((z - s->gridZ0) / s->cellSize), s->rows);
    return (long long)j * s->cols + i;
}

__device__ __forceinline__ int bucket_of(const Dev &d, long long cell) {
    return d.s->hashed ? (int)(cell % d.bucketCap) : (int)cell;
}

__global__ void k_bucket_count(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(q, 2 * d.s->surfEdges) {
        const int s = q >> 1;
        const int node = (q & 1) ? d.segB[s] : d.segA[s];
        const long long cell = cell_of(d.s, d.cr[node], d.cz[node]);
        d.entryCell[q] = cell;
        atomicAdd(&d.bucketCount[bucket_of(d, cell)], 1);
    }
}

__global__ void k_bucket_fill(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(q, 2 * d.s->surfEdges) {
        const long long cell = d.entryCell[q];
        const int pos = atomicAdd(&d.bucketCursor[bucket_of(d, cell)], 1);
        d.bucketEntry[pos] = q;
        d.bucketCell[pos] = cell;
    }
}

// Sorts each bucket by (cell, entry): the counting sort's filing order.
__global__ void k_bucket_sort(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(b, d.s->bucketScanN - 1) {
        const int lo = d.bucketStart[b], hi = d.bucketStart[b + 1];
        for (int k = lo + 1; k < hi; k++) {
            const int v = d.bucketEntry[k];
            const long long c = d.bucketCell[k];
            int j = k - 1;
            while (j >= lo && (d.bucketCell[j] > c || (d.bucketCell[j] == c && d.bucketEntry[j] > v))) {
                d.bucketEntry[j + 1] = d.bucketEntry[j];
                d.bucketCell[j + 1] = d.bucketCell[j];
                j--;
            }
            d.bucketEntry[j + 1] = v;
            d.bucketCell[j + 1] = c;
        }
    }
}

// ---------------------------------------------------------------------------- search

// Contact.excluded, Contact.java:620-639
__device__ __forceinline__ bool excluded(const Dev &d, int i, int n, int s) {
    const int a = d.segA[s], b = d.segB[s];
    if (d.pnr[i] * d.snr[s] + d.pnz[i] * d.snz[s] > -FACING) return true;
    if (a == n || b == n) return true;
    for (int k = d.segStart[i]; k < d.segStart[i + 1]; k++) {
        const int own = d.segOf[k];
        const int p = d.segA[own], q = d.segB[own];
        if (p == a || p == b || q == a || q == b) return true;
    }
    return false;
}

// Contact.depth, Contact.java:642-652
__device__ __forceinline__ double depth_of(const Dev &d, int n, int s) {
    const int a = d.segA[s], b = d.segB[s];
    const double len = d.slen[s];
    if (len <= 0.0) return 0.0;
    const double tr = (d.cr[b] - d.cr[a]) / len, tz = (d.cz[b] - d.cz[a]) / len;
    const double dr = d.cr[n] - d.cr[a], dz = d.cz[n] - d.cz[a];
    const double along = dr * tr + dz * tz;
    if (along < 0.0 || along > len) return 0.0;
    const double gap = dr * d.snr[s] + dz * d.snz[s];
    return gap < 0.0 ? -gap : 0.0;
}

// Contact.nearestPenetrated, Contact.java:570-606, one warp per slave. The reference visits
// the nine cells in (dj, di) order and each cell's bucket in order, keeping the first
// candidate of greatest depth. Here the nine bucket ranges are concatenated in that order,
// the lanes take the candidates round-robin, each lane keeps its first deepest (strictly
// greater replaces), and the warp reduction takes the greatest depth with the smallest
// position in the visit sequence: the same segment the serial loop keeps.
__global__ void __launch_bounds__(CB) k_contact_search(Dev d) {
    const DevScalars *s = d.s;
    if (!s->active) return;
    const int lane = threadIdx.x & 31;
    const int warpsTotal = gridDim.x * (blockDim.x >> 5);
    const int count = s->surfNodes;
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < count; i += warpsTotal) {
        const int n = d.surfNodes[i];
        const double crn = d.cr[n], czn = d.cz[n];
        const int ci = iclamp(jd2i((crn - s->gridR0) / s->cellSize), s->cols);
        const int cj = iclamp(jd2i((czn - s->gridZ0) / s->cellSize), s->rows);
        const int last = d.lastMaster[i];
        // lanes 0..8 describe the nine cells in visit order
        int lo = 0, len = 0;
        long long myCell = -1;
        if (lane < 9) {
            const int j = cj + lane / 3 - 1, ii = ci + lane % 3 - 1;
            if (j >= 0 && j < s->rows && ii >= 0 && ii < s->cols) {
                myCell = (long long)j * s->cols + ii;
                const int bkt = bucket_of(d, myCell);
                lo = d.bucketStart[bkt];
                len = d.bucketStart[bkt + 1] - lo;
            }
        }
        int off = len;                                   // inclusive scan over the nine
        for (int o = 1; o < 16; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += t;
        }
        const int total = __shfl_sync(0xffffffffu, off, 8);
        off -= len;                                      // exclusive
        double best = 0.0;
        int bestPos = 0x7fffffff, bestSeg = -1;
        bool fell = false;
        for (int base = 0; base < total; base += 32) {
            const int t = base + lane;
            // which of the nine ranges holds position t
            int c = 0;
#pragma unroll
            for (int q = 1; q < 9; q++) {
                const int oq = __shfl_sync(0xffffffffu, off, q);
                if (t >= oq) c = q;
            }
            const int oc = __shfl_sync(0xffffffffu, off, c);
            const int lc = __shfl_sync(0xffffffffu, lo, c);
            const long long cc = __shfl_sync(0xffffffffu, myCell, c);
            if (t >= total) continue;
            const int k = lc + (t - oc);
            if (d.bucketCell[k] != cc) continue;
            const int sg = d.bucketEntry[k] >> 1;
            if (excluded(d, i, n, sg)) continue;
            const double depth = depth_of(d, n, sg);
            if (depth <= 0.0) continue;
            if (depth > MAX_DEPTH * d.slen[sg]) {
                if (sg == last) fell = true;
                continue;
            }
            if (depth > best) {
                best = depth;
                bestPos = t;
                bestSeg = sg;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_down_sync(0xffffffffu, best, o);
            const int op = __shfl_down_sync(0xffffffffu, bestPos, o);
            const int os = __shfl_down_sync(0xffffffffu, bestSeg, o);
            if (ob > best || (ob == best && op < bestPos)) {
                best = ob;
                bestPos = op;
                bestSeg = os;
            }
        }
        const bool anyFell = __any_sync(0xffffffffu, fell);
        if (lane == 0) {
            d.dropped[i] = anyFell ? 1 : 0;
            d.master[i] = best > 0.0 ? bestSeg : -1;
        }
    }
}

// ---------------------------------------------------------------------------- resolve

// Contact.accumulate + resolve, Contact.java:446-462, :663-762: each slave's pair, computed
// independently (resolve reads velocities and masses only). Writes the twelve force terms of
// the pair as values to ADD (x - y is computed as x + (-y), which is the same IEEE result).
__global__ void __launch_bounds__(CB) k_contact_resolve(Dev d) {
    __shared__ double sh[CB / 32];
    const DevScalars *sc = d.s;
    if (!sc->active) return;
    double energy = 0.0, diss = 0.0;
    GRID_STRIDE(i, sc->surfNodes) {
        const int n = d.surfNodes[i];
        const int best = d.master[i];
        if (best < 0) {
            if (d.lastMaster[i] >= 0 && d.dropped[i]) atomicAdd(&d.s->escaped, 1);
            d.lastMaster[i] = -1;
            continue;
        }
        d.lastMaster[i] = best;
        const int s = best;
        const double dt = sc->dt;
        const double reference = d.dt0;
        const int a = d.segA[s], b = d.segB[s];
        const double depth = depth_of(d, n, s);
        const double len = d.slen[s];
        const double tr = (d.cr[b] - d.cr[a]) / len;            // parameter, :655-661
        const double tz = (d.cz[b] - d.cz[a]) / len;
        const double t = ((d.cr[n] - d.cr[a]) * tr + (d.cz[n] - d.cz[a]) * tz) / len;
        const double wa = 1.0 - t, wb = t;
        const double ma = d.mass[a], mb = d.mass[b];
        const double invMaster = 0.25 / ma + 0.25 / mb;
        if (!(invMaster > 0.0)) continue;
        const double mMaster = 1.0 / invMaster;
        const double mSlave = d.mass[n];
        const double mStar = mSlave * mMaster / (mSlave + mMaster);
        const double k = d.cScale * mStar / (reference * reference);
        const double nR = d.snr[s], nZ = d.snz[s];
        const double mTrue = 1.0 / (wa * wa / ma + wb * wb / mb);
        const double mTangent = mSlave * mTrue / (mSlave + mTrue);
        const double2 vn = d.V[n], va = d.V[a], vb = d.V[b];
        const double closing = (vn.x - wa * va.x - wb * vb.x) * nR
                               + (vn.y - wa * va.y - wb * vb.y) * nZ;
        const double damper = 2.0 * d.cDamping * mStar * sqrt(d.cScale) / reference;
        const double normal = jmax(0.0, k * depth - damper * closing);
        double *pv = d.pairVal + 12 * (size_t)i;
        pv[0] = normal * nR;
        pv[1] = normal * nZ;
        pv[4] = -(wa * normal * nR);
        pv[5] = -(wa * normal * nZ);
        pv[8] = -(wb * normal * nR);
        pv[9] = -(wb * normal * nZ);
        atomicAdd(&d.s->pairs, 1);
        energy += 0.5 * k * depth * depth;
        atomicMax(&d.s->maxPenBits, (unsigned long long)__double_as_longlong(depth));
        double dthis = 0.0;
        const double damperForce = normal - k * depth;
        if (damperForce != 0.0) {
            const double closingAfter = closing + damperForce * dt / mTangent;
            dthis -= damperForce * 0.5 * (closing + closingAfter) * dt;
        }
        uint8_t state = NF_CONTACT_PAIR;
        if (d.cFriction > 0.0) {
            const double tR = -nZ, tZ = nR;
            const double slide = (vn.x - wa * va.x - wb * vb.x) * tR
                                 + (vn.y - wa * va.y - wb * vb.y) * tZ;
            double tangent = -STICK_RELAXATION * mTangent * slide / dt;
            const double cone = d.cFriction * normal;
            bool slipped = false;
            if (tangent > cone) { tangent = cone; slipped = true; }
            else if (tangent < -cone) { tangent = -cone; slipped = true; }
            pv[2] = tangent * tR;
            pv[3] = tangent * tZ;
            pv[6] = -(wa * tangent * tR);
            pv[7] = -(wa * tangent * tZ);
            pv[10] = -(wb * tangent * tR);
            pv[11] = -(wb * tangent * tZ);
            const double after = slide + tangent * dt / mTangent;
            dthis += -tangent * 0.5 * (slide + after) * dt;
            state |= slipped ? NF_CONTACT_SLIP : NF_CONTACT_STICK;
        }
        diss += dthis;
        d.contactState[n] = state;
        d.pairNodes[i] = make_int4(n, a, b, 1);
    }
    const double e1 = block_sum_c(energy, sh);
    const double e2 = block_sum_c(diss, sh);
    if (threadIdx.x == 0) {
        d.partials[(PARTIAL_CONTACT + 0) * d.maxBlocks + blockIdx.x] = e1;
        d.partials[(PARTIAL_CONTACT + 1) * d.maxBlocks + blockIdx.x] = e2;
    }
}

__global__ void k_inc_count(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(i, d.s->surfNodes) {
        const int4 p = d.pairNodes[i];
        if (!p.w) continue;
        atomicAdd(&d.incCount[d.slotOf[p.x]], 1);
        atomicAdd(&d.incCount[d.slotOf[p.y]], 1);
        atomicAdd(&d.incCount[d.slotOf[p.z]], 1);
    }
}

__global__ void k_inc_fill(Dev d) {
    if (!d.s->active) return;
    GRID_STRIDE(i, d.s->surfNodes) {
        const int4 p = d.pairNodes[i];
        if (!p.w) continue;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.x]], 1)] = (i << 2) | 0;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.y]], 1)] = (i << 2) | 1;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.z]], 1)] = (i << 2) | 2;
    }
}

// Adds each node's contact terms in slave order, normal then tangent (Contact.java:717-754).
__global__ void k_inc_apply(Dev d) {
    if (!d.s->active) return;
    const bool friction = d.cFriction > 0.0;
    GRID_STRIDE(j, d.s->surfNodes) {
        const int lo = d.incStart[j], hi = d.incStart[j + 1];
        if (lo == hi) continue;
        for (int k = lo + 1; k < hi; k++) {
            const int v = d.incEntry[k];
            int q = k - 1;
            while (q >= lo && d.incEntry[q] > v) {
                d.incEntry[q + 1] = d.incEntry[q];
                q--;
            }
            d.incEntry[q + 1] = v;
        }
        const int node = d.surfNodes[j];
        double2 f = d.F[node];
        for (int k = lo; k < hi; k++) {
            const int ent = d.incEntry[k];
            const double *pv = d.pairVal + 12 * (size_t)(ent >> 2) + 4 * (ent & 3);
            f.x += pv[0];
            f.y += pv[1];
            if (friction) {
                f.x += pv[2];
                f.y += pv[3];
            }
        }
        d.F[node] = f;
    }
}

// ---------------------------------------------------------------------------- launch

int contact_partial_blocks() { return RESOLVE_BLOCKS; }

int launch_contact(Solver &S, bool) {
    Dev &d = S.d;
    const cudaStream_t st = S.stream;
    const int *rebuild = &d.s->rebuild;
    const int *active = &d.s->active;
    const int *slotN = &d.s->slotScanN;
    const int *bucketN = &d.s->bucketScanN;
    const int rg = REBUILD_GRID, sg = STEP_GRID;
    int n = 0;
#define L(kernel, grid, ...) do { kernel<<<(grid), CB, 0, st>>>(__VA_ARGS__); n++; } while (0)
    L(k_contact_begin, 1, d);
    // free surface, only on the steps after an erosion (or the first)
    L(k_surf_flags, rg, d);
    n += scan_exclusive(d.surfFlag, d.surfPos, 4 * d.E, &d.s->surfEdges, d.scanTmp, st, rebuild,
                        nullptr);
    L(k_zero_int, rg, d.nodeFlag, d.N, rebuild, nullptr);
    L(k_surf_emit, rg, d);
    n += scan_exclusive(d.nodeFlag, d.nodePos, d.N, &d.s->surfNodes, d.scanTmp, st, rebuild,
                        nullptr);
    L(k_surf_nodes, rg, d);
    L(k_seg_scan_n, 1, d);
    L(k_seg_count, rg, d);
    n += scan_exclusive(d.segCount, d.segStart, d.N + 1, nullptr, d.scanTmp, st, rebuild, slotN);
    L(k_copy_int, rg, d.segStart, d.segCursor, d.N + 1, rebuild, slotN);
    L(k_seg_fill, rg, d);
    L(k_seg_sort, rg, d);
    // geometry and grid
    L(k_contact_nodes, sg, d);
    L(k_contact_segs, sg, d);
    L(k_contact_pnorm, sg, d);
    L(k_grid_setup, 1, d);
    L(k_zero_int, sg, d.bucketCount, d.bucketCap + 1, active, bucketN);
    L(k_bucket_count, sg, d);
    n += scan_exclusive(d.bucketCount, d.bucketStart, d.bucketCap + 1, nullptr, d.scanTmp, st,
                        active, bucketN);
    L(k_copy_int, sg, d.bucketStart, d.bucketCursor, d.bucketCap + 1, active, bucketN);
    L(k_bucket_fill, sg, d);
    L(k_bucket_sort, sg, d);
    // search, resolve, ordered accumulation
    L(k_contact_search, SEARCH_GRID, d);
    L(k_contact_resolve, RESOLVE_BLOCKS, d);
    L(k_inc_count, sg, d);
    n += scan_exclusive(d.incCount, d.incStart, d.N + 1, nullptr, d.scanTmp, st, active, slotN);
    L(k_copy_int, sg, d.incStart, d.incCursor, d.N + 1, active, slotN);
    L(k_inc_fill, sg, d);
    L(k_inc_apply, sg, d);
#undef L
    return n;
}

}  // namespace nf
