// k_contact.cu -- penalty node-to-segment contact with a Coulomb cone
// (src/main/java/org/neofiz/solver/Contact.java), and the free-surface rebuild it needs after
// erosion (mesh/QuadMesh.java:188-226 via Contact.adopt, Contact.java:290-322).
//
// One cooperative, persistent kernel per step runs the whole contact pass as phases separated
// by grid-wide barriers: the surface rebuild (only on steps after an erosion), geometry, the
// counting-sort grid, the search, the pair forces and their ordered accumulation. It replaces
// some thirty launches of small kernels, whose launch gaps dominated the pass.
//
// The surface rebuild after erosion is incremental: only the edge groups of the elements
// eroded since the last rebuild can change, so their members are re-flagged, the edges that
// became free or stopped being free are ordered, and the segment and node lists are merged
// (each kept entry moves by the changes before it) instead of recompacting all 4 E element
// edges and all N nodes. The lists are the ones a full rebuild gives, entry for entry; the full
// rebuild runs at set-up and when an unusually large number of elements erodes at once.
//
// The reference's result depends on three orders, and each is reproduced exactly:
//   * the surface is listed in element order and its nodes ascending (ordered compactions,
//     i.e. exclusive scans of per-edge and per-node flags);
//   * the search visits the nine cells in (dj, di) order and, within a cell, the segments in
//     the order the counting sort filed them -- ascending segment, first endpoint before the
//     second (Contact.java:530-545, :578-603). Buckets are filled with atomics in any order;
//     each candidate carries its visit key (cell in the nine, 2 s + endpoint) instead, and
//     ties in depth go to the smallest key, the candidate the serial loop keeps;
//   * every node's force receives its contact terms in slave order, normal before tangent
//     (Contact.java:446-462, :717-754). Each pair's twelve terms are computed in parallel and
//     filed in fixed per-node lists; each node then sorts its list and adds in that order.
// The running totals (spring energy, dissipation) are audits; they are reduced in a fixed
// order per block over a fixed grid, so they are deterministic but not summed in the
// reference's serial order.
//
// The grid barrier is a counter and a generation word in device memory. The launch is
// cooperative, so every block is resident and the barrier cannot deadlock; its wait is bounded
// all the same: a block that waits longer than a second sets STATUS_TIMEOUT and an abort word
// that releases the others, and the kernel returns.
#include "nf_internal.h"

namespace nf {

constexpr int CB = 256;                  // threads per block
constexpr int CB_WARPS = CB / 32;
constexpr int MAX_COOP_BLOCKS_PER_SM = 4;
constexpr double MAX_DEPTH = 0.5;
constexpr double STICK_RELAXATION = 0.5;
constexpr double FACING = 0.25;
constexpr int INC_CAP = NF_INC_CAP;      // incident terms a surface node's fixed list holds
constexpr int SCAN_ITEMS = 8;            // values a thread scans in registers per tile
constexpr unsigned long long WAIT_LIMIT_NS = 1000000000ULL;   // one second
constexpr long long WAIT_LIMIT_SPINS = 1LL << 27;             // a bound independent of the timer

__device__ __forceinline__ unsigned long long okey(double v) {     // order-preserving image
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double unokey(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <typename T>
__device__ __forceinline__ T vload(const T *p) { return *(const volatile T *)p; }

// ---------------------------------------------------------------------------- block helpers

// Fixed-order block sum; the result is valid in thread 0. Leaves sh free for reuse.
__device__ double block_sum_c(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < CB_WARPS; w++) t += sh[w];
    __syncthreads();
    return t;
}

// Inclusive scan of one int per thread over the block; *total (in every thread) gets the sum.
__device__ int block_scan_incl(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    __syncthreads();
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < CB_WARPS ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < CB_WARPS) sh[lane] = w;
    }
    __syncthreads();
    const int r = x + (warp > 0 ? sh[warp - 1] : 0);
    *total = sh[CB_WARPS - 1];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------- grid barrier

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int *p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_relaxed(unsigned int *p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Sense-reversal barrier over all blocks of the cooperative grid. After the block's own
// barrier, thread 0 arrives on the counter with an acquire-release add (publishing what the
// block wrote, which the block barrier ordered before it) and waits with acquire loads for the
// generation to move; the last arriver resets the counter and moves the generation with a
// release store. Returns false when the wait ran out or another block gave up; the caller then
// leaves the kernel. The wait polls at most d.waitSpins times and for at most d.waitNs
// nanoseconds (defaults when zero).
__device__ bool grid_sync(const Dev &d) {
    __shared__ int ok;
    DevScalars *s = d.s;
    const long long spinLimit = d.waitSpins > 0 ? d.waitSpins : WAIT_LIMIT_SPINS;
    const unsigned long long nsLimit =
        d.waitNs > 0 ? (unsigned long long)d.waitNs : WAIT_LIMIT_NS;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int g = ld_relaxed(&s->barGen);
        const unsigned int arrived = atom_add_acq_rel(&s->barCount, 1u);
        int good = 1;
        if (arrived == gridDim.x - 1) {
            st_relaxed(&s->barCount, 0u);
            st_release(&s->barGen, g + 1u);
        } else {
            const unsigned long long t0 = global_ns();
            long long spins = 0;
            while (ld_acquire(&s->barGen) == g) {
                if (ld_relaxed(&s->barAbort)) {
                    good = 0;
                    break;
                }
                if (++spins > spinLimit || global_ns() - t0 > nsLimit) {
                    atomicOr(&s->status, STATUS_TIMEOUT);
                    atomicExch(&s->barAbort, 1u);
                    good = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Exclusive scan of in[0, n) into out (and into out2 when given: the cursor copy the atomic
// fills advance); zeroes in[] behind it when zeroIn; *total gets the sum when given. The
// block sums go through d.coopSums. Ends with a barrier; returns false when one ran out.
__device__ bool grid_scan(const Dev &d, int32_t *in, int32_t *out, int32_t *out2, int n,
                          int32_t *total, bool zeroIn) {
    __shared__ int sh[CB_WARPS];
    const int G = gridDim.x;
    const int chunk = (n + G - 1) / G;
    const int lo = min(n, (int)blockIdx.x * chunk), hi = min(n, lo + chunk);
    int local = 0;
    for (int i = lo + threadIdx.x; i < hi; i += CB) local += in[i];
    int bsum;
    block_scan_incl(local, sh, &bsum);
    if (threadIdx.x == 0) d.coopSums[blockIdx.x] = bsum;
    if (!grid_sync(d)) return false;
    // this block's offset: the sum over the earlier blocks' chunks
    int pre = 0;
    for (int j = threadIdx.x; j < (int)blockIdx.x; j += CB) pre += vload(&d.coopSums[j]);
    int carry;
    block_scan_incl(pre, sh, &carry);
    if (total && threadIdx.x == 0 && (int)blockIdx.x == G - 1) *total = carry + bsum;
    // tiles of CB x SCAN_ITEMS: each thread scans a run of SCAN_ITEMS in registers, so one
    // block scan serves SCAN_ITEMS values per thread
    for (int base = lo; base < hi; base += CB * SCAN_ITEMS) {
        const int first = base + threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int run = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            v[k] = first + k < hi ? in[first + k] : 0;
            run += v[k];
        }
        int tileTotal;
        const int incl = block_scan_incl(run, sh, &tileTotal);
        int at = carry + incl - run;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            const int i = first + k;
            if (i < hi) {
                out[i] = at;
                if (out2) out2[i] = at;
                if (zeroIn) in[i] = 0;
            }
            at += v[k];
        }
        carry += tileTotal;
    }
    return grid_sync(d);
}

// ---------------------------------------------------------------------------- contact geometry

// The search grid of one step (Contact.grid, Contact.java:515-545), derived from the bounding
// box by every block for itself, so no pass over the grid waits on a single thread.
struct Grid {
    double cellSize, r0, z0;
    int cols, rows, hashed, bucketN;
    long long cells;
};

__device__ void grid_from_box(const Dev &d, int nodes, Grid &g) {
    DevScalars *s = d.s;
    if (nodes == 0) {
        g.cellSize = 1.0;
        g.r0 = g.z0 = 0.0;
        g.cols = g.rows = 1;
        g.cells = 1;
        g.hashed = 0;
        g.bucketN = 2;
        return;
    }
    const double rlo = unokey(vload(&s->bbox[0])), zlo = unokey(vload(&s->bbox[1]));
    const double rhi = unokey(vload(&s->bbox[2])), zhi = unokey(vload(&s->bbox[3]));
    const double longest = __longlong_as_double((long long)vload(&s->longestBits));
    const double cellSize = longest > 0.0 ? 1.5 * longest : 1.0;
    g.cellSize = cellSize;
    g.r0 = rlo;
    g.z0 = zlo;
    const int a = jd2i((rhi - rlo) / cellSize) + 1;
    const int b = jd2i((zhi - zlo) / cellSize) + 1;
    g.cols = a > 1 ? a : 1;
    g.rows = b > 1 ? b : 1;
    g.cells = (long long)g.cols * (long long)g.rows;
    g.hashed = g.cells > d.bucketCap;
    g.bucketN = (int)((g.hashed ? (long long)d.bucketCap : g.cells) + 1);
}

__device__ __forceinline__ int iclamp(int v, int n) { return v < 0 ? 0 : v >= n ? n - 1 : v; }

__device__ __forceinline__ long long cell_of(const Grid &g, double r, double z) {
    const int i = iclamp(jd2i((r - g.r0) / g.cellSize), g.cols);
    const int j = iclamp(jd2i((z - g.z0) / g.cellSize), g.rows);
    return (long long)j * g.cols + i;
}

__device__ __forceinline__ int bucket_of(const Dev &d, const Grid &g, long long cell) {
    return g.hashed ? (int)(cell % d.bucketCap) : (int)cell;
}

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
// The segment's unit tangent (cr[b] - cr[a]) / len, (cz[b] - cz[a]) / len is (-snz, snr) bit
// for bit: the geometry phase formed snr = dz / len and snz = -dr / len from the same sums
// (cr = x0 + u), and (-dr) / len is -(dr / len) exactly. Reading it saves two divisions.
__device__ __forceinline__ double depth_of(const Dev &d, int n, int s) {
    const int a = d.segA[s];
    const double len = d.slen[s];
    if (len <= 0.0) return 0.0;
    const double tr = -d.snz[s], tz = d.snr[s];
    const double dr = d.cr[n] - d.cr[a], dz = d.cz[n] - d.cz[a];
    const double along = dr * tr + dz * tz;
    if (along < 0.0 || along > len) return 0.0;
    const double gap = dr * d.snr[s] + dz * d.snz[s];
    return gap < 0.0 ? -gap : 0.0;
}

// Files one incident term (pair i, role r as i << 2 | r) in node slot j's fixed list; a list
// that overflows switches the step to the general path (a scan over the counts).
__device__ __forceinline__ void inc_push(const Dev &d, int j, int entry) {
    const int pos = atomicAdd(&d.incCount[j], 1);
    if (pos < INC_CAP) d.incSlots[(size_t)j * INC_CAP + pos] = entry;
    else d.s->incOverflow = 1;
}

// Contact.accumulate + resolve, Contact.java:446-462, :663-762, for slave i (node n) and its
// master segment s: writes the pair's twelve force terms as values to ADD (x - y is computed
// as x + (-y), the same IEEE result) and files them at the pair's three nodes. Adds the
// pair's spring energy and dissipation.
__device__ void resolve_pair(const Dev &d, int i, int n, int s, double &energy, double &diss) {
    const double dt = d.s->dt;
    const double reference = d.dt0;
    const int a = d.segA[s], b = d.segB[s];
    const double depth = depth_of(d, n, s);
    const double len = d.slen[s];
    const double tr = -d.snz[s];                            // parameter, :655-661 (the
    const double tz = d.snr[s];                             // tangent as in depth_of)
    const double t = ((d.cr[n] - d.cr[a]) * tr + (d.cz[n] - d.cz[a]) * tz) / len;
    const double wa = 1.0 - t, wb = t;
    const double ma = d.mass[a], mb = d.mass[b];
    const double invMaster = 0.25 / ma + 0.25 / mb;
    if (!(invMaster > 0.0)) return;
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
    inc_push(d, i, (i << 2) | 0);              // the slave's slot is i
    inc_push(d, d.slotOf[a], (i << 2) | 1);
    inc_push(d, d.slotOf[b], (i << 2) | 2);
}

// Contact.nearestPenetrated, Contact.java:570-606, then the pair, for slave i, by one whole
// warp. The reference visits the nine cells in (dj, di) order and each cell's entries in the
// order its counting sort filed them, ascending entry (2 s + endpoint), and keeps the first
// candidate of greatest depth. Here the nine bucket ranges are concatenated, the lanes take
// the candidates round-robin, and each candidate carries its visit key (cell in the nine,
// entry): the warp keeps the greatest depth with the smallest key, which is the candidate the
// serial loop keeps, so the buckets need no order. A candidate's depth is zero unless its gap
// is negative; that test is exact and reads only what the fill staged beside the entry, so it
// runs first, before the exclusions and the divisions.
// Contact.nearestPenetrated (Contact.java:570-606) for four surface slots per warp, eight lanes
// (a group) each: the deepest admissible segment and whether the last step's master was seen
// too deep. Every candidate carries its visit key (cell in the nine, then the bucket entry),
// and ties in depth go to the smallest key, the candidate the serial loop keeps. All 32 lanes
// run every shuffle; a lane's group answer is valid when slot < nodes.
constexpr int SG = 8;                          // lanes per slave
__device__ void search_group(const Dev &d, const Grid &g, int slot, int nodes, double &bestOut,
                             int &segOut, bool &fellOut) {
    const int lane = threadIdx.x & 31, gl = lane & (SG - 1);
    const bool live = slot < nodes;
    double2 xn = make_double2(0.0, 0.0);
    int n = -1, last = -1, ci = 0, cj = 0;
    if (live) {
        xn = d.slaveXY[slot];
        n = d.surfNodes[slot];
        last = d.lastMaster[slot];
        ci = iclamp(jd2i((xn.x - g.r0) / g.cellSize), g.cols);
        cj = iclamp(jd2i((xn.y - g.z0) / g.cellSize), g.rows);
    }
    // the nine cells in visit order: lane gl takes cell gl, lane 0 also cell 8
    int lo = 0, len = 0, lo8 = 0, len8 = 0;
    long long myCell = -1, cell8 = -1;
    if (live) {
        {
            const int j = cj + gl / 3 - 1, ii = ci + gl % 3 - 1;
            if (j >= 0 && j < g.rows && ii >= 0 && ii < g.cols) {
                myCell = (long long)j * g.cols + ii;
                const int bkt = bucket_of(d, g, myCell);
                lo = d.bucketStart[bkt];
                len = d.bucketStart[bkt + 1] - lo;
            }
        }
        if (gl == 0) {
            const int j = cj + 1, ii = ci + 1;
            if (j < g.rows && ii < g.cols) {
                cell8 = (long long)j * g.cols + ii;
                const int bkt = bucket_of(d, g, cell8);
                lo8 = d.bucketStart[bkt];
                len8 = d.bucketStart[bkt + 1] - lo8;
            }
        }
    }
    int off = len;                              // inclusive scan over cells 0..7
    for (int o = 1; o < SG; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, off, o, SG);
        if (gl >= o) off += t;
    }
    const int off8 = __shfl_sync(0xffffffffu, off, SG - 1, SG);
    off -= len;                                 // exclusive
    lo8 = __shfl_sync(0xffffffffu, lo8, 0, SG);
    len8 = __shfl_sync(0xffffffffu, len8, 0, SG);
    cell8 = __shfl_sync(0xffffffffu, cell8, 0, SG);
    const int total = off8 + len8;
    int rounds = total;                         // the longest group's candidates, warp-wide
    for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
    double best = 0.0;
    unsigned long long bestKey = ~0ULL;
    int bestSeg = -1;
    bool fell = false;
    for (int base = 0; base < rounds; base += SG) {
        const int t = base + gl;
        int c = 0;                              // which of the nine ranges holds position t
#pragma unroll
        for (int q = 1; q < SG; q++) {
            const int oq = __shfl_sync(0xffffffffu, off, q, SG);
            if (t >= oq) c = q;
        }
        if (t >= off8) c = 8;
        const int src = c < SG ? c : 0;
        const int oc0 = __shfl_sync(0xffffffffu, off, src, SG);
        const int lc0 = __shfl_sync(0xffffffffu, lo, src, SG);
        const long long cc0 = __shfl_sync(0xffffffffu, myCell, src, SG);
        if (t >= total) continue;
        const int oc = c < SG ? oc0 : off8, lc = c < SG ? lc0 : lo8;
        const long long cc = c < SG ? cc0 : cell8;
        const int k = lc + (t - oc);
        const long long kc = d.bucketCell[k];
        const int entry = d.bucketEntry[k];
        const double2 pa = d.bucketA[k], nrm = d.bucketN[k];
        const double len = d.bucketL[k];
        if (kc != cc) continue;
        // depth_of from what the filing staged beside the entry (the segment's first node,
        // normal and length: the same values, the same expressions): zero unless the slave is
        // behind the segment and projects onto it
        const double dr = xn.x - pa.x, dz = xn.y - pa.y;
        const double gap = dr * nrm.x + dz * nrm.y;
        if (!(gap < 0.0)) continue;
        if (len <= 0.0) continue;
        const double along = dr * -nrm.y + dz * nrm.x;
        if (along < 0.0 || along > len) continue;
        const double depth = -gap;
        // the exclusions read the slave's own rings (dependent loads); a candidate that fails
        // them is skipped whatever its depth, so testing them after the depth changes nothing
        const int sg = entry >> 1;
        if (excluded(d, slot, n, sg)) continue;
        if (depth > MAX_DEPTH * len) {
            if (sg == last) fell = true;
            continue;
        }
        const unsigned long long key = ((unsigned long long)c << 32) | (unsigned int)entry;
        if (depth > best || (depth == best && key < bestKey)) {
            best = depth;
            bestKey = key;
            bestSeg = sg;
        }
    }
    for (int o = SG / 2; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o, SG);
        const unsigned long long ok = __shfl_down_sync(0xffffffffu, bestKey, o, SG);
        const int os = __shfl_down_sync(0xffffffffu, bestSeg, o, SG);
        if (ob > best || (ob == best && ok < bestKey)) {
            best = ob;
            bestKey = ok;
            bestSeg = os;
        }
    }
    const unsigned fellBits = __ballot_sync(0xffffffffu, fell);
    fellOut = ((fellBits >> (lane & ~(SG - 1))) & ((1u << SG) - 1u)) != 0u;
    bestOut = __shfl_sync(0xffffffffu, best, 0, SG);
    segOut = __shfl_sync(0xffffffffu, bestSeg, 0, SG);
}

// The pair of surface slot i from its search (Contact.java:446-462): master, last master,
// the escape count and the pair forces; one lane.
__device__ void finish_slave(const Dev &d, int i, double best, int bestSeg, bool anyFell,
                             double &energy, double &diss) {
    const int last = d.lastMaster[i];
    d.master[i] = best > 0.0 ? bestSeg : -1;
    if (!(best > 0.0)) {                      // no pair: Contact.java:446-452
        if (last >= 0 && anyFell) atomicAdd(&d.s->escaped, 1);
        d.lastMaster[i] = -1;
        return;
    }
    d.lastMaster[i] = bestSeg;
    resolve_pair(d, i, d.surfNodes[i], bestSeg, energy, diss);
}

// ---------------------------------------------------------------------------- the pass

// More erosions than this since the last rebuild take the full rebuild (the change lists are
// ordered by counting, quadratic in their length).
constexpr int INC_MAX_DEAD = 512;

// Position of v in the ascending a[0, n): the number of entries below it.
__device__ __forceinline__ int lower_bound_i(const int32_t *a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Rank of v among the distinct a[0, n): the number of entries below it.
__device__ __forceinline__ int rank_in(const int32_t *a, int n, int v) {
    int r = 0;
    for (int j = 0; j < n; j++) r += a[j] < v;
    return r;
}

// Items are dealt to warps across the blocks first (warp w of block b takes the 32 items from
// (w G + b) 32 on), so that a short list still spreads over every SM.
#define FOR_GRID(i, count)                                                                    \
    for (int i = ((threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);     \
         i < (count); i += gridDim.x * CB)
#define SYNC() do { if (!grid_sync(d)) return; } while (0)

// The per-step totals this pass accumulates into (Contact.begin, Contact.java:424-436) are
// reset by the step's first kernel (contact_step_reset), so the pass needs no opening barrier.
__global__ void __launch_bounds__(CB, 2) k_contact_pass(Dev d) {
    __shared__ double shd[CB_WARPS];
    __shared__ Grid grid;
    DevScalars *s = d.s;
    if (!vload(&s->active)) return;
    const int gt = blockIdx.x * CB + threadIdx.x;

    if (vload(&s->stale)) {
        // Contact.adopt, Contact.java:290-322: the free surface (QuadMesh.surface over the live
        // elements, QuadMesh.java:188-226), edges in element order, nodes ascending
        const int oldEdges = vload(&s->surfEdges), oldNodes = vload(&s->surfNodes);
        const int nDead = vload(&s->newDeadCount);
        const int epoch = vload(&s->rebuildEpoch) + 1;
        if (vload(&s->fullRebuild) || nDead > INC_MAX_DEAD) {
            // every element edge: free when it is the only live member of its group
            FOR_GRID(q, 4 * d.E) {
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
            FOR_GRID(n, d.N) {
                d.nodeFlag[n] = 0;
                d.nodeFree[n] = 0;
            }
            SYNC();
            if (!grid_scan(d, d.surfFlag, d.surfPos, nullptr, 4 * d.E, &s->surfEdges, false))
                return;
            FOR_GRID(q, 4 * d.E) {
                if (!d.surfFlag[q]) continue;
                const int e = q >> 2, k = q & 3;
                const int4 c = d.conn[e];
                const int nn[4] = {c.x, c.y, c.z, c.w};
                const int a = nn[k], b = nn[(k + 1) & 3];
                const int p = d.surfPos[q];
                d.segA[p] = a;
                d.segB[p] = b;
                d.segQ[p] = q;
                d.nodeFlag[a] = 1;
                d.nodeFlag[b] = 1;
                atomicAdd(&d.nodeFree[a], 1);
                atomicAdd(&d.nodeFree[b], 1);
            }
            SYNC();
            if (!grid_scan(d, d.nodeFlag, d.nodePos, nullptr, d.N, &s->surfNodes, false)) return;
            FOR_GRID(n, d.N) {
                if (d.nodeFlag[n]) {
                    const int slot = d.nodePos[n];
                    d.surfNodes[slot] = n;
                    d.slotOf[n] = slot;
                    d.lastMaster[slot] = -1;             // :319-321
                    d.master[slot] = -1;
                    d.dropped[slot] = 0;
                    d.segCount[slot] = d.nodeFree[n];    // its incident free edges
                } else {
                    d.slotOf[n] = -1;
                }
            }
            if (gt == 0) d.segCount[vload(&s->surfNodes)] = 0;
            SYNC();
        } else {
            // only the edge groups of the elements eroded since the last rebuild can change:
            // re-flag their members (each once: the epoch stamp), list the edges that became
            // free or stopped being free, keep each node's count of incident free edges, and
            // note the nodes whose count changed
            FOR_GRID(t, 4 * nDead) {
                const int g = d.edgeGroup[4 * d.newDead[t >> 2] + (t & 3)];
                const int g0 = d.groupStart[g], g1 = d.groupStart[g + 1];
                int live = 0;
                for (int m = g0; m < g1; m++)
                    if (!d.dead[d.groupMember[m] >> 2]) live++;
                for (int m = g0; m < g1; m++) {
                    const int q = d.groupMember[m];
                    if (atomicExch(&d.edgeStamp[q], epoch) == epoch) continue;
                    const int now = !d.dead[q >> 2] && live == 1;
                    if (now == d.surfFlag[q]) continue;
                    d.surfFlag[q] = now;
                    if (now) d.addE[atomicAdd(&s->nAddE, 1)] = q;
                    else d.remE[atomicAdd(&s->nRemE, 1)] = q;
                    const int4 c = d.conn[q >> 2];
                    const int nn[4] = {c.x, c.y, c.z, c.w};
                    const int ends[2] = {nn[q & 3], nn[(q + 1) & 3]};
                    for (int k = 0; k < 2; k++) {
                        atomicAdd(&d.nodeFree[ends[k]], now ? 1 : -1);
                        if (atomicExch(&d.nodeStamp[ends[k]], epoch) != epoch)
                            d.touched[atomicAdd(&s->nTouched, 1)] = ends[k];
                    }
                }
            }
            SYNC();
            const int nAddE = vload(&s->nAddE), nRemE = vload(&s->nRemE);
            const int nTouched = vload(&s->nTouched);
            // the changed edges in ascending order; the nodes that joined or left the surface
            FOR_GRID(i, nAddE) {
                const int q = d.addE[i];
                d.addES[rank_in(d.addE, nAddE, q)] = q;
            }
            FOR_GRID(i, nRemE) {
                const int q = d.remE[i];
                d.remES[rank_in(d.remE, nRemE, q)] = q;
            }
            FOR_GRID(i, nTouched) {
                const int n = d.touched[i];
                const bool was = d.slotOf[n] >= 0, is = d.nodeFree[n] > 0;
                if (is && !was) d.addN[atomicAdd(&s->nAddN, 1)] = n;
                else if (was && !is) d.remN[atomicAdd(&s->nRemN, 1)] = n;
            }
            SYNC();
            const int nAddN = vload(&s->nAddN), nRemN = vload(&s->nRemN);
            FOR_GRID(i, nAddN) {
                const int n = d.addN[i];
                d.addNS[rank_in(d.addN, nAddN, n)] = n;
            }
            FOR_GRID(i, nRemN) {
                const int n = d.remN[i];
                d.remNS[rank_in(d.remN, nRemN, n)] = n;
            }
            // the merged edge list: a kept edge moves back by the removed edges before it and
            // on by the added ones; an added edge lands after the kept edges before it
            FOR_GRID(p, oldEdges) {
                const int q = d.segQ[p];
                if (!d.surfFlag[q]) continue;
                const int np = p - lower_bound_i(d.remES, nRemE, q) + lower_bound_i(d.addES, nAddE, q);
                d.tmpA[np] = d.segA[p];
                d.tmpB[np] = d.segB[p];
                d.tmpQ[np] = q;
            }
            FOR_GRID(r, nAddE) {
                const int q = d.addES[r];
                const int np = lower_bound_i(d.segQ, oldEdges, q) - lower_bound_i(d.remES, nRemE, q) + r;
                const int4 c = d.conn[q >> 2];
                const int nn[4] = {c.x, c.y, c.z, c.w};
                d.tmpA[np] = nn[q & 3];
                d.tmpB[np] = nn[(q + 1) & 3];
                d.tmpQ[np] = q;
            }
            SYNC();
            const int newEdges = oldEdges - nRemE + nAddE, newNodes = oldNodes - nRemN + nAddN;
            FOR_GRID(p, newEdges) {
                d.segA[p] = d.tmpA[p];
                d.segB[p] = d.tmpB[p];
                d.segQ[p] = d.tmpQ[p];
            }
            // the merged node list, the same way
            FOR_GRID(i, oldNodes) {
                const int n = d.surfNodes[i];
                if (d.nodeFree[n] == 0) continue;
                d.tmpNodes[i - lower_bound_i(d.remNS, nRemN, n) + lower_bound_i(d.addNS, nAddN, n)] = n;
            }
            FOR_GRID(r, nAddN) {
                const int n = d.addNS[r];
                d.tmpNodes[lower_bound_i(d.surfNodes, oldNodes, n) - lower_bound_i(d.remNS, nRemN, n) + r] = n;
            }
            FOR_GRID(r, nRemN) d.slotOf[d.remNS[r]] = -1;
            if (gt == 0) {
                s->surfEdges = newEdges;
                s->surfNodes = newNodes;
            }
            SYNC();
            FOR_GRID(i, newNodes) {
                const int n = d.tmpNodes[i];
                d.surfNodes[i] = n;
                d.slotOf[n] = i;
                d.lastMaster[i] = -1;                    // :319-321
                d.master[i] = -1;
                d.dropped[i] = 0;
                d.segCount[i] = d.nodeFree[n];
            }
            if (gt == 0) d.segCount[newNodes] = 0;
            SYNC();
        }
        // each surface node's segments, ascending (:298-313)
        const int edges = vload(&s->surfEdges), nodes = vload(&s->surfNodes);
        if (!grid_scan(d, d.segCount, d.segStart, d.segCursor, nodes + 1, nullptr, false)) return;
        FOR_GRID(e, edges) {
            d.segOf[atomicAdd(&d.segCursor[d.slotOf[d.segA[e]]], 1)] = e;
            d.segOf[atomicAdd(&d.segCursor[d.slotOf[d.segB[e]]], 1)] = e;
        }
        SYNC();
        FOR_GRID(i, nodes) {
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
        if (gt == 0) {
            s->stale = 0;
            s->fullRebuild = 0;
            s->newDeadCount = 0;
            s->rebuildEpoch = epoch;
            s->nAddE = s->nRemE = s->nTouched = s->nAddN = s->nRemN = 0;
        }
        SYNC();
    }
    const int nodes = vload(&s->surfNodes), edges = vload(&s->surfEdges);

    // Contact.geometry, Contact.java:467-500: current coordinates, the bounding box, segment
    // lengths and normals (from X0 + U directly, the same sums the coordinates hold)
    {
        unsigned long long kr0 = ~0ULL, kz0 = ~0ULL, kr1 = 0ULL, kz1 = 0ULL, lb = 0ULL;
        FOR_GRID(i, nodes) {
            const int n = d.surfNodes[i];
            const double2 x = d.X0[n], u = d.U[n];
            const double cr = x.x + u.x, cz = x.y + u.y;
            d.cr[n] = cr;
            d.cz[n] = cz;
            d.slaveXY[i] = make_double2(cr, cz);
            d.incCount[i] = 0;
            d.pairNodes[i] = make_int4(-1, -1, -1, 0);
            const unsigned long long kr = okey(cr), kz = okey(cz);
            kr0 = min(kr0, kr); kr1 = max(kr1, kr);
            kz0 = min(kz0, kz); kz1 = max(kz1, kz);
        }
        if (gt == 0) d.incCount[nodes] = 0;
        FOR_GRID(e, edges) {
            const int a = d.segA[e], b = d.segB[e];
            const double2 xa = d.X0[a], ua = d.U[a], xb = d.X0[b], ub = d.U[b];
            const double dr = (xb.x + ub.x) - (xa.x + ua.x);
            const double dz = (xb.y + ub.y) - (xa.y + ua.y);
            const double len = sqrt(dr * dr + dz * dz);
            d.slen[e] = len;
            if (len > 0.0) {
                d.snr[e] = dz / len;
                d.snz[e] = -dr / len;
            } else {
                d.snr[e] = 0.0;
                d.snz[e] = 0.0;
            }
            lb = max(lb, (unsigned long long)__double_as_longlong(len));
        }
        // extrema are exact in any order: reduce in the warp, one atomic per warp
        for (int o = 16; o > 0; o >>= 1) {
            kr0 = min(kr0, __shfl_down_sync(0xffffffffu, kr0, o));
            kz0 = min(kz0, __shfl_down_sync(0xffffffffu, kz0, o));
            kr1 = max(kr1, __shfl_down_sync(0xffffffffu, kr1, o));
            kz1 = max(kz1, __shfl_down_sync(0xffffffffu, kz1, o));
            lb = max(lb, __shfl_down_sync(0xffffffffu, lb, o));
        }
        if ((threadIdx.x & 31) == 0) {
            if (kr1 != 0ULL) {
                atomicMin(&s->bbox[0], kr0);
                atomicMin(&s->bbox[1], kz0);
                atomicMax(&s->bbox[2], kr1);
                atomicMax(&s->bbox[3], kz1);
            }
            if (lb != 0ULL) atomicMax(&s->longestBits, lb);
        }
    }
    SYNC();

    // the grid, in every block; node normals; the counting sort's counts (:530-545).
    // bucketCount is all zero on entry and is left all zero.
    if (threadIdx.x == 0) {
        grid_from_box(d, nodes, grid);
        if (blockIdx.x == 0) {
            s->cellSize = grid.cellSize;
            s->gridR0 = grid.r0;
            s->gridZ0 = grid.z0;
            s->cols = grid.cols;
            s->rows = grid.rows;
            s->cells = grid.cells;
            s->hashed = grid.hashed;
            s->bucketScanN = grid.bucketN;
            if (grid.hashed) atomicOr(&s->status, STATUS_GRID_HASHED);
        }
    }
    __syncthreads();
    const Grid g = grid;
    FOR_GRID(i, nodes) {
        double sr = 0.0, sz = 0.0;
        for (int k = d.segStart[i]; k < d.segStart[i + 1]; k++) {
            sr += d.snr[d.segOf[k]];
            sz += d.snz[d.segOf[k]];
        }
        const double len = sqrt(sr * sr + sz * sz);
        d.pnr[i] = len > 0.0 ? sr / len : 0.0;
        d.pnz[i] = len > 0.0 ? sz / len : 0.0;
    }
    FOR_GRID(q, 2 * edges) {
        const int e = q >> 1;
        const int node = (q & 1) ? d.segB[e] : d.segA[e];
        const long long cell = cell_of(g, d.cr[node], d.cz[node]);
        d.entryCell[q] = cell;
        atomicAdd(&d.bucketCount[bucket_of(d, g, cell)], 1);
    }
    SYNC();
    if (!grid_scan(d, d.bucketCount, d.bucketStart, d.bucketCursor, g.bucketN, nullptr, true))
        return;
    // file the entries; stage beside each what the search's gap test reads
    FOR_GRID(q, 2 * edges) {
        const long long cell = d.entryCell[q];
        const int e = q >> 1;
        const int a = d.segA[e];
        const int pos = atomicAdd(&d.bucketCursor[bucket_of(d, g, cell)], 1);
        d.bucketEntry[pos] = q;
        d.bucketCell[pos] = cell;
        d.bucketA[pos] = make_double2(d.cr[a], d.cz[a]);
        d.bucketN[pos] = make_double2(d.snr[e], d.snz[e]);
        d.bucketL[pos] = d.slen[e];
    }
    SYNC();

    // the search and the pair forces: each warp searches four slaves at a time, eight lanes
    // each, and the groups' first lanes then compute the four pairs' forces side by side (long
    // dependent chains of divisions). The totals are per-block partials, folded in a fixed
    // order at the step's end.
    {
        double energy = 0.0, diss = 0.0;
        const int warpsTotal = gridDim.x * CB_WARPS;
        const int group = (threadIdx.x & 31) / SG;
        for (int w = (threadIdx.x >> 5) * gridDim.x + blockIdx.x; w * (32 / SG) < nodes;
             w += warpsTotal) {
            const int slot = w * (32 / SG) + group;
            double best;
            int seg;
            bool fell;
            search_group(d, g, slot, nodes, best, seg, fell);
            if ((threadIdx.x & (SG - 1)) == 0 && slot < nodes)
                finish_slave(d, slot, best, seg, fell, energy, diss);
        }
        const double e1 = block_sum_c(energy, shd);
        const double e2 = block_sum_c(diss, shd);
        if (threadIdx.x == 0) {
            d.partials[(PARTIAL_CONTACT + 0) * d.maxBlocks + blockIdx.x] = e1;
            d.partials[(PARTIAL_CONTACT + 1) * d.maxBlocks + blockIdx.x] = e2;
        }
    }
    SYNC();
    const bool friction = d.cFriction > 0.0;
    if (!vload(&s->incOverflow)) {
        // each node adds its terms in slave order, normal then tangent (:717-754): the fixed
        // list, sorted in registers by an odd-even transposition network
        FOR_GRID(j, nodes) {
            const int c = d.incCount[j];
            if (c == 0) continue;
            int e[INC_CAP];
#pragma unroll
            for (int k = 0; k < INC_CAP; k++)
                e[k] = k < c ? d.incSlots[(size_t)j * INC_CAP + k] : 0x7fffffff;
#pragma unroll
            for (int r = 0; r < INC_CAP; r++) {
#pragma unroll
                for (int k = r & 1; k + 1 < INC_CAP; k += 2) {
                    const int x = min(e[k], e[k + 1]), y = max(e[k], e[k + 1]);
                    e[k] = x;
                    e[k + 1] = y;
                }
            }
            const int node = d.surfNodes[j];
            double2 f = d.F[node];
#pragma unroll
            for (int k = 0; k < INC_CAP; k++) {
                if (k < c) {
                    const double *pv = d.pairVal + 12 * (size_t)(e[k] >> 2) + 4 * (e[k] & 3);
                    f.x += pv[0];
                    f.y += pv[1];
                    if (friction) {
                        f.x += pv[2];
                        f.y += pv[3];
                    }
                }
            }
            d.F[node] = f;
        }
        return;
    }
    // the general path: incidence lists by a scan over the counts
    if (!grid_scan(d, d.incCount, d.incStart, d.incCursor, nodes + 1, nullptr, false)) return;
    FOR_GRID(i, nodes) {
        const int4 p = d.pairNodes[i];
        if (!p.w) continue;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.x]], 1)] = (i << 2) | 0;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.y]], 1)] = (i << 2) | 1;
        d.incEntry[atomicAdd(&d.incCursor[d.slotOf[p.z]], 1)] = (i << 2) | 2;
    }
    SYNC();
    FOR_GRID(j, nodes) {
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

#undef SYNC
#undef FOR_GRID

// ---------------------------------------------------------------------------- launch

// Blocks of the cooperative pass: as many as can be resident at once, at most four per SM.
// Fixed per device, so the partial sums have a fixed order. Needs the device current.
int contact_coop_blocks(int sms) {
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_contact_pass, CB, 0) != cudaSuccess ||
        perSm < 1)
        perSm = 1;
    if (perSm > MAX_COOP_BLOCKS_PER_SM) perSm = MAX_COOP_BLOCKS_PER_SM;
    return perSm * sms;
}

int launch_contact(Solver &S, bool) {
    Dev &d = S.d;
    void *args[] = {&d};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)d.coopBlocks);
    cfg.blockDim = dim3(CB);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = S.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelExC(&cfg, (const void *)k_contact_pass, args);
    return 1;
}

}  // namespace nf
