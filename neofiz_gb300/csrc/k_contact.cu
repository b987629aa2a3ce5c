// k_contact.cu -- penalty node-to-segment contact with a Coulomb cone
// (src/main/java/org/neofiz/solver/Contact.java), and the free-surface rebuild it needs after
// erosion (mesh/QuadMesh.java:188-226 via Contact.adopt, Contact.java:290-322).
//
// One cooperative, persistent kernel per step runs the whole contact pass as phases separated
// by grid-wide barriers: the surface rebuild (only on steps after an erosion), geometry, the
// counting-sort grid, the search, the pair forces and their ordered accumulation. It replaces
// some thirty launches of small kernels, whose launch gaps dominated the pass.
//
// A segment is named by its element edge q = 4 e + corner and a surface node by its node
// number, and all per-segment and per-node state is indexed by them. The reference numbers
// its segments by their rank among the free edges in element order and its surface nodes by
// rank in ascending node order; ranks are monotone in q and in the node number, so wherever
// the reference's answer depends on an order, ordering by q or by node number gives the same
// answer, and the surface needs no ordered lists at all: the free edges and the surface nodes
// are kept as lists in any order, appended to and struck out as erosion changes them, and
// each node keeps its own free edges in ascending q. After erosion only the edge groups of the
// eroded elements are re-flagged and only the nodes they touch are revisited (two phases);
// the first rebuild flags every element edge. Segment numbers are formed only when a caller
// reads them (the host ranks the free edges).
//
// The reference's result depends on three orders, and each is reproduced exactly:
//   * each node's segments, for its normal and its exclusion rings, in ascending segment
//     order (ascending q);
//   * the search visits the nine cells in (dj, di) order and, within a cell, the segments in
//     the order the counting sort filed them -- ascending segment, first endpoint before the
//     second (Contact.java:530-545, :578-603). Buckets are filled with atomics in any order;
//     each candidate carries its visit key (cell in the nine, 2 q + endpoint) instead, and
//     ties in depth go to the smallest key, the candidate the serial loop keeps;
//   * every node's force receives its contact terms in slave order, normal before tangent
//     (Contact.java:446-462, :717-754). Each pair's twelve terms are computed in parallel and
//     filed in fixed per-node lists of entries (slave node << 2 | role); each node then sorts
//     its list and adds in that order.
// The running totals (spring energy, dissipation) are audits: each slave's terms are kept per
// node and summed over a fixed grid of node numbers in a fixed order, so they are deterministic
// but not summed in the reference's serial order.
//
// The grid barrier is a counter and a generation word in device memory. The launch is
// cooperative, so every block is resident and the barrier cannot deadlock; its wait is bounded
// all the same: a block that waits longer than a second sets STATUS_TIMEOUT and an abort word
// that releases the others, and the kernel returns.
#include "nf_internal.h"
#include "nf_surface.cuh"

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

// Fixed-order block sum; the result is valid in thread 0. Leaves sh free for reuse. A warp of
// +0s skips its tree (its sum is +0 either way).
__device__ double block_sum_c(double v, double *sh) {
    if (__any_sync(0xffffffffu, __double_as_longlong(v) != 0))
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
    float screen;                // the FP32 screen's margin (search_group)
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
        g.screen = 0.0f;
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
    // every surface node lies within W = max(rhi - rlo, zhi - zlo) of the origin in each
    // coordinate; 2^-18 W bounds the FP32 screen's error twice over
    const double w = rhi - rlo > zhi - zlo ? rhi - rlo : zhi - zlo;
    g.screen = (float)(w * 0x1p-18);
}

__device__ __forceinline__ int iclamp(int v, int n) { return v < 0 ? 0 : v >= n ? n - 1 : v; }

__device__ __forceinline__ int bucket_of(const Dev &d, const Grid &g, long long cell) {
    return g.hashed ? (int)(cell % d.bucketCap) : (int)cell;
}

// Contact.depth, Contact.java:642-652
// The segment's unit tangent (cr[b] - cr[a]) / len, (cz[b] - cz[a]) / len is (-snz, snr) bit
// for bit: the geometry phase formed snr = dz / len and snz = -dr / len from the same sums
// (cr = x0 + u), and (-dr) / len is -(dr / len) exactly. Reading it saves two divisions.
__device__ __forceinline__ double depth_of(const Dev &d, int n, int q) {
    const int a = d.segA[q];
    const double len = d.slen[q];
    if (len <= 0.0) return 0.0;
    const double tr = -d.snz[q], tz = d.snr[q];
    const double dr = d.cr[n] - d.cr[a], dz = d.cz[n] - d.cz[a];
    const double along = dr * tr + dz * tz;
    if (along < 0.0 || along > len) return 0.0;
    const double gap = dr * d.snr[q] + dz * d.snz[q];
    return gap < 0.0 ? -gap : 0.0;
}

// Files one incident term (the pair of slave node m, role r, as m << 2 | r) in node j's fixed
// list; a list that overflows switches the step to the general path (a scan over the counts).
__device__ __forceinline__ void inc_push(const Dev &d, int j, int entry) {
    const int pos = atomicAdd(&d.incCount[j], 1);
    if (pos < INC_CAP) d.incSlots[(size_t)j * INC_CAP + pos] = entry;
    else d.s->incOverflow = 1;
}

// x is a normal number below 2^1000 in size (the exponent field alone).
__device__ __forceinline__ bool normal_below_2p1000(double x) {
    const unsigned e = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu;
    return e - 1u < 2022u;
}

// Contact.accumulate + resolve, Contact.java:446-462, :663-762, for slave node n and its
// master segment q: writes the pair's twelve force terms as values to ADD (x - y is computed
// as x + (-y), the same IEEE result) and files them at the pair's three nodes; keeps the
// pair's spring energy and dissipation at the slave.
__device__ void resolve_pair(const Dev &d, int n, int q) {
    const double dt = d.s->dt;
    const double reference = d.dt0;
    const int a = d.segA[q], b = d.segB[q];
    const double depth = depth_of(d, n, q);
    const double len = d.slen[q];
    const double tr = -d.snz[q];                            // parameter, :655-661 (the
    const double tz = d.snr[q];                             // tangent as in depth_of)
    const double t = ((d.cr[n] - d.cr[a]) * tr + (d.cz[n] - d.cz[a]) * tz) / len;
    const double wa = 1.0 - t, wb = t;
    const double ma = d.mass[a], mb = d.mass[b];
    // 0.25 / m is 0.25 (1 / m) exactly for a normal mass below 2^1000 (a power of two scales
    // a rounded quotient without rounding again), and 1 / m is the kept invMass
    const double qa = normal_below_2p1000(ma) ? 0.25 * d.invMass[a] : 0.25 / ma;
    const double qb = normal_below_2p1000(mb) ? 0.25 * d.invMass[b] : 0.25 / mb;
    const double invMaster = qa + qb;
    if (!(invMaster > 0.0)) return;
    const double mMaster = 1.0 / invMaster;
    const double mSlave = d.mass[n];
    const double mStar = mSlave * mMaster / (mSlave + mMaster);
    const double k = d.cScale * mStar / (reference * reference);
    const double nR = d.snr[q], nZ = d.snz[q];
    const double mTrue = 1.0 / (wa * wa / ma + wb * wb / mb);
    const double mTangent = mSlave * mTrue / (mSlave + mTrue);
    const double2 vn = d.V[n], va = d.V[a], vb = d.V[b];
    const double closing = (vn.x - wa * va.x - wb * vb.x) * nR
                           + (vn.y - wa * va.y - wb * vb.y) * nZ;
    const double damper = 2.0 * d.cDamping * mStar * d.cSqrtScale / reference;
    const double normal = jmax(0.0, k * depth - damper * closing);
    double *pv = d.pairVal + 12 * (size_t)n;
    pv[0] = normal * nR;
    pv[1] = normal * nZ;
    pv[4] = -(wa * normal * nR);
    pv[5] = -(wa * normal * nZ);
    pv[8] = -(wb * normal * nR);
    pv[9] = -(wb * normal * nZ);
    atomicAdd(&d.s->pairs, 1);
    d.pairEnergy[n] = 0.5 * k * depth * depth;
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
    d.pairDiss[n] = dthis;
    d.contactState[n] = state;
    d.pairNodes[n] = make_int4(n, a, b, 1);
    inc_push(d, n, (n << 2) | 0);
    inc_push(d, a, (n << 2) | 1);
    inc_push(d, b, (n << 2) | 2);
}

// Contact.nearestPenetrated (Contact.java:570-606) for 32 / SG slaves per warp, SG lanes (a
// group) each: the deepest admissible segment and whether the last step's master was seen too
// deep. Entry idx of the surface-node list is the group's slave (none when idx is past the
// list or struck out). The nine bucket ranges are concatenated and the lanes take the
// candidates round-robin; every candidate carries its visit key (cell in the nine, then the
// bucket entry 2 q + end): ties in depth go to the smallest key, the candidate the serial loop
// keeps, so neither the buckets nor the order the lanes test in matter.
//
// An FP32 screen first drops every candidate the exact test would reject for lying in front of
// the segment or beyond its ends: positions relative to the grid origin are below W (the
// larger box side) in size, so the FP32 gap and projection differ from the FP64 ones by less
// than 2^-19 W, and a candidate is dropped only when its FP32 value clears the bound by
// 2^-18 W (g.screen). The few that pass take the exact FP64 test, each lane its own. The
// grid's buckets as the search reads them: the counting-sort layout (bucket b's entries at
// [start[b], start[b + 1]), each with its cell) or the direct-indexed one (cell c's entries at
// [c cap, c cap + count[c]), every entry in its own cell).
struct BucketView {
    const int32_t *start, *count;
    const long long *cell;                     // null in the direct-indexed layout
    const int32_t *entry;
    const float4 *f;                           // first node - grid origin, normal (FP32)
    const float *fl;                           // length (FP32)
    const int2 *ab;                            // the segment's ends
    const double2 *a, *n;                      // its first node and normal
    const double *l;                           // its length
    int cap;                                   // 0: the counting-sort layout
};
__device__ __forceinline__ void bucket_range(const BucketView &v, int b, int &lo, int &len) {
    if (v.cap) {
        lo = b * v.cap;
        len = v.count[b];
    } else {
        lo = v.start[b];
        len = v.start[b + 1] - lo;
    }
}

constexpr int SG = 8;                          // lanes per slave
constexpr int KEPT = 4;                        // screened candidates a lane keeps for later
constexpr int OWN_KEPT = 4;                    // a slave's own segments held in registers
__device__ void search_group(const Dev &d, const Grid &g, const BucketView &v, int idx,
                             int listLen, double &bestOut, int &segOut, bool &fellOut) {
    const int lane = threadIdx.x & 31, gl = lane & (SG - 1);
    int n = idx < listLen ? d.nodeList[idx] : -1;
    const bool live = n >= 0;
    double2 xn = make_double2(0.0, 0.0), pn = make_double2(0.0, 0.0);
    float xs = 0.0f, ys = 0.0f;
    int last = -1, ci = 0, cj = 0;
    // the slave's own ring (Contact.excluded's second half): its free edges' ends, the first
    // OWN_KEPT in registers
    int ownCount = 0, ownP[OWN_KEPT], ownR[OWN_KEPT];
#pragma unroll
    for (int k = 0; k < OWN_KEPT; k++) ownP[k] = ownR[k] = -1;
    if (live) {
        xn = make_double2(d.cr[n], d.cz[n]);
        pn = make_double2(d.pnr[n], d.pnz[n]);
        last = d.lastMaster[n];
        const int2 cell = d.nodeCell[n];
        ci = cell.x;
        cj = cell.y;
        xs = (float)(xn.x - g.r0);
        ys = (float)(xn.y - g.z0);
        ownCount = d.nodeFree[n];
        const int32_t *own = d.nodeSeg + (size_t)n * d.segCap;
#pragma unroll
        for (int k = 0; k < OWN_KEPT; k++) {
            if (k < ownCount) {
                const int q = own[k];
                ownP[k] = d.segA[q];
                ownR[k] = d.segB[q];
            }
        }
    }
    // the nine cells in visit order: lane gl takes cell gl, lane 0 also cell 8
    int lo = 0, len = 0, lo8 = 0, len8 = 0;
    long long myCell = -1, cell8 = -1;
    if (live) {
        const int j = cj + gl / 3 - 1, ii = ci + gl % 3 - 1;
        if (j >= 0 && j < g.rows && ii >= 0 && ii < g.cols) {
            myCell = (long long)j * g.cols + ii;
            bucket_range(v, bucket_of(d, g, myCell), lo, len);
        }
        if (gl == 0) {
            const int j8 = cj + 1, i8 = ci + 1;
            if (j8 < g.rows && i8 < g.cols) {
                cell8 = (long long)j8 * g.cols + i8;
                bucket_range(v, bucket_of(d, g, cell8), lo8, len8);
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
    // every lane keeps the group's nine ranges (start in the concatenation, first slot, cell)
    int offs[8], los[8];
    long long cellq[8];
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
        offs[qq] = __shfl_sync(0xffffffffu, off, qq, SG);
        los[qq] = __shfl_sync(0xffffffffu, lo, qq, SG);
        cellq[qq] = __shfl_sync(0xffffffffu, myCell, qq, SG);
    }
    // position t of the concatenation: its range c (0..8), its slot k and the range's cell
    auto locate = [&](int t, int &c, int &k, long long &cc) {
        c = 0;
        int oc = offs[0], lc = los[0];
        cc = cellq[0];
#pragma unroll
        for (int qq = 1; qq < 8; qq++) {
            if (t >= offs[qq]) {
                c = qq;
                oc = offs[qq];
                lc = los[qq];
                cc = cellq[qq];
            }
        }
        if (t >= off8) {
            c = 8;
            oc = off8;
            lc = lo8;
            cc = cell8;
        }
        k = lc + (t - oc);
    };
    double best = 0.0;
    unsigned long long bestKey = ~0ULL;
    int bestSeg = -1;
    bool fell = false;
    // the exact test of position t (Contact.depth, Contact.java:642-652, and the exclusions):
    // the segment's ends, first node, normal and length as the filing staged them beside the
    // entry (the values the geometry phase left)
    auto exact = [&](int t) {
        int c, k;
        long long cc;
        locate(t, c, k, cc);
        if (v.cell && v.cell[k] != cc) return;          // a hashed bucket shares cells
        const int entry = v.entry[k];
        const int sg = entry >> 1;
        const double2 pa = v.a[k], nq = v.n[k];
        const double dr = xn.x - pa.x, dz = xn.y - pa.y;
        const double gap = dr * nq.x + dz * nq.y;
        if (!(gap < 0.0)) return;
        const double slen = v.l[k];
        if (slen <= 0.0) return;
        const double along = dr * -nq.y + dz * nq.x;
        if (along < 0.0 || along > slen) return;
        const double depth = -gap;
        // Contact.excluded (Contact.java:620-639): facing, an end of its own, or sharing a node
        // with one of the slave's own segments; a candidate that fails it is skipped whatever
        // its depth, so testing it after the depth changes nothing
        if (pn.x * nq.x + pn.y * nq.y > -FACING) return;
        const int2 ab = v.ab[k];
        if (ab.x == n || ab.y == n) return;
        bool ring = false;
#pragma unroll
        for (int j = 0; j < OWN_KEPT; j++)
            ring = ring || (j < ownCount && (ownP[j] == ab.x || ownP[j] == ab.y ||
                                             ownR[j] == ab.x || ownR[j] == ab.y));
        if (!ring && ownCount > OWN_KEPT) {
            const int32_t *own = d.nodeSeg + (size_t)n * d.segCap;
            for (int j = OWN_KEPT; j < ownCount && !ring; j++) {
                const int p = d.segA[own[j]], r = d.segB[own[j]];
                ring = p == ab.x || p == ab.y || r == ab.x || r == ab.y;
            }
        }
        if (ring) return;
        if (depth > MAX_DEPTH * slen) {
            if (sg == last) fell = true;
            return;
        }
        const unsigned long long key = ((unsigned long long)c << 32) | (unsigned int)entry;
        if (depth > best || (depth == best && key < bestKey)) {
            best = depth;
            bestKey = key;
            bestSeg = sg;
        }
    };
    int kept[KEPT];
#pragma unroll
    for (int j = 0; j < KEPT; j++) kept[j] = -1;
    for (int t = gl; t < total; t += SG) {
        int c, k;
        long long cc;
        locate(t, c, k, cc);
        const float4 f = v.f[k];
        const float dr = xs - f.x, dz = ys - f.y;
        if (dr * f.z + dz * f.w > g.screen) continue;
        const float along = dr * -f.w + dz * f.z;
        if (along < -g.screen || along > v.fl[k] + g.screen) continue;
        bool placed = false;
#pragma unroll
        for (int j = 0; j < KEPT; j++) {
            if (!placed && kept[j] < 0) {
                kept[j] = t;
                placed = true;
            }
        }
        if (!placed) exact(t);
    }
#pragma unroll
    for (int j = 0; j < KEPT; j++)
        if (kept[j] >= 0) exact(kept[j]);
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

// The pair of slave node n from its search (Contact.java:446-462): master, last master, the
// escape count and the pair forces; one lane.
__device__ void finish_slave(const Dev &d, int n, double best, int bestSeg, bool anyFell) {
    const int last = d.lastMaster[n];
    d.master[n] = best > 0.0 ? bestSeg : -1;
    if (!(best > 0.0)) {                      // no pair: Contact.java:446-452
        if (last >= 0 && anyFell) atomicAdd(&d.s->escaped, 1);
        d.lastMaster[n] = -1;
        return;
    }
    d.lastMaster[n] = bestSeg;
    resolve_pair(d, n, bestSeg);
}

// ---------------------------------------------------------------------------- the pass

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
    const bool rebuilt = vload(&s->stale) != 0;
    // the surface changed this step, here or in the gather's launch (surface_rebuild_block)
    const bool changed = rebuilt || vload(&s->rebuiltNow) != 0;

    if (rebuilt) {
        // Contact.adopt, Contact.java:290-322: the free surface, QuadMesh.surface over the
        // live elements (QuadMesh.java:188-226): an element edge is free when it is the only
        // live member of its group of equal edges
        const int epoch = vload(&s->rebuildEpoch) + 1;
        if (vload(&s->fullRebuild)) {
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
                d.nodeFree[n] = 0;
                d.nodePos[n] = -1;
                d.pairNodes[n] = make_int4(-1, -1, -1, 0);
                d.incCount[n] = 0;
            }
            if (gt == 0) {
                s->edgeListLen = 0;
                s->nodeListLen = 0;
            }
            SYNC();
            FOR_GRID(q, 4 * d.E) {
                if (!d.surfFlag[q]) {
                    d.edgePos[q] = -1;
                    continue;
                }
                const int pos = atomicAdd(&s->edgeListLen, 1);
                d.edgeList[pos] = q;
                d.edgePos[q] = pos;
                atomicAdd(&d.nodeFree[d.segA[q]], 1);
                atomicAdd(&d.nodeFree[d.segB[q]], 1);
            }
            SYNC();
            FOR_GRID(n, d.N) {
                if (d.nodeFree[n] == 0) continue;
                const int pos = atomicAdd(&s->nodeListLen, 1);
                d.nodeList[pos] = n;
                d.nodePos[n] = pos;
                build_node_segs(d, n);
            }
            if (gt == 0) {
                s->surfEdges = vload(&s->edgeListLen);
            }
        } else {
            // only the edge groups of the elements eroded since the last rebuild can change:
            // re-flag their members (each once: the epoch stamp), append the edges that became
            // free to the list and strike out those that stopped being free, keep each node's
            // count of free edges, and note the nodes touched
            const SurfaceCounters k{&s->edgeListLen, &s->surfEdges, &s->nTouched,
                                    &s->nodeListLen, &s->surfNodes};
            const int nDead = vload(&s->newDeadCount);
            FOR_GRID(t, 4 * nDead) surface_reflag(d, t, epoch, k);
            SYNC();
            // the touched nodes: join or leave the surface, and list their free edges again
            const int nTouched = vload(&s->nTouched);
            FOR_GRID(i, nTouched) surface_touched(d, i, k);
        }
        if (gt == 0) {
            s->stale = 0;
            s->newDeadCount = 0;
            s->rebuildEpoch = epoch;
        }
        const bool full = vload(&s->fullRebuild) != 0;
        SYNC();
        // after a full rebuild the list has no struck-out entries: its length is the count
        if (gt == 0) {
            if (full) {
                s->surfNodes = vload(&s->nodeListLen);
                s->fullRebuild = 0;
            }
            s->nTouched = 0;
        }
    }
    const int nodeLen = vload(&s->nodeListLen), edgeLen = vload(&s->edgeListLen);

    // Contact.geometry, Contact.java:467-500: current coordinates, the bounding box, segment
    // lengths and normals (from X0 + U directly, the same sums the coordinates hold). After a
    // rebuild every surface node forgets its last master (Contact.adopt, :319-321).
    {
        unsigned long long kr0 = ~0ULL, kz0 = ~0ULL, kr1 = 0ULL, kz1 = 0ULL, lb = 0ULL;
        FOR_GRID(i, nodeLen) {
            const int n = d.nodeList[i];
            if (n < 0) continue;
            const double2 x = d.X0[n], u = d.U[n];
            const double cr = x.x + u.x, cz = x.y + u.y;
            d.cr[n] = cr;
            d.cz[n] = cz;
            d.incCount[n] = 0;
            d.pairNodes[n] = make_int4(-1, -1, -1, 0);
            if (changed) {
                d.lastMaster[n] = -1;
                d.master[n] = -1;
                d.dropped[n] = 0;
            }
            const unsigned long long kr = okey(cr), kz = okey(cz);
            kr0 = min(kr0, kr); kr1 = max(kr1, kr);
            kz0 = min(kz0, kz); kz1 = max(kz1, kz);
        }
        if (gt == 0) d.incCount[d.N] = 0;
        FOR_GRID(i, edgeLen) {
            const int q = d.edgeList[i];
            if (q < 0) continue;
            const int a = d.segA[q], b = d.segB[q];
            const double2 xa = d.X0[a], ua = d.U[a], xb = d.X0[b], ub = d.U[b];
            const double dr = (xb.x + ub.x) - (xa.x + ua.x);
            const double dz = (xb.y + ub.y) - (xa.y + ua.y);
            const double len = sqrt(dr * dr + dz * dz);
            d.slen[q] = len;
            if (len > 0.0) {
                d.snr[q] = dz / len;
                d.snz[q] = -dr / len;
            } else {
                d.snr[q] = 0.0;
                d.snz[q] = 0.0;
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
    if (gt == 0) s->rebuiltNow = 0;             // every block has read it

    // the grid, in every block; node normals; the counting sort's counts (:530-545).
    // bucketCount is all zero on entry and is left all zero.
    const int nodes = vload(&s->surfNodes);
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
    // Per surface node: its normal from its segments in ascending order; its grid cell, once
    // (the search reads it for the node as a slave); and the filing of every segment end at the
    // node under that cell. A grid of at most fastCells - 1 cells is indexed directly: each
    // entry takes the next of its cell's slots (fastLimit of the fastCap reserved) and is filed
    // there at once, with the FP32 values the search's screen reads. A larger (or hashed) grid,
    // or a cell that outgrows its slots, takes the counting sort: the counts, an exclusive
    // scan, the filing.
    const bool fast = !g.hashed && g.cells < d.fastCells;
    FOR_GRID(i, nodeLen) {
        const int n = d.nodeList[i];
        if (n < 0) continue;
        const int32_t *own = d.nodeSeg + (size_t)n * d.segCap;
        const int count = d.nodeFree[n];
        double sr = 0.0, sz = 0.0;
        for (int k = 0; k < count; k++) {
            sr += d.snr[own[k]];
            sz += d.snz[own[k]];
        }
        const double len = sqrt(sr * sr + sz * sz);
        d.pnr[n] = len > 0.0 ? sr / len : 0.0;
        d.pnz[n] = len > 0.0 ? sz / len : 0.0;
        // Contact.cellOf, Contact.java:553-557
        const int ci = iclamp(jd2i((d.cr[n] - g.r0) / g.cellSize), g.cols);
        const int cj = iclamp(jd2i((d.cz[n] - g.z0) / g.cellSize), g.rows);
        d.nodeCell[n] = make_int2(ci, cj);
        const long long cell = (long long)cj * g.cols + ci;
        // the node's ends, two at a time: both slots are claimed before either is written, so
        // the atomics' round trips overlap
        for (int k0 = 0; k0 < count; k0 += 2) {
            int qs[2], as[2], pos[2];
#pragma unroll
            for (int j = 0; j < 2; j++) {
                qs[j] = k0 + j < count ? own[k0 + j] : -1;
                as[j] = qs[j] >= 0 ? d.segA[qs[j]] : -1;
                pos[j] = fast && qs[j] >= 0 ? atomicAdd(&d.fastCount[cell], 1) : 0;
            }
#pragma unroll
            for (int j = 0; j < 2; j++) {
                if (qs[j] < 0) continue;
                const int q = qs[j], a = as[j];
                const int entry = 2 * q + (a == n ? 0 : 1);
                d.entryCell[entry] = cell;
                if (fast) {
                    if (pos[j] < d.fastLimit) {
                        const size_t slot = (size_t)cell * d.fastCap + pos[j];
                        const double2 pa = make_double2(d.cr[a], d.cz[a]);
                        const double2 nq = make_double2(d.snr[q], d.snz[q]);
                        const double lq = d.slen[q];
                        d.fastEntry[slot] = entry;
                        d.fastF[slot] = make_float4((float)(pa.x - g.r0), (float)(pa.y - g.z0),
                                                    (float)nq.x, (float)nq.y);
                        d.fastFL[slot] = (float)lq;
                        d.fastAB[slot] = make_int2(a, d.segB[q]);
                        d.fastA[slot] = pa;
                        d.fastN[slot] = nq;
                        d.fastL[slot] = lq;
                    } else {
                        s->fastOverflow = 1;
                    }
                } else {
                    atomicAdd(&d.bucketCount[bucket_of(d, g, cell)], 1);
                }
            }
        }
    }
    SYNC();
    const bool direct = fast && !vload(&s->fastOverflow);
    if (!direct) {
        if (!grid_scan(d, fast ? d.fastCount : d.bucketCount, d.bucketStart, d.bucketCursor,
                       g.bucketN, nullptr, true))
            return;
        FOR_GRID(t, 2 * edgeLen) {
            const int q = d.edgeList[t >> 1];
            if (q < 0) continue;
            const int entry = 2 * q + (t & 1);
            const long long cell = d.entryCell[entry];
            const int a = d.segA[q];
            const int pos = atomicAdd(&d.bucketCursor[bucket_of(d, g, cell)], 1);
            const double2 pa = make_double2(d.cr[a], d.cz[a]);
            const double2 nq = make_double2(d.snr[q], d.snz[q]);
            const double lq = d.slen[q];
            d.bucketEntry[pos] = entry;
            d.bucketCell[pos] = cell;
            d.bucketF[pos] = make_float4((float)(pa.x - g.r0), (float)(pa.y - g.z0),
                                         (float)nq.x, (float)nq.y);
            d.bucketFL[pos] = (float)lq;
            d.bucketAB[pos] = make_int2(a, d.segB[q]);
            d.bucketA[pos] = pa;
            d.bucketN[pos] = nq;
            d.bucketL[pos] = lq;
        }
        SYNC();
    }
    BucketView view;
    if (direct) {
        view = BucketView{nullptr, d.fastCount, nullptr, d.fastEntry, d.fastF, d.fastFL,
                          d.fastAB, d.fastA, d.fastN, d.fastL, d.fastCap};
    } else {
        view = BucketView{d.bucketStart, nullptr, d.bucketCell, d.bucketEntry, d.bucketF,
                          d.bucketFL, d.bucketAB, d.bucketA, d.bucketN, d.bucketL, 0};
    }

    // the search and the pair forces: each warp searches 32 / SG slaves at a time, SG lanes
    // each, and the groups' first lanes then compute the pairs' forces side by side (long
    // dependent chains of divisions)
    {
        const int warpsTotal = gridDim.x * CB_WARPS;
        const int group = (threadIdx.x & 31) / SG;
        for (int w = (threadIdx.x >> 5) * gridDim.x + blockIdx.x; w * (32 / SG) < nodeLen;
             w += warpsTotal) {
            const int idx = w * (32 / SG) + group;
            double best;
            int seg;
            bool fell;
            search_group(d, g, view, idx, nodeLen, best, seg, fell);
            if ((threadIdx.x & (SG - 1)) == 0 && idx < nodeLen) {
                const int n = d.nodeList[idx];
                if (n >= 0) finish_slave(d, n, best, seg, fell);
            }
        }
    }
    SYNC();
    if (direct) FOR_GRID(c, (int)g.cells) d.fastCount[c] = 0;   // all zero again for the next step
    const bool friction = d.cFriction > 0.0;
    // the pairs' spring energy and dissipation, summed over a fixed grid of node numbers
    {
        double energy = 0.0, diss = 0.0;
        FOR_GRID(n, d.N) {
            if (d.pairNodes[n].w) {
                energy += d.pairEnergy[n];
                diss += d.pairDiss[n];
            }
        }
        const double e1 = block_sum_c(energy, shd);
        const double e2 = block_sum_c(diss, shd);
        if (threadIdx.x == 0) {
            d.partials[(PARTIAL_CONTACT + 0) * d.maxBlocks + blockIdx.x] = e1;
            d.partials[(PARTIAL_CONTACT + 1) * d.maxBlocks + blockIdx.x] = e2;
        }
    }
    if (!vload(&s->incOverflow)) {
        // each node adds its terms in slave order, normal then tangent (:717-754): the fixed
        // list, sorted in registers by an odd-even transposition network
        FOR_GRID(i, nodeLen) {
            const int node = d.nodeList[i];
            if (node < 0) continue;
            const int c = d.incCount[node];
            if (c == 0) continue;
            int e[INC_CAP];
#pragma unroll
            for (int k = 0; k < INC_CAP; k++)
                e[k] = k < c ? d.incSlots[(size_t)node * INC_CAP + k] : 0x7fffffff;
#pragma unroll
            for (int r = 0; r < INC_CAP; r++) {
#pragma unroll
                for (int k = r & 1; k + 1 < INC_CAP; k += 2) {
                    const int x = min(e[k], e[k + 1]), y = max(e[k], e[k + 1]);
                    e[k] = x;
                    e[k + 1] = y;
                }
            }
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
    // the general path: incidence lists by a scan over every node's count
    if (!grid_scan(d, d.incCount, d.incStart, d.incCursor, d.N + 1, nullptr, false)) return;
    FOR_GRID(i, nodeLen) {
        const int m = d.nodeList[i];
        if (m < 0) continue;
        const int4 p = d.pairNodes[m];
        if (!p.w) continue;
        d.incEntry[atomicAdd(&d.incCursor[p.x], 1)] = (m << 2) | 0;
        d.incEntry[atomicAdd(&d.incCursor[p.y], 1)] = (m << 2) | 1;
        d.incEntry[atomicAdd(&d.incCursor[p.z], 1)] = (m << 2) | 2;
    }
    SYNC();
    FOR_GRID(i, nodeLen) {
        const int node = d.nodeList[i];
        if (node < 0) continue;
        const int lo = d.incStart[node], hi = d.incStart[node + 1];
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
