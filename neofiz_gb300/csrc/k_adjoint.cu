// k_adjoint.cu -- the hand-written adjoint of the batched FP64 timestep: gradients of a final
// measurement with respect to Johnson-Cook A, B, n, C, m, the kinematic hardening modulus and
// the wall friction. There is no adjoint in the reference.
//
// One block owns one instance. The forward kernel runs the instance to its t_end with the
// batched step (nf_batch_step.cuh, bit-identical to the plain path) and saves the whole state
// every `every` steps. The backward kernel walks the segments from the last: it restores the
// segment's checkpoint, re-runs the segment saving the state before each step (the tape) and
// each step's shortest edge, then runs the reverse of each step (nf_adjoint.h): the nodal
// update recomputed from the tape, the element reverse (its forward recomputed in the same
// order, so every branch is the forward's), the per-node gather of the elements' adjoints in
// the forward gather's order, the nodal reverse, and the CFL step's dependence on the
// shortest edge. Per-thread parameter adjoints are summed by a fixed tree at the end.
#include "nf_batch_step.cuh"
#include "nf_adjoint.h"

namespace nf {

constexpr int ADJ_T = 256;

// One saved state of an instance with n nodes and e elements, 16-byte aligned fields.
struct StateBlock {
    double2 *U, *V, *F, *hg;
    double *sig, *back, *epsP, *wP, *scal;   // scal: dt, dtPrevious, time, steps, minEdge
    double *dStr, *dSoft, *dWidth;           // damage state
    uint8_t *flags;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

size_t adj_state_bytes(int n, int e) {
    return 3 * al16(16 * (size_t)n) + 2 * al16(32 * (size_t)e) + al16(16 * (size_t)e)
           + 5 * al16(8 * (size_t)e) + 64 + al16((size_t)n);
}
size_t adj_bar_bytes(int n, int e, int k) {
    return 3 * al16(16 * (size_t)n) + 2 * al16(32 * (size_t)e) + al16(16 * (size_t)e)
           + 4 * al16(8 * (size_t)e) + al16(128 * (size_t)e) + al16(32 * (size_t)k);
}
size_t adj_seed_bytes(int n, int e) { return al16(16 * (size_t)n) + al16(32 * (size_t)e); }

__device__ StateBlock state_at(char *p, int n, int e) {
    StateBlock s;
    s.U = (double2 *)p; p += al16(16 * (size_t)n);
    s.V = (double2 *)p; p += al16(16 * (size_t)n);
    s.F = (double2 *)p; p += al16(16 * (size_t)n);
    s.sig = (double *)p; p += al16(32 * (size_t)e);
    s.back = (double *)p; p += al16(32 * (size_t)e);
    s.hg = (double2 *)p; p += al16(16 * (size_t)e);
    s.epsP = (double *)p; p += al16(8 * (size_t)e);
    s.wP = (double *)p; p += al16(8 * (size_t)e);
    s.dStr = (double *)p; p += al16(8 * (size_t)e);
    s.dSoft = (double *)p; p += al16(8 * (size_t)e);
    s.dWidth = (double *)p; p += al16(8 * (size_t)e);
    s.scal = (double *)p; p += 64;
    s.flags = (uint8_t *)p;
    return s;
}

// The adjoint arrays of an instance.
struct BarBlock {
    double2 *U, *V, *F, *hg;
    double *sig, *back, *epsP, *wP, *corner;   // corner: 16 per element (4 corners x ur uz vr vz)
    double *dStr, *dSoft;                      // damage state
    double *edge;                              // 4 per pressure edge: a (r, z), b (r, z)
};

__device__ BarBlock bar_at(char *p, int n, int e, int k) {
    BarBlock s;
    s.U = (double2 *)p; p += al16(16 * (size_t)n);
    s.V = (double2 *)p; p += al16(16 * (size_t)n);
    s.F = (double2 *)p; p += al16(16 * (size_t)n);
    s.sig = (double *)p; p += al16(32 * (size_t)e);
    s.back = (double *)p; p += al16(32 * (size_t)e);
    s.hg = (double2 *)p; p += al16(16 * (size_t)e);
    s.epsP = (double *)p; p += al16(8 * (size_t)e);
    s.wP = (double *)p; p += al16(8 * (size_t)e);
    s.dStr = (double *)p; p += al16(8 * (size_t)e);
    s.dSoft = (double *)p; p += al16(8 * (size_t)e);
    s.corner = (double *)p; p += al16(128 * (size_t)e);
    s.edge = (double *)p; p += al16(32 * (size_t)k);
    return s;
}

// Copies the instance's evolving state between the solver arrays and a block (save: to the
// block). Each node is copied by the thread that owns it in the step's node loops.
template <int T>
__device__ void copy_state(const Dev &d, const BatchInst &in, StateBlock s, bool save) {
    const int n = in.n1 - in.n0, e = in.e1 - in.e0;
    for (int i = threadIdx.x; i < n; i += T) {
        const int g = in.n0 + i;
        if (save) {
            s.U[i] = d.U[g]; s.V[i] = d.V[g]; s.F[i] = d.F[g]; s.flags[i] = d.flags[g];
        } else {
            d.U[g] = s.U[i]; d.V[g] = s.V[i]; d.F[g] = s.F[i]; d.flags[g] = s.flags[i];
        }
    }
    for (int j = threadIdx.x; j < e; j += T) {
        const int g = in.e0 + j;
        double2 *a = reinterpret_cast<double2 *>(d.sig + 4 * (size_t)g);
        double2 *b = reinterpret_cast<double2 *>(d.back + 4 * (size_t)g);
        double2 *sa = reinterpret_cast<double2 *>(s.sig + 4 * (size_t)j);
        double2 *sb = reinterpret_cast<double2 *>(s.back + 4 * (size_t)j);
        if (save) {
            sa[0] = a[0]; sa[1] = a[1]; sb[0] = b[0]; sb[1] = b[1];
            s.hg[j] = d.hg[g]; s.epsP[j] = d.epsP[g]; s.wP[j] = d.wP[g];
            if (d.hasDamage) {
                s.dStr[j] = d.dStrength[g]; s.dSoft[j] = d.dSoft[g]; s.dWidth[j] = d.dWidth[g];
            }
        } else {
            a[0] = sa[0]; a[1] = sa[1]; b[0] = sb[0]; b[1] = sb[1];
            d.hg[g] = s.hg[j]; d.epsP[g] = s.epsP[j]; d.wP[g] = s.wP[j];
            if (d.hasDamage) {
                d.dStrength[g] = s.dStr[j]; d.dSoft[g] = s.dSoft[j]; d.dWidth[g] = s.dWidth[j];
            }
        }
    }
}

__device__ nf_adj_mat adj_mat_of(const MatDev &m) {
    nf_adj_mat o;
    o.lambda = m.lambda; o.mu = m.mu; o.sy0 = m.sy0; o.hIso = m.hIso; o.hKin = m.hKin;
    o.a = m.a; o.b = m.b; o.n = m.n; o.c = m.c; o.m = m.m; o.refRate = m.refRate;
    o.room = m.room; o.melt = m.melt; o.thermalCoefficient = m.thermalCoefficient;
    o.jc = m.jc;
    return o;
}

// The element's inputs: reference and post-nodal node values from the solver arrays, the
// point state before the step from the tape block.
__device__ void elem_in(const Dev &d, const BatchInst &in, const StateBlock &pre, int le,
                        nf_adj_elem_in *x) {
    const int e = in.e0 + le;
    const int4 c = d.conn[e];
    const int nn[4] = {c.x, c.y, c.z, c.w};
    for (int k = 0; k < 4; k++) {
        const double2 x0 = d.X0[nn[k]], u = d.U[nn[k]], v = d.V[nn[k]];
        x->x0r[k] = x0.x; x->x0z[k] = x0.y;
        x->ur[k] = u.x; x->uz[k] = u.y;
        x->vr[k] = v.x; x->vz[k] = v.y;
        x->sig[k] = pre.sig[4 * le + k];
        x->back[k] = pre.back[4 * le + k];
    }
    x->epsP = pre.epsP[le];
    x->work = pre.wP[le];
    x->hgR = pre.hg[le].x;
    x->hgZ = pre.hg[le].y;
    x->damaged = d.hasDamage;
    if (d.hasDamage) {
        x->dm.failureStrain = d.dFail[e];
        x->dm.strength = pre.dStr[le];
        x->dm.softening = pre.dSoft[le];
        x->dm.fractureEnergy = d.dGf[e];
        x->dm.youngs = d.mats[d.emat[e]].youngs;
        x->dm.geometry = d.dGeom + 5 * (size_t)e;
    }
}

// BurstCase.loadCapacity (BurstCase.java:533-553) of the instance's current state: the hoop
// stress times the current element area summed by a fixed tree, over the bore radius and the
// height (exact extrema). Valid in every thread.
template <int T>
__device__ double capacity_of(const Dev &d, const BatchInst &in, double *shRed) {
    __shared__ double shExt[3];
    double hoop = 0.0;
    for (int e = in.e0 + threadIdx.x; e < in.e1; e += T) {
        const int4 c = d.conn[e];
        const int nn[4] = {c.x, c.y, c.z, c.w};
        double sum = 0.0;
        for (int k = 0; k < 4; k++) {
            const int i = nn[k], j = nn[(k + 1) & 3];
            const double2 xi = d.X0[i], xj = d.X0[j];
            double ri = xi.x, rj = xj.x, zi = xi.y, zj = xj.y;
            if (d.finite) {
                const double2 ui = d.U[i], uj = d.U[j];
                ri = xi.x + ui.x; rj = xj.x + uj.x; zi = xi.y + ui.y; zj = xj.y + uj.y;
            }
            sum += ri * zj - rj * zi;
        }
        hoop += d.sig[4 * (size_t)e + 2] * (0.5 * sum);
    }
    const double total = block_total<T>(hoop, shRed);
    double bore = DMAX, low = DMAX, high = -DMAX;
    for (int i = in.n0 + threadIdx.x; i < in.n1; i += T) {
        const double2 x = d.X0[i];
        double r = x.x, z = x.y;
        if (d.finite) {
            const double2 u = d.U[i];
            r = x.x + u.x;
            z = x.y + u.y;
        }
        bore = fmin(bore, r);
        low = fmin(low, z);
        high = fmax(high, z);
    }
    for (int o = 16; o > 0; o >>= 1) {
        bore = fmin(bore, __shfl_down_sync(0xffffffffu, bore, o));
        low = fmin(low, __shfl_down_sync(0xffffffffu, low, o));
        high = fmax(high, __shfl_down_sync(0xffffffffu, high, o));
    }
    if (threadIdx.x == 0) {
        shExt[0] = DMAX; shExt[1] = DMAX; shExt[2] = -DMAX;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        // order-free extrema of finite values: a lock-free min over warps through shared
        // memory would need atomics on doubles; the first thread folds the warps instead
        shRed[threadIdx.x >> 5] = bore;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 0; w < T / 32; w++) shExt[0] = fmin(shExt[0], shRed[w]);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) shRed[threadIdx.x >> 5] = low;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 0; w < T / 32; w++) shExt[1] = fmin(shExt[1], shRed[w]);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) shRed[threadIdx.x >> 5] = high;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < T / 32; w++) shExt[2] = fmax(shExt[2], shRed[w]);
        shRed[T / 32] = total / (shExt[0] * (shExt[2] - shExt[1]));
    }
    __syncthreads();
    const double cap = shRed[T / 32];
    __syncthreads();
    return cap;
}

// Forward: every instance to its t_end, a checkpoint every `every` steps, the final state.
__global__ void __launch_bounds__(ADJ_T) k_adj_forward(Dev d, BatchDev b, AdjDev a) {
    __shared__ double shMin[ADJ_T / 32 + 1];
    __shared__ int wallCount[2][2];
    const int k = blockIdx.x;
    const BatchInst in = b.inst[k];
    BatchScalars *scp = b.sc + k;
    const int n = in.n1 - in.n0, e = in.e1 - in.e0;
    double dt = scp->dt, dtPrev = scp->dtPrevious, time = scp->time;
    double minEdge = scp->minEdgeSquared;
    long long steps = scp->steps;
    double impulse = 0.0, loss = 0.0, fric = 0.0;
    if (threadIdx.x == 0) {
        wallCount[0][0] = wallCount[0][1] = wallCount[1][0] = wallCount[1][1] = 0;
    }
    __syncthreads();
    const MixedGeo none{nullptr, nullptr, nullptr, 0};
    char *ckpt = a.ckpt + a.ckptOff[k];
    const size_t bytes = a.stateBytes[k];
    double peak = -DMAX;
    long long peakStep = 0;
    int taken = 0;
    for (;; taken++) {
        if (!(time < in.tEnd)) break;
        if (steps % a.every == 0) {
            const long long c = steps / a.every;
            if (c >= a.ckptCap[k]) {
                if (threadIdx.x == 0) atomicOr(a.overflow, 1);
                break;
            }
            StateBlock s = state_at(ckpt + c * bytes, n, e);
            copy_state<ADJ_T>(d, in, s, true);
            if (threadIdx.x == 0) {
                s.scal[0] = dt; s.scal[1] = dtPrev; s.scal[2] = time;
                s.scal[3] = (double)steps; s.scal[4] = minEdge;
            }
        }
        const int par = taken & 1;
        if (threadIdx.x == 0) {
            wallCount[par ^ 1][0] = 0;
            wallCount[par ^ 1][1] = 0;
        }
        minEdge = batch_step<false, ADJ_T>(d, in, dt, dtPrev, time, steps, none, nullptr, nullptr,
                                           0, &scp->status, &wallCount[par][0],
                                           &wallCount[par][1], impulse, loss, fric, shMin);
        if (a.sampleEvery > 0 && steps % a.sampleEvery == 0) {
            __syncthreads();
            const double cap = capacity_of<ADJ_T>(d, in, shMin);
            if (cap > peak) {                  // the same decision in every thread
                peak = cap;
                peakStep = steps;
                StateBlock pk = state_at(a.peak + a.peakOff[k], n, e);
                copy_state<ADJ_T>(d, in, pk, true);
                if (threadIdx.x == 0) {
                    pk.scal[0] = dt; pk.scal[1] = dtPrev; pk.scal[2] = time;
                    pk.scal[3] = (double)steps; pk.scal[4] = minEdge;
                }
            }
        }
    }
    const double ti = block_total<ADJ_T>(impulse, shMin);
    const double tl = block_total<ADJ_T>(loss, shMin);
    const double tf = block_total<ADJ_T>(fric, shMin);
    StateBlock fin = state_at(a.fin + a.finOff[k], n, e);
    copy_state<ADJ_T>(d, in, fin, true);
    if (threadIdx.x == 0) {
        scp->dt = dt; scp->dtPrevious = dtPrev; scp->time = time; scp->steps = steps;
        scp->minEdgeSquared = minEdge;
        if (taken > 0) {
            scp->wContact = wallCount[(taken - 1) & 1][0];
            scp->wStuck = wallCount[(taken - 1) & 1][1];
        }
        scp->wImpulse += ti; scp->wEnergyLoss += tl; scp->wFriction += tf;
        scp->done = 1;
        a.steps[k] = steps;
        a.peakStep[k] = peakStep;
        a.peakValue[k] = peak;
        fin.scal[0] = dt; fin.scal[1] = dtPrev; fin.scal[2] = time; fin.scal[3] = (double)steps;
        fin.scal[4] = minEdge;
    }
}

// The reverse of one step whose pre-step state is `pre`.
// The wall counters and status word of the recomputed nodal update go to `scratch` (shared
// memory: atomics need a shared or global address).
__device__ void reverse_step(const Dev &d, const BatchInst &in, const MatDev &mat, StateBlock pre,
                             BarBlock bar, double *pacc, double *shRed, int *shOwner,
                             double *shDtb, double *shDtPrevb, double *shTimeb, int *scratch) {
    const int n = in.n1 - in.n0, e = in.e1 - in.e0;
    const double dt = pre.scal[0], dtPrev = pre.scal[1], minEdge = pre.scal[4];
    const double dtAvg = 0.5 * (dtPrev + dt);
    const double half = 0.5 * in.damping * dtAvg;
    const double decay = (1.0 - half) / (1.0 + half), gain = dtAvg / (1.0 + half);
    // u', v' of this step, from the tape
    {
        double i0 = 0.0, l0 = 0.0, f0 = 0.0;
        const NodalCoef co{decay, gain, dtAvg, dt};
        const WallRef w{in.hasWall, in.wallPlane, in.wallFriction, scratch, scratch + 1};
        const MixedGeo none{nullptr, nullptr, nullptr, 0};
        for (int i = threadIdx.x; i < n; i += ADJ_T) {
            const int g = in.n0 + i;
            d.U[g] = pre.U[i]; d.V[g] = pre.V[i]; d.F[g] = pre.F[i]; d.flags[g] = pre.flags[i];
            nodal_node(d, g, co, w, none, reinterpret_cast<uint32_t *>(scratch + 2), i0, l0, f0);
        }
    }
    if (threadIdx.x == 0) *shOwner = 0x7fffffff;
    __syncthreads();
    const int finite = d.finite;
    double edgeb = 0.0;
    if (finite && minEdge > 0.0 && minEdge < DMAX) {
        edgeb = *shDtb * in.cfl * sqrt(in.massScale) / in.wave * 0.5 / sqrt(minEdge);
        for (int le = threadIdx.x; le < e; le += ADJ_T) {
            nf_adj_elem_in x;
            elem_in(d, in, pre, le, &x);
            if (nf_adj_edge_owner(&x, dt, finite, minEdge) >= 0) atomicMin(shOwner, le);
        }
    }
    __syncthreads();
    const int owner = *shOwner;
    const nf_adj_mat m = adj_mat_of(mat);
    double dtb = 0.0;
    for (int le = threadIdx.x; le < e; le += ADJ_T) {
        nf_adj_elem_in x;
        elem_in(d, in, pre, le, &x);
        nf_adj_elem_bar ab;
        const int4 c = d.conn[in.e0 + le];
        const int nn[4] = {c.x - in.n0, c.y - in.n0, c.z - in.n0, c.w - in.n0};
        for (int k = 0; k < 4; k++) {
            ab.g[k] = bar.F[nn[k]].x;
            ab.g[4 + k] = bar.F[nn[k]].y;
            ab.sig[k] = bar.sig[4 * le + k];
            ab.back[k] = bar.back[4 * le + k];
        }
        ab.epsP = bar.epsP[le];
        ab.work = bar.wP[le];
        ab.hgR = bar.hg[le].x;
        ab.hgZ = bar.hg[le].y;
        ab.strength = d.hasDamage ? bar.dStr[le] : 0.0;
        ab.softening = d.hasDamage ? bar.dSoft[le] : 0.0;
        ab.edgeOwner = le == owner ? nf_adj_edge_owner(&x, dt, finite, minEdge) : -1;
        ab.edgeb = edgeb;
        nf_adj_element_reduced(&x, &m, dt, d.axi, finite, d.thickness, in.hourglass, &ab, &dtb,
                               pacc);
        for (int k = 0; k < 4; k++) {
            bar.sig[4 * le + k] = ab.sig[k];
            bar.back[4 * le + k] = ab.back[k];
            double *cr = bar.corner + 16 * (size_t)le + 4 * k;
            cr[0] = ab.ur[k]; cr[1] = ab.uz[k]; cr[2] = ab.vr[k]; cr[3] = ab.vz[k];
        }
        bar.epsP[le] = ab.epsP;
        bar.wP[le] = ab.work;
        bar.hg[le] = make_double2(ab.hgR, ab.hgZ);
        if (d.hasDamage) {
            bar.dStr[le] = ab.strength;
            bar.dSoft[le] = ab.softening;
        }
    }
    // pressure edges, loaded at this step's end time (:1203-1207, :1511-1556)
    double tpress = 0.0;
    const double tnow = pre.scal[2] + dt;
    for (int j = threadIdx.x; j < in.k1 - in.k0; j += ADJ_T) {
        const int2 ed = d.pedges[in.k0 + j];
        const int la = ed.x - in.n0, lb = ed.y - in.n0;
        const double cb[4] = {bar.F[la].x, bar.F[lb].x, bar.F[la].y, bar.F[lb].y};
        const double2 xa = d.X0[ed.x], xb = d.X0[ed.y], ua = d.U[ed.x], ub = d.U[ed.y];
        nf_adj_pressure_edge(xa.x, xa.y, xb.x, xb.y, ua.x, ua.y, ub.x, ub.y, tnow, in.pressure,
                             in.ramp, d.axi, finite, d.thickness, cb, bar.edge + 4 * (size_t)j,
                             bar.edge + 4 * (size_t)j + 2, &tpress);
    }
    __syncthreads();
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += ADJ_T) {
        const int g = in.n0 + i;
        double ub[2] = {bar.U[i].x, bar.U[i].y}, vb[2] = {bar.V[i].x, bar.V[i].y}, fb[2];
        for (int s = d.nodeSlotStart[g]; s < d.nodeSlotStart[g + 1]; s++) {
            const int slot = d.nodeSlot[s];
            if (slot >= 8 * d.E) {              // a pressure edge's slot
                const double *c = bar.edge + 4 * (size_t)((slot >> 3) - d.E - in.k0) + 2 * (slot & 7);
                ub[0] += c[0]; ub[1] += c[1];
                continue;
            }
            const double *cr = bar.corner + 16 * (size_t)((slot >> 3) - in.e0) + 4 * (slot & 7);
            ub[0] += cr[0]; ub[1] += cr[1]; vb[0] += cr[2]; vb[1] += cr[3];
        }
        const uint8_t fl = pre.flags[i];
        const double mass = d.mass[g];
        nf_adj_node(d.X0[g].y, pre.U[i].x, pre.U[i].y, pre.V[i].x, pre.V[i].y, pre.F[i].x,
                    pre.F[i].y, mass, d.invMass[g], fl & 1, (fl >> 1) & 1, (fl >> 2) & 1,
                    in.hasWall, in.wallPlane, in.wallFriction, decay, gain, dt, ub, vb, fb, acc);
        bar.U[i] = make_double2(ub[0], ub[1]);
        bar.V[i] = make_double2(vb[0], vb[1]);
        bar.F[i] = make_double2(fb[0], fb[1]);
    }
    pacc[NF_ADJ_P_MU] += acc[3];
    const double tDt = block_total<ADJ_T>(dtb + acc[2], shRed);
    const double tDecay = block_total<ADJ_T>(acc[0], shRed);
    const double tGain = block_total<ADJ_T>(acc[1], shRed);
    const double tTime = block_total<ADJ_T>(tpress, shRed);
    if (threadIdx.x == 0) {
        const double dtAvgb = nf_adj_dtavg(tDecay, tGain, dtAvg, in.damping);
        *shTimeb += tTime;                      // time' = time + dt
        *shDtb = *shDtPrevb + tDt + 0.5 * dtAvgb + *shTimeb;
        *shDtPrevb = 0.5 * dtAvgb;
    }
    __syncthreads();
}

// Backward: the reverse sweep over all steps of every instance, segment by segment.
__global__ void __launch_bounds__(ADJ_T) k_adj_backward(Dev d, BatchDev b, AdjDev a) {
    __shared__ double shMin[ADJ_T / 32 + 1];
    __shared__ double shRed[ADJ_T / 32 + 1];
    __shared__ int shOwner;
    __shared__ int scratch[3];                   // wall counts and status of recomputed steps
    __shared__ double shDtb[NF_ADJ_MAX_WIDTH], shDtPrevb[NF_ADJ_MAX_WIDTH];
    __shared__ double shTimeb[NF_ADJ_MAX_WIDTH];
    const int k = blockIdx.x;
    const int W = a.width;
    const BatchInst in = b.inst[k];
    const MatDev mat = d.mats[k];
    const int n = in.n1 - in.n0, e = in.e1 - in.e0;
    const long long N = a.steps[k];
    const size_t bytes = a.stateBytes[k];
    char *ckpt = a.ckpt + a.ckptOff[k];
    char *tape = a.tape + a.tapeOff[k];
    const int nk = in.k1 - in.k0;
    // per objective: its parameter adjoints, summed per thread over every step
    double pacc[NF_ADJ_MAX_WIDTH][NF_ADJ_P_COUNT];
    for (int w = 0; w < NF_ADJ_MAX_WIDTH; w++)
        for (int p = 0; p < NF_ADJ_P_COUNT; p++) pacc[w][p] = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < NF_ADJ_MAX_WIDTH; w++) shDtb[w] = shDtPrevb[w] = shTimeb[w] = 0.0;
        scratch[0] = scratch[1] = scratch[2] = 0;
    }
    __syncthreads();
    const MixedGeo none{nullptr, nullptr, nullptr, 0};
    uint32_t *scratchStatus = reinterpret_cast<uint32_t *>(scratch + 2);
    const long long segments = (N + a.every - 1) / a.every;
    for (long long sgi = segments - 1; sgi >= 0; sgi--) {
        StateBlock c = state_at(ckpt + sgi * bytes, n, e);
        copy_state<ADJ_T>(d, in, c, false);
        double dt = c.scal[0], dtPrev = c.scal[1], time = c.scal[2];
        long long steps = (long long)c.scal[3];
        __syncthreads();
        const long long start = sgi * a.every;
        const long long end = start + a.every < N ? start + a.every : N;
        double i0 = 0.0, l0 = 0.0, f0 = 0.0;
        for (long long j = start; j < end; j++) {
            StateBlock t = state_at(tape + (j - start) * bytes, n, e);
            copy_state<ADJ_T>(d, in, t, true);
            if (threadIdx.x == 0) {
                t.scal[0] = dt; t.scal[1] = dtPrev; t.scal[2] = time; t.scal[3] = (double)steps;
            }
            const double me = batch_step<false, ADJ_T>(d, in, dt, dtPrev, time, steps, none,
                                                       nullptr, nullptr, 0, scratchStatus,
                                                       &scratch[0], &scratch[1], i0, l0, f0,
                                                       shMin);
            if (threadIdx.x == 0) t.scal[4] = me;
        }
        __syncthreads();
        for (long long j = end - 1; j >= start; j--) {
            const StateBlock pre = state_at(tape + (j - start) * bytes, n, e);
            for (int w = 0; w < W; w++) {
                BarBlock bar = bar_at(a.bar + w * a.barPlane + a.barOff[k], n, e, nk);
                if (j == a.seedStep[(size_t)w * b.count + k] - 1) {
                    // objective w's seed enters after its step m
                    const char *sd = a.seed + w * a.seedPlane + a.seedOff[k];
                    const double2 *seedU = reinterpret_cast<const double2 *>(sd);
                    const double *seedSig =
                        reinterpret_cast<const double *>(sd + al16(16 * (size_t)n));
                    for (int i = threadIdx.x; i < n; i += ADJ_T) {
                        bar.U[i].x += seedU[i].x;
                        bar.U[i].y += seedU[i].y;
                    }
                    for (int q = threadIdx.x; q < 4 * e; q += ADJ_T) bar.sig[q] += seedSig[q];
                    __syncthreads();
                }
                // the forward values each objective's reverse reads are recomputed from the
                // same tape entry, so every objective sees the same bits
                reverse_step(d, in, mat, pre, bar, pacc[w], shRed, &shOwner, &shDtb[w],
                             &shDtPrevb[w], &shTimeb[w], scratch);
            }
        }
    }
    for (int w = 0; w < W; w++)
        for (int p = 0; p < NF_ADJ_P_COUNT; p++) {
            const double t = block_total<ADJ_T>(pacc[w][p], shRed);
            if (threadIdx.x == 0)
                a.grad[((size_t)w * b.count + k) * NF_ADJ_P_COUNT + p] = t;
        }
    // the solver arrays back to the forward's final state
    StateBlock fin = state_at(a.fin + a.finOff[k], n, e);
    copy_state<ADJ_T>(d, in, fin, false);
}

// Raises the context's per-thread stack limit to what the adjoint kernels' frames need (the
// reverse sweep spills registers) plus room for their non-inlined callees, if the limit is
// lower. The device call graph has no cycles, so the frames are fixed at compile time.
cudaError_t adjoint_reserve_stack() {
    size_t need = 0;
    const void *kernels[2] = {(const void *)k_adj_forward, (const void *)k_adj_backward};
    for (const void *f : kernels) {
        cudaFuncAttributes at;
        const cudaError_t e = cudaFuncGetAttributes(&at, f);
        if (e != cudaSuccess) return e;
        if (at.localSizeBytes > need) need = at.localSizeBytes;
    }
    need += 512;
    size_t cur = 0;
    const cudaError_t e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
    if (e != cudaSuccess) return e;
    return need > cur ? cudaDeviceSetLimit(cudaLimitStackSize, need) : cudaSuccess;
}

void launch_adjoint_forward(const Dev &d, const BatchDev &b, const AdjDev &a, cudaStream_t st) {
    if (b.count > 0) k_adj_forward<<<b.count, ADJ_T, 0, st>>>(d, b, a);
}

void launch_adjoint_backward(const Dev &d, const BatchDev &b, const AdjDev &a, cudaStream_t st) {
    if (b.count > 0) k_adj_backward<<<b.count, ADJ_T, 0, st>>>(d, b, a);
}

}  // namespace nf
