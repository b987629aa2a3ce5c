// k_mixed.cu -- the mixed-precision form of the timestep: element constitutive, hourglass and
// force arithmetic in FP32 with FP32 element state; nodal kinematics, the per-node force
// gather, contact and every audit stay FP64.
//
// The element kernel never touches FP64. Absolute coordinates in FP32 would lose the element
// geometry (a 0.05 mm element 20 mm from the origin keeps only ~5 significant digits), so the
// nodal update (k_prepare_mixed before the first step) writes each node's mid-step and current
// positions as a pair of floats (hi = fl(P), lo = fl(P - hi), split by integer arithmetic in
// nf_fpconv.h with the conversions' bits); an element forms its edge vectors as
// (hi_i - hi_0) + (lo_i - lo_0), which is exact in the first term (Sterbenz) and rounds once,
// i.e. the difference to FP32 precision. The element kernel restates reducedIntegration
// (ExplicitSolver.java:1373-1504) and fullIntegration (:1219-1339) in float on those
// relative coordinates (B and strains are translation invariant; the axisymmetric radius is
// formed from the hi parts).
#include "nf_bodies.cuh"

namespace nf {

constexpr int MB = 128;

__device__ __forceinline__ unsigned long long dbits_m(double x) {
    return (unsigned long long)__double_as_longlong(x);
}

// Per node: mid-step position (for the B matrix), current position (for the inversion test)
// as float pairs, and the displacement increment v * strainDt as floats.
__global__ void k_prepare_mixed(Dev d, int zeroStrain) {
    if (!d.s->active) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    prepare_node(d, i, zeroStrain ? 0.0 : d.s->dt, MixedGeo{d.pMid, d.pCur, d.vdt, 0});
}

// Element damage (mean over points) and signed current area, FP32 (:663-691): whether live
// element e goes, adding the strain energy it held to energy.
__device__ __forceinline__ void erode_element_mixed(const Dev &d, int e, double &energy) {
    if (d.gone[e]) return;
    bool failed = false;
    if (d.hasDamage) {
        float sum = 0.0f;
        for (int g = 0; g < d.ppe; g++) {
            const int p = e * d.ppe + g;
            sum += damage_at(d.dStrF[p], d.dSoftF[p], d.dFailF[e], d.epsPF[p]);
        }
        failed = sum / d.ppe >= (float)d.erosionDamage;
    }
    const int4 c = d.conn[e];
    const float4 p0 = d.pCur[c.x], p1 = d.pCur[c.y], p2 = d.pCur[c.z], p3 = d.pCur[c.w];
    const float r1 = diff_hl(p1, p0, 0), r2 = diff_hl(p2, p0, 0), r3 = diff_hl(p3, p0, 0);
    const float z1 = diff_hl(p1, p0, 1), z2 = diff_hl(p2, p0, 1), z3 = diff_hl(p3, p0, 1);
    // shoelace with node 0 at the origin
    const float a = (r1 * z2 - r2 * z1) + (r2 * z3 - r3 * z2);
    const bool inverted = 0.5f * a <= 0.0f;
    if (failed || inverted) {
        d.gone[e] = 1;
        atomicAdd(&d.s->erodedCount, 1);
        if (inverted && !failed) atomicAdd(&d.s->invertedCount, 1);
        const MatF &m = d.matsF[d.emat[e]];
        for (int g = 0; g < d.ppe; g++) {
            const int p = e * d.ppe + g;
            const float4 s = reinterpret_cast<const float4 *>(d.sigF)[p];
            const double s0 = s.x, s1 = s.y, s2 = s.z, s3 = s.w;
            const double press = (s0 + s1 + s2) / 3.0;
            const double aa = s0 - press, bb = s1 - press, cc = s2 - press;
            const double density = (aa * aa + bb * bb + cc * cc + 2.0 * s3 * s3) / (4.0 * (double)m.mu)
                                   + press * press / (2.0 * (double)m.bulk);
            energy += density * d.gaussVol[p];
        }
        if (d.hasContact) {
            d.dead[e] = 1;
            d.s->stale = 1;
            d.newDead[atomicAdd(&d.s->newDeadCount, 1)] = e;   // at most E, ever
        }
    }
}

// The block's eroded energy into its partial, in a fixed order (deterministic). A block whose
// terms are all +0 has a sum of +0: one vote instead of the tree.
__device__ __forceinline__ void erode_partial_mixed(const Dev &d, double energy) {
    __shared__ double sh[MB / 32];
    double t = 0.0;
    if (__syncthreads_or(__double_as_longlong(energy) != 0)) {
        for (int o = 16; o > 0; o >>= 1) energy += __shfl_down_sync(0xffffffffu, energy, o);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) sh[warp] = energy;
        __syncthreads();
        for (int w = 0; w < MB / 32; w++) t += sh[w];
    }
    if (threadIdx.x == 0) d.partials[PARTIAL_ERODE * d.maxBlocks + blockIdx.x] = t;
}

// The erosion pass on its own (the full-integration mixed form).
__global__ void __launch_bounds__(MB) k_erode_mixed(Dev d) {
    if (!d.s->active) return;
    double energy = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d.E; e += gridDim.x * blockDim.x)
        erode_element_mixed(d, e, energy);
    erode_partial_mixed(d, energy);
}

__device__ __forceinline__ void min_edge_commit_f(Dev &d, float minEdge) {
    for (int o = 16; o > 0; o >>= 1) minEdge = fminf(minEdge, __shfl_down_sync(0xffffffffu, minEdge, o));
    if ((threadIdx.x & 31) == 0) atomicMin(&d.s->minEdgeBits, dbits_m((double)minEdge));
}

// reducedIntegration (ExplicitSolver.java:1373-1504) in FP32. With `erode` each element first
// decides its own erosion: that reads only its own points and nodes, which no other element's
// update writes, so it is the same as an erosion pass over all elements before any update.
// The pass waits on its node gathers: eight blocks per SM (64 registers, a few spilled) hide
// more of that than six (80 registers), 76 against 82 us on a 1M-quad scene.
__global__ void __launch_bounds__(MB, 8) k_element_reduced_mixed(Dev d, int zeroStrain, int erode) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    float minEdge = 3.4028235e38f;
    double energy = 0.0;
    if (e < d.E) {
        if (erode) erode_element_mixed(d, e, energy);
        element_reduced_f32(d, e, zeroStrain ? 0.0f : (float)d.s->dt, (float)d.hourglass, d.pMid,
                            d.vdt, 0, minEdge);
    }
    min_edge_commit_f(d, minEdge);
    if (erode) erode_partial_mixed(d, energy);
}

// fullIntegration (ExplicitSolver.java:1219-1339) in FP32.
__global__ void __launch_bounds__(MB) k_element_full_mixed(Dev d, int zeroStrain) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    float minEdge = 3.4028235e38f;
    if (e < d.E) {
        float4 *ef = reinterpret_cast<float4 *>(d.contribF + 8 * (size_t)e);
        if (d.gone != nullptr && d.gone[e]) {
            ef[0] = make_float4(0.f, 0.f, 0.f, 0.f);
            ef[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const float strainDt = zeroStrain ? 0.0f : (float)d.s->dt;
            const MatF &fl = d.matsF[d.emat[e]];
            const int4 c = d.conn[e];
            const float4 p0 = d.pMid[c.x], p1 = d.pMid[c.y], p2 = d.pMid[c.z], p3 = d.pMid[c.w];
            const float2 w0 = d.vdt[c.x], w1 = d.vdt[c.y], w2 = d.vdt[c.z], w3 = d.vdt[c.w];
            const float r0 = 0.0f, z0 = 0.0f;
            const float r1 = diff_hl(p1, p0, 0), r2 = diff_hl(p2, p0, 0), r3 = diff_hl(p3, p0, 0);
            const float z1 = diff_hl(p1, p0, 1), z2 = diff_hl(p2, p0, 1), z3 = diff_hl(p3, p0, 1);
            const float R0 = p0.x, R1 = p1.x, R2 = p2.x, R3 = p3.x;   // absolute, for 2 pi r
            const float a0 = w0.x, a1 = w1.x, a2 = w2.x, a3 = w3.x;
            const float c0 = w0.y, c1 = w1.y, c2 = w2.y, c3 = w3.y;
            if (d.finite) minEdge = shortestEdge(minEdge, r0, r1, r2, r3, z0, z1, z2, z3);
            float g0r = 0, g1r = 0, g2r = 0, g3r = 0, g0z = 0, g1z = 0, g2z = 0, g3z = 0;
            const float G = 0.57735026918962576f;
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const float xi = (g == 0 || g == 3) ? -G : G;
                const float eta = (g < 2) ? -G : G;
                const float xm = 1.0f - xi, xp = 1.0f + xi, em = 1.0f - eta, ep = 1.0f + eta;
                const float N0 = 0.25f * xm * em, N1 = 0.25f * xp * em;
                const float N2 = 0.25f * xp * ep, N3 = 0.25f * xm * ep;
                const float dN0x = -0.25f * em, dN1x = 0.25f * em, dN2x = 0.25f * ep, dN3x = -0.25f * ep;
                const float dN0e = -0.25f * xm, dN1e = -0.25f * xp, dN2e = 0.25f * xp, dN3e = 0.25f * xm;
                const float J00 = dN0x * r0 + dN1x * r1 + dN2x * r2 + dN3x * r3;
                const float J01 = dN0x * z0 + dN1x * z1 + dN2x * z2 + dN3x * z3;
                const float J10 = dN0e * r0 + dN1e * r1 + dN2e * r2 + dN3e * r3;
                const float J11 = dN0e * z0 + dN1e * z1 + dN2e * z2 + dN3e * z3;
                const float det = J00 * J11 - J01 * J10;
                const float inv = 1.0f / det;
                const float d0r = (J11 * dN0x - J01 * dN0e) * inv;
                const float d1r = (J11 * dN1x - J01 * dN1e) * inv;
                const float d2r = (J11 * dN2x - J01 * dN2e) * inv;
                const float d3r = (J11 * dN3x - J01 * dN3e) * inv;
                const float d0z = (-J10 * dN0x + J00 * dN0e) * inv;
                const float d1z = (-J10 * dN1x + J00 * dN1e) * inv;
                const float d2z = (-J10 * dN2x + J00 * dN2e) * inv;
                const float d3z = (-J10 * dN3x + J00 * dN3e) * inv;
                const float dEpsR = d0r * a0 + d1r * a1 + d2r * a2 + d3r * a3;
                const float dEpsZ = d0z * c0 + d1z * c1 + d2z * c2 + d3z * c3;
                const float dRdZ = d0z * a0 + d1z * a1 + d2z * a2 + d3z * a3;
                const float dZdR = d0r * c0 + d1r * c1 + d2r * c2 + d3r * c3;
                float rg = 0.0f, dEpsT = 0.0f;
                if (d.axi) {
                    rg = N0 * R0 + N1 * R1 + N2 * R2 + N3 * R3;
                    dEpsT = (N0 * a0 + N1 * a1 + N2 * a2 + N3 * a3) / rg;
                }
                const int p = e * 4 + g;
                float sg[4];
                point_update_mixed(d, e, p, fl, dEpsR, dEpsZ, dEpsT, dRdZ + dZdR,
                                   0.5f * (dZdR - dRdZ), strainDt, sg);
                const float sR = sg[0], sZ = sg[1], sT = sg[2], sRZ = sg[3];
                const float dV = d.axi ? 2.0f * 3.14159265358979f * rg * det
                                       : (float)d.thickness * det;
                if (d.axi) {
                    const float hh = sT / rg * dV;
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
            ef[0] = make_float4(g0r, g1r, g2r, g3r);
            ef[1] = make_float4(g0z, g1z, g2z, g3z);
        }
    }
    min_edge_commit_f(d, minEdge);
}

// Pressure edges: the load in FP64 (few edges), stored as float contributions.
__global__ void k_pressure_mixed(Dev d) {
    if (!d.s->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.K) return;
    pressure_edge_f32(d, e, d.s->time, d.targetPressure, d.rampDuration);
}

// The per-node gather (:1147-1165) of float contributions into FP64 forces, same order.
__global__ void __launch_bounds__(MB) k_gather_mixed(Dev d) {
    if (!d.s->active) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    d.F[n] = gather_node_f32(d, n);
    if (d.hasContact) d.contactState[n] = 0;
}

// State conversion between the FP64 and FP32 element arrays. what: 1 the element state,
// 2 the damage parameters and state.
__global__ void k_convert_state(Dev d, int toFloat, size_t points, int what) {
    const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (p < points && (what & 1)) {
        for (int k = 0; k < 4; k++) {
            if (toFloat) {
                d.sigF[4 * p + k] = (float)d.sig[4 * p + k];
                d.backF[4 * p + k] = (float)d.back[4 * p + k];
            } else {
                d.sig[4 * p + k] = d.sigF[4 * p + k];
                d.back[4 * p + k] = d.backF[4 * p + k];
            }
        }
        if (toFloat) {
            d.epsPF[p] = (float)d.epsP[p];
            d.wPF[p] = (float)d.wP[p];
        } else {
            d.epsP[p] = d.epsPF[p];
            d.wP[p] = d.wPF[p];
            if (d.jcYield) {                   // the kept yield radii follow the new state
                const MatDev &f = d.mats[d.emat[p]];
                if (f.jc) d.jcYield[p] = jc_yield(f, d.epsP[p], d.wP[p]);
            }
        }
    }
    if (p < points && (what & 2)) {
        if (d.dStrength && d.dStrF) {
            if (toFloat) {
                d.dStrF[p] = (float)d.dStrength[p];
                d.dSoftF[p] = (float)d.dSoft[p];
                d.dWidthF[p] = (float)d.dWidth[p];
            } else {
                d.dStrength[p] = d.dStrF[p];
                d.dSoft[p] = d.dSoftF[p];
                d.dWidth[p] = d.dWidthF[p];
            }
        }
    }
    if (p < (size_t)d.E && (what & 1)) {
        if (toFloat) {
            d.hgF[p] = make_float2((float)d.hg[p].x, (float)d.hg[p].y);
            d.hgKF[p] = (float)d.hgK[p];
        } else {
            d.hg[p] = make_double2(d.hgF[p].x, d.hgF[p].y);
            d.hgK[p] = d.hgKF[p];
        }
    }
    if (p < (size_t)d.E && (what & 2) && toFloat && d.dFail && d.dFailF) {
        d.dFailF[p] = (float)d.dFail[p];
        d.dGfF[p] = (float)d.dGf[p];
        for (int k = 0; k < 5; k++) d.dGeomF[5 * p + k] = (float)d.dGeom[5 * p + k];
    }
}

int launch_prepare_mixed(Solver &S, int zeroStrain) {
    if (S.d.N <= 0) return 0;
    k_prepare_mixed<<<grid_for(S.d.N, MB), MB, 0, S.stream>>>(S.d, zeroStrain);
    return 1;
}
int launch_erode_mixed(Solver &S) {
    k_erode_mixed<<<element_grid(S), MB, 0, S.stream>>>(S.d);
    return 1;
}
int launch_element_mixed(Solver &S, int zeroStrain, bool erode) {
    if (S.d.E <= 0) return 0;
    if (S.d.full) k_element_full_mixed<<<grid_for(S.d.E, MB), MB, 0, S.stream>>>(S.d, zeroStrain);
    else k_element_reduced_mixed<<<grid_for(S.d.E, MB), MB, 0, S.stream>>>(S.d, zeroStrain, erode ? 1 : 0);
    return 1;
}
int launch_pressure_mixed(Solver &S) {
    k_pressure_mixed<<<grid_for(S.d.K, MB), MB, 0, S.stream>>>(S.d);
    return 1;
}
int launch_gather_mixed(Solver &S) {
    k_gather_mixed<<<grid_for(S.d.N, MB), MB, 0, S.stream>>>(S.d);
    return 1;
}
void launch_convert_state(Solver &S, bool toFloat, int what) {
    const size_t P = (size_t)S.d.E * S.d.ppe;
    const size_t n = P > (size_t)S.d.E ? P : (size_t)S.d.E;
    if (n) k_convert_state<<<grid_for((long long)n, 256), 256, 0, S.stream>>>(S.d, toFloat ? 1 : 0, P, what);
}

}  // namespace nf
