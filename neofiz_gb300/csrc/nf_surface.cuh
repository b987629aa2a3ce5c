// nf_surface.cuh -- the contact surface's incremental rebuild after erosion (Contact.adopt,
// Contact.java:290-332, over QuadMesh.surface, QuadMesh.java:188-226), shared by the contact
// pass (many blocks, separated by a grid barrier) and by one block of the gather's launch (the
// usual few eroded elements a step).
//
// The surface is kept as unordered lists keyed by element edge q = 4 e + corner and node
// number: an element edge is free when it is the only live member of its group of equal edges.
#pragma once

#include "nf_internal.h"

namespace nf {

// Node n's free edges in ascending q, from the corners of its elements (the node slots of the
// force gather): at corner c of element e the edges 4 e + c (leaving it) and 4 e + (c + 3) % 4
// (arriving at it).
// Four slots at a time: their indices, then the eight edges' flags, are loaded before any is
// used, so the loads overlap instead of chaining; the edges are taken in the slots' order.
static __device__ void build_node_segs(const Dev &d, int n) {
    int32_t *out = d.nodeSeg + (size_t)n * d.segCap;
    int count = 0;
    const int k1 = d.nodeSlotStart[n + 1];
    for (int k = d.nodeSlotStart[n]; k < k1; k += 4) {
        int q1[4], q0[4], f1[4], f0[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int v = k + j < k1 ? d.nodeSlot[k + j] : 8 * d.E;
            const bool edge = v < 8 * d.E;           // not a pressure edge's slot
            const int e = v >> 3, c = v & 7;
            q1[j] = edge ? 4 * e + c : -1;
            q0[j] = edge ? 4 * e + ((c + 3) & 3) : -1;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            f1[j] = q1[j] >= 0 ? d.surfFlag[q1[j]] : 0;
            f0[j] = q0[j] >= 0 ? d.surfFlag[q0[j]] : 0;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (f1[j] && count < d.segCap) out[count++] = q1[j];
            if (f0[j] && count < d.segCap) out[count++] = q0[j];
        }
    }
    for (int i = 1; i < count; i++) {
        const int v = out[i];
        int j = i - 1;
        while (j >= 0 && out[j] > v) {
            out[j + 1] = out[j];
            j--;
        }
        out[j + 1] = v;
    }
}

// The list counters a rebuild advances: the scalars themselves in the contact pass, copies in
// shared memory in the one-block rebuild (written back at its end).
struct SurfaceCounters {
    int *edgeListLen, *surfEdges, *nTouched, *nodeListLen, *surfNodes;
};

// Item t of the re-flagging: edge t & 3 of the element newDead[t >> 2]. Its group's members are
// re-flagged (each once a rebuild: the epoch stamp); an edge that became free is appended to the
// edge list and one that stopped being free is struck out; each node keeps its count of free
// edges, and the nodes touched are noted.
__device__ __forceinline__ void surface_reflag(const Dev &d, int t, int epoch,
                                               const SurfaceCounters &k) {
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
        if (now) {
            const int pos = atomicAdd(k.edgeListLen, 1);
            d.edgeList[pos] = q;
            d.edgePos[q] = pos;
        } else {
            d.edgeList[d.edgePos[q]] = -1;
            d.edgePos[q] = -1;
        }
        atomicAdd(k.surfEdges, now ? 1 : -1);
        const int ends[2] = {d.segA[q], d.segB[q]};
        for (int j = 0; j < 2; j++) {
            atomicAdd(&d.nodeFree[ends[j]], now ? 1 : -1);
            if (atomicExch(&d.nodeStamp[ends[j]], epoch) != epoch)
                d.touched[atomicAdd(k.nTouched, 1)] = ends[j];
        }
    }
}

// Item i of the touched nodes: join or leave the surface, and list the node's free edges again.
__device__ __forceinline__ void surface_touched(const Dev &d, int i, const SurfaceCounters &k) {
    const int n = d.touched[i];
    const bool was = d.nodePos[n] >= 0, is = d.nodeFree[n] > 0;
    if (is && !was) {
        const int pos = atomicAdd(k.nodeListLen, 1);
        d.nodeList[pos] = n;
        d.nodePos[n] = pos;
        atomicAdd(k.surfNodes, 1);
    } else if (was && !is) {
        d.nodeList[d.nodePos[n]] = -1;
        d.nodePos[n] = -1;
        atomicAdd(k.surfNodes, -1);
        d.pairNodes[n] = make_int4(-1, -1, -1, 0);
        d.incCount[n] = 0;
    }
    if (is) build_node_segs(d, n);
}

// The incremental rebuild in one block: the re-flagging, a block barrier, the touched nodes.
// Leaves the rebuild's marks as the contact pass's own rebuild does, and rebuiltNow set, so
// the pass's geometry phase still makes every surface node forget its last master.
constexpr int SURFACE_BLOCK_DEAD = 256;   // most eroded elements one block rebuilds for
// The block is the only writer of the lists while it runs, so their counters live in shared
// memory (atomics there cost tens of cycles, a global one returning its value hundreds).
static __device__ void surface_rebuild_block(const Dev &d) {
    DevScalars *s = d.s;
    __shared__ int c[5];
    if (threadIdx.x == 0) {
        c[0] = s->edgeListLen;
        c[1] = s->surfEdges;
        c[2] = s->nTouched;
        c[3] = s->nodeListLen;
        c[4] = s->surfNodes;
    }
    __syncthreads();
    const SurfaceCounters k{&c[0], &c[1], &c[2], &c[3], &c[4]};
    const int epoch = s->rebuildEpoch + 1;
    const int nDead = s->newDeadCount;
    for (int t = threadIdx.x; t < 4 * nDead; t += blockDim.x) surface_reflag(d, t, epoch, k);
    __syncthreads();
    const int nTouched = c[2];
    for (int i = threadIdx.x; i < nTouched; i += blockDim.x) surface_touched(d, i, k);
    __syncthreads();
    if (threadIdx.x == 0) {
        s->edgeListLen = c[0];
        s->surfEdges = c[1];
        s->nodeListLen = c[3];
        s->surfNodes = c[4];
        s->stale = 0;
        s->newDeadCount = 0;
        s->rebuildEpoch = epoch;
        s->nTouched = 0;
        s->rebuiltNow = 1;
    }
}

}  // namespace nf
