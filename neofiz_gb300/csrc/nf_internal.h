// nf_internal.h -- device-side layout of one solver handle and the launchers that advance it.
//
// Layout in HBM (structure of arrays, everything resident across steps):
//   nodes     X0 (r,z), U (ur,uz), V (vr,vz), F (fr,fz) as double2; mass double; flags uint8
//             (bit0 fixed radial, bit1 fixed axial, bit2 on wall)
//   elements  conn int4; material index int32; hourglass force double2 (hgR,hgZ); hourglass
//             stiffness double; eroded uint8
//   points    stress and back stress double[4] per point ({rr, zz, tt, rz}); plastic strain,
//             plastic work double per point; damage strength/softening/width per point;
//             failure strain, fracture energy, reference geometry[5] per element
//   sources   contribution double[8] per element and per pressure edge (four radial, then
//             four axial), gathered per node through the CSR nodeSlotStart/nodeSlot in the
//             reference's serial order (ExplicitSolver.java:139-170, :347-366)
//   scalars   one DevScalars record: dt, time, step count and every running total, so a step
//             never needs the host.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include <cstring>
#include <cmath>

#include "../../include/neofiz.h"
#include "nf_device.cuh"

namespace nf {

// Status-word bits (nf_status_word).
enum : uint32_t {
    STATUS_NONFINITE = NF_STATUS_NONFINITE,          // a nodal velocity or displacement
                                                     // stopped being finite
    STATUS_GRID_HASHED = 2u,     // informational: the contact grid outgrew direct indexing
    STATUS_BUCKET_OVERFLOW = NF_STATUS_BUCKET_OVERFLOW,   // a contact bucket exceeded its bound
    STATUS_TIMEOUT = NF_STATUS_TIMEOUT,              // a grid barrier of the contact pass
                                                     // waited past its limit
};

struct DevScalars {
    double dt, dtPrevious, time;
    double decay, gain, dtAvg;
    unsigned long long minEdgeBits;          // Double bits of the running min edge^2
    long long steps;
    long long stepsTaken;                    // steps taken by the current nf_step/nf_run_until
    long long maxSteps;                      // bound of the current call
    double tEnd;                             // time bound of the current call
    double minEdgeSquared;                   // from the last assembly
    int active;                              // the run predicate: time < tEnd && taken < max
    int pad0;
    // rigid wall (RigidWall.java:103-107)
    double wImpulse, wEnergyLoss, wFriction;
    int wContact, wStuck;                    // the last step's counts
    int wContactAcc, wStuckAcc;              // this step's counts as the nodal update adds them
    // erosion (ExplicitSolver.java:228-234)
    int erodedCount, invertedCount;
    double erodedEnergy;
    // contact (Contact.java:236-250)
    int stale, surfEdges, surfNodes, pairs, escaped, rebuild;   // surfEdges/surfNodes: how
                                             // many free edges and surface nodes there are
    int edgeListLen, nodeListLen;            // lengths of the lists, removed entries included
    double cEnergy, cDissipation;
    unsigned long long maxPenBits;
    unsigned long long bbox[4];              // order-preserving bits of rlo, zlo, -rhi, -zhi
    unsigned long long longestBits;
    double cellSize, gridR0, gridZ0;
    int cols, rows;
    long long cells;
    int hashed, pad2;
    int slotScanN, bucketScanN;              // live lengths of the per-step scans
    uint32_t status;
    uint32_t barCount, barGen, barAbort;     // grid barrier of the cooperative contact pass
    int incOverflow;                         // a node's incident terms outgrew its fixed list
    int fastOverflow;                        // a cell of the direct-indexed grid overflowed
    int rebuiltNow;                          // the gather's launch rebuilt the surface this step
    // the free-surface rebuild (Contact.adopt): a full rebuild at set-up, an incremental one
    // after erosion (elements eroded since the last rebuild, changes this rebuild)
    int fullRebuild, newDeadCount, rebuildEpoch, nTouched;
};

// The element pass's Johnson-Cook work list (FP64 reduced integration). Points whose return
// map evaluated the Johnson-Cook power laws in one step are listed for the next, ordered by
// cost class (solve iterations) from the most expensive down; the next element pass runs the
// listed elements first, packed into warps of equal cost, then every other element. A warp
// issues at most one FP64 instruction per 64 cycles and the SM's pipe takes one per 19, so a
// long solve is a serial chain whose time grows with the warps sharing its SM: the pass runs
// with two blocks per SM (eight warps) and the longest solves start first. A point that stayed
// elastic close to its yield surface (COST_NEAR_YIELD) is listed too, ahead of every solve
// class: yielding again after unloading, or for the first time, takes the longest solves, and
// such a point in a warp of elastic points makes the whole warp run its solve. The elements'
// results do not depend on the order they are computed in.
constexpr int HOT_CLASSES = COST_NEAR_YIELD + 1;   // 0 none, 1 flow-stress powers,
                                                   // 1 + iterations, near yield
struct HotList {
    int count;                               // listed elements in this step's order
    int nextCount;                           // entries appended by this step's pass
    int epoch;                               // stamp of this step's listed elements
    int pad;
    int classCount[HOT_CLASSES];             // the appended (and kept) entries per cost class
    int fill[HOT_CLASSES];                   // entries placed so far per class (hot_build)
    int done;                                // blocks of hot_build that have finished
};

struct Dev {
    // sizes and switches
    int N, E, K, ppe;
    int axi, finite, full, hasWall, hasDamage, hasErosion, hasContact;
    double thickness, cfl, fastestWave, massScale, damping, hourglass;
    double gravR, gravZ, targetPressure, rampDuration, erosionDamage;
    double wallPlane, wallFriction;
    double cFriction, cScale, cDamping, dt0;
    double cSqrtScale;                       // sqrt(cScale), rounded once
    int nmat;
    int sms;                                 // multiprocessors on the device
    // nodes
    double2 *X0, *U, *V, *F;
    double *mass, *invMass;
    uint8_t *flags, *wallState, *contactState;
    // elements / points
    int4 *conn;
    int32_t *emat;
    MatDev *mats;
    double *sig, *back, *epsP, *wP;
    // [E] jc_yield of each Johnson-Cook point's plastic strain and work (one-point FP64 pass
    // with a Johnson-Cook material; null otherwise), kept current with them
    double2 *jcYield;
    double2 *hg;
    double *hgK;
    uint8_t *gone, *dead;
    double *dFail, *dGf, *dGeom, *dStrength, *dSoft, *dWidth;
    // sources
    double *contribution;
    int32_t *nodeSlotStart, *nodeSlot;
    int2 *pedges;
    // partial sums (deterministic reductions)
    double *partials;                        // [PARTIAL_SLOTS * maxBlocks]
    int maxBlocks;
    // surface / contact. Segments are identified by their element edge q = 4 e + corner and
    // surface nodes by their node number: ascending q is the reference's segment order
    // (QuadMesh.surface lists free edges in element order) and ascending node number its
    // surface-node order, so every order-dependent result keys on these.
    int32_t *edgeGroup, *groupStart, *groupMember;   // element-edge -> group of equal edges
    int32_t *surfFlag;                       // [4E] 1 while the element edge is free
    int32_t *segA, *segB;                    // [4E] end nodes of each element edge
    int32_t *edgeList, *edgePos;             // [4E] the free edges in any order (-1: no longer
                                             // free), and each edge's place in it
    int32_t *nodeList, *nodePos;             // [N] the surface nodes in any order (-1: left the
                                             // surface), and each node's place (-1: none)
    int32_t *nodeFree;                       // [N] free edges incident to each node
    int2 *nodeCell;                          // [N] a surface node's grid cell (column, row)
    int32_t *nodeSeg;                        // [N x segCap] each surface node's free edges,
    int segCap;                              // ascending (2 x the largest node valence)
    int32_t *edgeStamp, *nodeStamp;          // [4E], [N] rebuild epoch of the last visit
    int32_t *touched;                        // [N] nodes whose free edges changed
    int32_t *newDead;                        // [E] elements eroded since the last rebuild
    double *cr, *cz;                         // [N]
    double *snr, *snz, *slen;                // [4E] by element edge
    double *pnr, *pnz;                       // [N]
    int32_t *lastMaster, *master;            // [N] by node: the master element edge, or -1
    uint8_t *dropped;                        // [N]
    int32_t *bucketCount, *bucketStart, *bucketCursor;   // [bucketCap + 1]
    int32_t *bucketEntry;                    // [8E] entries (2 q + end)
    // [8E] by position, for the search's FP32 screen: the segment's first node relative to the
    // grid origin and its normal (float4), and its length (float); for the exact test: the
    // segment's ends (int2), first node and normal (double2) and length
    float4 *bucketF;
    float *bucketFL;
    int2 *bucketAB;
    double2 *bucketA, *bucketN;
    double *bucketL;
    long long *bucketCell;                   // [8E] cell of each filed entry, by position
    long long *entryCell;                    // [8E] cell of each entry, by entry
    // the direct-indexed grid: cell c's entries in slots [c fastCap, c fastCap + fastCount[c])
    // when the grid has at most fastCells cells and none holds more than fastCap entries
    int32_t *fastCount;                      // [fastCells]
    int32_t *fastEntry;                      // [fastCells x fastCap]
    float4 *fastF;                           // [fastCells x fastCap] as bucketF
    float *fastFL;                           // [fastCells x fastCap] as bucketFL
    int2 *fastAB;                            // [fastCells x fastCap] as bucketAB
    double2 *fastA, *fastN;                  // [fastCells x fastCap] as bucketA, bucketN
    double *fastL;                           // [fastCells x fastCap] as bucketL
    int fastCells, fastCap;                  // cells indexed directly, slots per cell
    int fastLimit;                           // slots a step may use, <= fastCap (nf_set_grid_slots)
    int bucketCap;
    // pair records, per node
    int4 *pairNodes;                         // [N] (n, a, b, valid)
    double *pairVal;                         // [12 per node]: role-major (n,a,b) x (normal r,z, tangent r,z)
    double *pairEnergy, *pairDiss;           // [N]
    int32_t *incCount, *incStart, *incCursor, *incEntry;   // [N + 1] per node, entries (n<<2 | role)
    int32_t *incSlots;                       // [NF_INC_CAP per node] fixed lists
    // mixed precision: FP32 element state, float contributions, per-node float positions
    int mixed;
    MatF *matsF;
    float *sigF, *backF, *epsPF, *wPF, *hgKF, *contribF;
    float2 *hgF;
    float *dStrF, *dSoftF, *dWidthF, *dFailF, *dGfF, *dGeomF;
    float4 *pMid, *pCur;
    // compensated form (batches): displacement and reference position as float pairs
    // (r hi, r lo, z hi, z lo), velocity, gathered force and (mass, 1/mass) in FP32
    float4 *uC, *x0C;
    float2 *vC, *fC, *mC;
    int comp;
    float2 *vdt;
    double *gaussVol;                        // reference volume of each point
    // scan workspace; the cooperative contact pass's grid and its per-block scan sums
    int32_t *scanTmp;
    int scanTmpSize;
    // Johnson-Cook work list (null when no material is Johnson-Cook)
    HotList *hot;
    int32_t *hotList, *hotStamp;             // [hotCap] element order, [E] listing epoch
    int2 *hotNext;                           // [hotCap] (element, cost class) appended
    int hotCap;
    int hotSmem;                             // the listed pass's occupancy-limiting request
    int coopBlocks;
    int32_t *coopSums;
    // limits of the contact pass's grid-barrier wait (0: the defaults, 2^27 polls or one
    // second); nf_set_wait_limit lowers them so that tests can make a wait run out
    long long waitSpins, waitNs;
    DevScalars *s;
};

constexpr int NF_INC_CAP = 8;
constexpr int NF_GRID_SLOTS = 64;            // slots per cell of the direct-indexed contact grid

// Contact.begin, Contact.java:424-436: the per-step totals and extrema the contact pass
// accumulates into; run by the step's first kernel, before the pass.
__device__ inline void contact_step_reset(DevScalars *s) {
    s->pairs = 0;
    s->maxPenBits = 0ULL;
    s->bbox[0] = ~0ULL;   // min r
    s->bbox[1] = ~0ULL;   // min z
    s->bbox[2] = 0ULL;    // max r
    s->bbox[3] = 0ULL;    // max z
    s->longestBits = 0ULL;
    s->incOverflow = 0;
    s->fastOverflow = 0;
    s->barCount = 0;      // a fresh grid barrier
    s->barAbort = 0;
}

enum { PARTIAL_WALL = 0, PARTIAL_ERODE = 3, PARTIAL_CONTACT = 4, PARTIAL_SLOTS = 6 };

struct Solver {
    Dev d{};
    cudaStream_t stream = nullptr;
    int device = 0;
    long long hostSteps = 0;     // mirror of the device step count (steps are deterministic)
    bool hasWall = false;
    std::string err;
    // host copies needed by reads and set-up
    int N = 0, E = 0, K = 0, ppe = 1;
    int formulation = 0, integration = 0, kinematics = 0;
    double *hostScratch = nullptr;
    size_t hostScratchBytes = 0;
    std::vector<nf_material> materials;
    std::vector<int32_t> emat;
    std::vector<double> hostR, hostZ;
    std::vector<int32_t> hostConn;
    double massScale = 1.0;
    double hourglass = 0.05;
    bool contactSet = false, damageSet = false, erosionSet = false;
    int gridSlots = NF_GRID_SLOTS;   // nf_set_grid_slots, applied when the contact data exists
    // launch bookkeeping
    cudaStream_t ownStream = nullptr;
    long long launches = 0;
    bool unbounded = false;      // nf_step mode: no time or step bound on the device
    // graph replay of whole steps: one- and sixteen-step graphs captured for a given Dev
    cudaGraphExec_t graph1 = nullptr, graph16 = nullptr;
    int graphKernels1 = 0, graphKernels16 = 0;
    Dev graphDev{};
    bool graphValid = false;
    bool noGraphs = false;       // capture failed once: steps are enqueued directly
    // a device-side wait that ran out leaves the state invalid: later run calls refuse
    nf_status failed = NF_OK;
    void *arena = nullptr;       // nf_create's set-up arrays, one allocation
    size_t arenaBytes = 0;
    // per-group event profiling
    bool profiling = false;
    struct Rec { int group; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    double profMs[NF_GROUP_COUNT] = {0};
    long long profSteps = 0;
    void mark(int group, bool begin);
};

// ------------------------------------------------------------------------------------ batches
// Many independent scenes of one formulation in one set of concatenated arrays, described by
// one Dev (conn and node slots hold global indices; emat[e] is the element's instance, whose
// material is mats[instance]). Each instance keeps its own step, time and totals.
struct BatchInst {
    int n0, n1, e0, e1;                      // its nodes and elements
    int k0, k1;                              // its pressure edges
    int hasWall, pad;
    double cfl, wave, massScale, damping, hourglass;
    double wallPlane, wallFriction, tEnd;
    double pressure, ramp;                   // setPressureRamp
};

struct BatchScalars {
    double dt, dtPrevious, time, minEdgeSquared;
    double wImpulse, wEnergyLoss, wFriction;
    long long steps, stepLimit;
    int wContact, wStuck;
    uint32_t status;
    int done;                                // time >= tEnd or the step limit reached
};

// BurstCase.run's measurement (BurstCase.java:446-490) on the device: every `every` steps each
// instance samples its wall capacity, hoop strain and applied pressure, keeps the running
// peak, and stops once the ramp has reached its ceiling and the capacity has fallen `margin`
// below the peak. every == 0: off.
struct BurstState {
    double peakCapacity, peakStrain, peakApplied;
    double capacity, strain, applied;        // the last sample
    int samples, traversed;
};
struct BurstDev {
    int every, traceCap;
    double margin;
    const double *meanRadius;                // [count] for the hoop strain
    BurstState *state;                       // [count]
    double *trace;                           // [count * traceCap * 4]: t, strain, capacity, applied
    double *scratch;                         // [E]: each element's hoop stress x area
};

struct BatchDev {
    const BatchInst *inst;
    BatchScalars *sc;
    const int32_t *order;                    // instances, most expensive first
    int32_t *queue;                          // next position in order (per launch)
    int32_t *remaining;                      // instances not done
    unsigned long long *measure;             // [3 per instance] order-preserving extrema
    int count;
    int maxNodes;                            // the largest instance's node count
    BurstDev burst;
};

// The adjoint's device buffers (k_adjoint.cu): per instance a run of checkpoint blocks, one
// final-state block, a tape of `every` blocks and the adjoint arrays; byte offsets by instance.
struct AdjDev {
    char *ckpt, *fin, *tape, *bar, *peak, *seed;
    const long long *ckptOff, *finOff, *tapeOff, *barOff, *peakOff, *seedOff;
    const long long *ckptCap;                // checkpoints available per instance
    const long long *stateBytes;             // bytes of one state block per instance
    long long *steps;                        // the forward's step count per instance
    long long *peakStep;                     // the sampled capacity peak: its step and value
    double *peakValue;
    // The backward pass carries `width` objectives (1..NF_ADJ_MAX_WIDTH) through one segment
    // recompute: objective w's adjoint arrays, seed, seed step and gradients sit in plane w
    // (bar + w barPlane, seed + w seedPlane, seedStep[w count + k], grad[(w count + k) P + p]).
    const long long *seedStep;               // the objective's seed enters after this step
    double *grad;
    int *overflow;
    int every, sampleEvery, width;
    long long barPlane, seedPlane;
};
constexpr int NF_ADJ_MAX_WIDTH = 3;
size_t adj_state_bytes(int n, int e);
size_t adj_bar_bytes(int n, int e, int k);
size_t adj_seed_bytes(int n, int e);
cudaError_t adjoint_reserve_stack();
void launch_adjoint_forward(const Dev &d, const BatchDev &b, const AdjDev &a, cudaStream_t st);
void launch_adjoint_backward(const Dev &d, const BatchDev &b, const AdjDev &a, cudaStream_t st);

// A launch configuration of the batched step (chosen by the autotuner).
struct BatchShape {
    int threads;                             // 128 or 256
    int stage;                               // mixed: node geometry in shared memory
    int blocksPerSm;
    int chunk;                               // steps per instance per launch
};

// Launchers (k_batch.cu).
// mode: NF_PRECISION_FP64, NF_PRECISION_MIXED or NF_PRECISION_COMPENSATED
int batch_max_blocks_per_sm(int mode, const BatchShape &shape, int maxNodes);
size_t batch_shared_bytes(int mode, const BatchShape &shape, int maxNodes);
void launch_batch_initial(const Dev &d, const BatchDev &b, bool mixed, cudaStream_t st);
void launch_batch_arm(const BatchDev &b, long long maxSteps, cudaStream_t st);
void launch_batch_comp(const Dev &d, bool toFloat, cudaStream_t st);
const void *comp_steps_kernel(const BatchShape &shape);      // k_batch_comp.cu
cudaError_t launch_batch_steps(const Dev &d, const BatchDev &b, int mode,
                               const BatchShape &shape, int sms, cudaStream_t st);
void launch_batch_measure(const Dev &d, const BatchDev &b, cudaStream_t st);

// Set-up helpers of api.cu shared with api_batch.cu.
const char *validate_material(const nf_material &m);
MatDev material_constants(const nf_material &m, int formulation);
double material_wave(const nf_material &m);
MatF material_constants_f32(const MatDev &m);
double element_signed_area(const double *r, const double *z, const int32_t *conn, int e);
void setup_lumped_mass(const double *r, const double *z, const int32_t *conn, int E,
                       const nf_material *materials, const int32_t *emat, bool axi,
                       double thickness, double *mass);
void setup_node_slots(const int32_t *conn, int N, int E, const int32_t *pedges, int K,
                      int32_t *slotStart, int32_t *slots);
double setup_min_edge(const double *r, const double *z, const int32_t *conn, int E);
void set_thread_error(const char *message);

// Launchers (k_step.cu). Each returns the number of kernels it enqueued.
int launch_initial_assembly(Solver &S);
int launch_step(Solver &S, bool predicated);
int launch_advance(Solver &S);
void launch_audits(Solver &S, nf_audit *out);
// The audits in two halves: per-block partial sums into a device buffer of
// audit_partial_doubles(d) doubles (enqueued, no wait), and their fixed-order host reduction.
size_t audit_partial_doubles(const Dev &d);
void launch_audit_partials(Solver &S, double *buf);
void reduce_audit_partials(const Solver &S, const double *h, nf_audit *out);
// api.cu helpers for the device film (k_film.cu).
void solver_state_to_double(Solver &S);
nf_status solver_fail(Solver &S, nf_status st, const char *message);
nf_status solver_sync(Solver &S);
void launch_measure(Solver &S, nf_measure *out);
// jc_yield of every Johnson-Cook point's current state into d.jcYield (enqueued on st).
void launch_jc_yield(const Dev &d, cudaStream_t st);
void launch_material_points(const MatDev &m, int count, double *sig, double *back, double *epsP,
                            double *work, const double *strain, double strainDt,
                            const double *fail, const double *gf, const double *youngs,
                            const double *geom, double *strength, double *soft, double *width,
                            double *dgamma, cudaStream_t stream);
// Launchers (k_mixed.cu)
int launch_prepare_mixed(Solver &S, int zeroStrain);
int launch_erode_mixed(Solver &S);
int launch_element_mixed(Solver &S, int zeroStrain, bool erode);
int launch_pressure_mixed(Solver &S);
int launch_gather_mixed(Solver &S);
void launch_convert_state(Solver &S, bool toFloat, int what);
int launch_point_volumes(Solver &S, double *out);
// Launchers (k_contact.cu)
int launch_contact(Solver &S, bool predicated);
// Launchers (k_scan.cu)
int scan_exclusive(const int32_t *in, int32_t *out, int n, int32_t *totalOut, int32_t *tmp,
                   cudaStream_t stream, const int *pred, const int *nDev);
int contact_coop_blocks(int sms);
int listed_pass_smem(int device);
size_t scan_tmp_ints(int n);

int grid_for(long long n, int block);
// Fixed grids of the node and element kernels that reduce per block, striding over the items.
// The nodal update takes one node per thread up to sixteen blocks per SM (every block resident
// at once, no second pass over the nodes); the element kernels stop at eight.
inline int nodal_grid(const Solver &S) {
    const int g = grid_for(S.d.N, 128), cap = 16 * S.d.sms;
    return g < cap ? g : cap;
}
inline int element_grid(const Solver &S) {
    const int g = grid_for(S.d.E, 128), cap = 8 * S.d.sms;
    return g < cap ? g : cap;
}

}  // namespace nf
