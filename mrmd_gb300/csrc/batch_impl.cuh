// Internals of the batched replica engine shared by its translation units
// (batch.cu: stepping, rebuilds, graphs, autotuner; batch_adjoint.cu: the
// adjoint of the step for differentiation).
#pragma once

#include <cmath>
#include <vector>

#include "adress_impl.cuh"
#include "common.cuh"
#include "integrate_impl.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"

namespace mrmd_batch_impl
{
using namespace mrmd_impl;

constexpr int TB = 256;
constexpr double COMP_SCALE = 4294967296.0;  // 2^32: fixed point of the compensation histogram

// list entries with this bit refer to a ghost whose pair instance in the
// reference's half list is (ghost's source, image of the row molecule)
constexpr int32_t REVERSED = (int32_t)0x80000000u;

enum : uint32_t
{
    FLAG_GHOST_OVERFLOW = 1u,
    FLAG_LIST_OVERFLOW = 2u,
    FLAG_UNSAFE_INTERVAL = 4u,
    FLAG_FAR_LIST_OVERFLOW = 8u,
    FLAG_CLUSTER_LIST_OVERFLOW = 16u,
};

// list layouts (mrmd_batch_tuning::listLayout)
enum : int32_t
{
    LAYOUT_ROWS = 0,      // one full row per molecule
    LAYOUT_NEAR_FAR = 1,  // near and far rows per molecule (mixed form)
    LAYOUT_CLUSTER = 2,   // 8 x 4 cluster pairs with a pair mask
};
constexpr int CLUSTER_I = 8;  // molecules of an i-cluster (rows of one warp)
constexpr int CLUSTER_J = 4;  // cell-sorted slots of a j-cluster (lanes of one row)

// Per-replica constants.
struct RepDev
{
    double lo[3], mx[3], L[3], minIn[3], maxIn[3];  // box corners, lengths, inner corners
    double gmn[3], grdx[3];  // ghost-inclusive cell grid
    int32_t gn[3];
    int32_t cellBase;
    double splitScale, splitInv;  // mixed form: the split's quantum 2^-q
    long long sko[3];             // the split origin / 2^-q (gmn rounded down to the 2^-q grid)
    int32_t sq;                   // q
    float soff[3];                // gmn - the split origin, [0, 2^-q)
    SlabDev slab;
    int32_t consistent;  // slab weights of every image equal those of its real molecule
    int32_t lbase, n;
    int32_t tfBase, tfBins;
    double tfMin, tfBinSize, tfInvBin, tfBinVolume;
    uint64_t seed;
};

// Device scalars (one struct, snapshotted with the state).
struct Scalars
{
    unsigned long long step;    // global step number of the next step
    unsigned long long tfSamples;
    unsigned long long run;     // LJ_IdealGas run counter
    double maxDisp;             // largest displacement of any molecule since the last rebuild
    double dispStep;            // max |x - x_rebuild|^2 of the current step
    int32_t numGhost;           // total ghosts written at the last rebuild (true count on overflow)
    int32_t maxCount;           // largest list row seen (true count on overflow)
    int32_t maxCountF;          // the same for the far rows of the split layout
    int32_t maxCountC;          // the same for the cluster-pair rows of the cluster layout
    uint32_t overflow;          // ghost / list overflow of the rebuilds since the host cleared it
    uint32_t flags;             // sticky: a molecule moved skin/2 between rebuilds
    uint32_t done;              // tail-kernel block ticket
    // decisions of the current step, set once per step (64-bit modulos are
    // long instruction sequences; no per-thread kernel repeats them)
    int32_t ringSlot;           // step % ring
    int32_t sampleComp;         // run % compensation sampling interval == 0
    int32_t sampleTf;           // TF enabled and step % TF sampling interval == 0
};

// the step decisions of (step, run)
__host__ __device__ inline void set_step_flags(Scalars& s, unsigned long long step, unsigned long long run,
                                               int32_t ring, int64_t compSampling, int32_t tfEnabled,
                                               int64_t tfSampleInterval)
{
    s.ringSlot = (int32_t)(step % (unsigned long long)ring);
    s.sampleComp = compSampling > 0 && (run % (unsigned long long)compSampling) == 0;
    s.sampleTf = tfEnabled && (step % (unsigned long long)tfSampleInterval) == 0;
}

// Everything the kernels read: pointers and run constants.
struct BDev
{
    const RepDev* reps;
    int32_t R, N, gCap;
    int32_t listCap;
    int64_t totalCells;
    double4* pos;  // [N + gCap]
    double4* vel;  // [N]
    double4* force;
    double* mass;
    int32_t* orig;
    int32_t* slotRep;  // [N + gCap]
    int32_t* gSrc;     // [gCap]
    uint8_t* gShift;   // [gCap] 2 bits per axis: 1 = +L, 2 = -L
    uint8_t* imgFlags; // [N] bit 2d: has a +L image on axis d, bit 2d+1: has a -L image
    float4* ref;       // [N] position at the last rebuild, relative to the replica's grid origin
    int2* xImg;        // [N] slots of the ghost images shifted by -L / +L in x only (-1: none)
    int32_t* gCount;   // [N + 1] images per local, then exclusive offsets
    double4* lam;      // [N + gCap] (lambda, modulated lambda, grad lambda x, 0)
    double* lamt;      // [N + gCap] modulated lambda
    float2* lamtf;     // [N + gCap] modulated lambda as a double-float
    float4* hi;        // mixed split coordinates [N + gCap]
    float4* lo;
    // cells
    int32_t* cellOf;
    int32_t* cellStart;  // [totalCells + 1]
    int32_t* cursor;
    int32_t* unordered;
    int32_t* sorted;
    float4* spos;
    // list (32-row tiles); with the split layout the near rows (pairs closer
    // than r_split + skin/2 at the rebuild) and the far rows
    int32_t* counts;
    int32_t* nbrs;
    int32_t* countsF;
    int32_t* nbrsF;
    int32_t listCapF;
    int32_t split;      // 1: near/far rows (mixed form only)
    int32_t farF32;     // mixed form: pairs at and beyond r_split in FP32 (near/far and cluster layouts)
    // cluster layout: i-cluster c holds the locals [clusters[c].x, clusters[c].x
    // + clusters[c].y), at most CLUSTER_I of one replica, aligned to the
    // replica's first molecule; its row lists cluster pairs (first sorted
    // position of the j-cluster, pair mask, reversed mask, 0), the j-cluster
    // being CLUSTER_J consecutive cell-sorted slots aligned to the replica's
    // first cell; mask bit 4a + b: row a with slot b
    int2* clusters;
    int32_t numClusters;
    int32_t listCapC;
    int32_t* countsC;
    int4* clist;
    float rsplitSq;     // r_split^2: FP32 pair arithmetic at and beyond it
    float nearSqF;      // (r_split + skin/2)^2: near rows at the rebuild
    // shadow for the cell sort of locals
    double4* sPos;
    double4* sVel;
    double* sMass;
    int32_t* sOrig;
    // thermodynamic force and compensation energy
    double* tfForce;                   // [sum bins]
    unsigned long long* tfDensity;     // [sum bins] counts
    double* tfWork;                    // [3 * sum bins]: density, smoothed, gradient
    const double* tfFF;                // modulation / target density
    int64_t totalBins;
    long long* compEnergy;             // [R][200] fixed point
    unsigned long long* compCounter;   // [R][200]
    double* compMean;                  // [R][200]
    double* energyRing;                // [ring][R]
    int32_t ring;
    Scalars* sc;
    // physics
    LJDev lj;
    double rcSqr;
    RcSq rc2;
    double dt, zeta, temperature;
    double dtHalfOverMass;  // dt/2 / m (molecules have unit mass)
    double ouDamping, ouSigma;  // Ornstein-Uhlenbeck coefficients of the unit mass (UpdateSteps.hpp:56-79)
    double rlist, halfSkin;
    double cgMargin;  // distance beyond the hybrid region that counts as staying coarse grained
    int64_t K, tfSampleInterval, tfUpdateInterval, compSampling, compUpdate;  // compSampling 0: frozen
    int32_t tfEnabled;
    double tfSigma, tfRange;
    double listRsq;
    float listRsqLo, listRsqHi;
};

__device__ __forceinline__ double coord(const double4& p, int d) { return d == 0 ? p.x : (d == 1 ? p.y : p.z); }

__device__ __forceinline__ void set_coord(double4& p, int d, double v)
{
    if (d == 0)
        p.x = v;
    else if (d == 1)
        p.y = v;
    else
        p.z = v;
}

// velocity-Verlet kick and drift: kick_fma / drift_fma (integrate_impl.cuh),
// the reference's v += dt/2m F and x += dt v, each rounded once

// lambda, modulated lambda and grad lambda (x) of one slot, plus the mixed
// form's split coordinates (UpdateMolecules.hpp:39-69 for a single site).
template <bool MIXED>
__device__ __forceinline__ void slot_derived(const BDev& B, const RepDev& R, int64_t s, const double4& x,
                                             float4* hiOut = nullptr, float4* loOut = nullptr)
{
    double l, m, g;
    slab_eval(R.slab, x.x, l, m, g);
    B.lam[s] = make_double4(l, m, g, 0.0);
    B.lamt[s] = m;
    if (MIXED)
    {
        // the conversions on the integer pipe (the same values as the FP64
        // conversions: this kernel is bound by the FP64 pipe)
        const float h = f64_to_f32_rn(m);
        B.lamtf[s] = make_float2(h, f64_to_f32_rn(__dsub_rn(m, f32_to_f64(h))));
        const float invQ = (float)R.splitInv;
        float4 hv, lv;
        split_bits(x.x, R.sko[0], R.sq, invQ, hv.x, lv.x);
        split_bits(x.y, R.sko[1], R.sq, invQ, hv.y, lv.y);
        split_bits(x.z, R.sko[2], R.sq, invQ, hv.z, lv.z);
        hv.w = 0.0f;
        lv.w = 0.0f;
        B.hi[s] = hv;
        B.lo[s] = lv;
        if (hiOut) *hiOut = hv;
        if (loOut) *loOut = lv;
    }
}

// Everything a step changes (positions, velocities, forces, the order of
// the locals, the TF and compensation tables, the device scalars).
struct Snap
{
    double4 *pos = nullptr, *vel = nullptr, *force = nullptr;
    double* mass = nullptr;
    int32_t* orig = nullptr;
    double* tfForce = nullptr;
    unsigned long long* tfDensity = nullptr;
    long long* compE = nullptr;
    unsigned long long* compC = nullptr;
    double* compM = nullptr;
    Scalars* sc = nullptr;
};

}  // namespace mrmd_batch_impl

struct mrmd_batch
{
    using Snap = mrmd_batch_impl::Snap;
    using BDev = mrmd_batch_impl::BDev;
    using RepDev = mrmd_batch_impl::RepDev;
    using Scalars = mrmd_batch_impl::Scalars;
    mrmd_batch_config cfg{};
    int32_t R = 0, N = 0;
    std::vector<RepDev> reps;
    std::vector<int64_t> offsets;  // [R + 1] molecule offsets
    int64_t totalCells = 0, totalBins = 0;
    double listExtent = 0.0;
    BDev B{};
    RepDev* dReps = nullptr;
    double* dTfFF = nullptr;
    Snap sn;  // state before the running graph (overflow roll-back)
    Scalars* hSc = nullptr;    // pinned
    double* hRing = nullptr;   // pinned [ring][R]
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graphKernels = 0;
    unsigned* dSync = nullptr;  // persistent steps: barrier count, generation, error word
    int64_t steps = 0, rebuilds = 0, graphLaunches = 0, recoveries = 0;
    bool needRebuild = true;  // ghosts and list do not match the locals (new tuning, restored state)
};

namespace mrmd_batch_impl
{
template <typename T>
int grow(mrmd_ctx* ctx, T*& p, int64_t oldCount, int64_t newCount)
{
    T* q = nullptr;
    MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&q), sizeof(T) * (size_t)(newCount > 0 ? newCount : 1)));
    if (p && oldCount > 0)
    {
        const int64_t c = oldCount < newCount ? oldCount : newCount;
        MRMD_CUDA(ctx, cudaMemcpyAsync(q, p, sizeof(T) * (size_t)c, cudaMemcpyDeviceToDevice, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    dfree(p);
    p = q;
    return MRMD_OK;
}

void drop_graph(mrmd_batch* b);
int set_capacity(mrmd_ctx* ctx, mrmd_batch* b, int32_t gCap, int32_t listCap, int32_t listCapF = -1,
                 int32_t listCapC = -1);
// ghosts, cells and the list of the current local positions (no wrap), with
// the overflow check and buffer growth of an eager step
int rebuild_checked(mrmd_ctx* ctx, mrmd_batch* b, bool sort);
// one step, asynchronously; checkRebuild verifies a rebuild on the host
int step(mrmd_ctx* ctx, mrmd_batch* b, int64_t st, bool checkRebuild);
// weights (and split coordinates) of the locals at their current positions
int derive_locals(mrmd_ctx* ctx, mrmd_batch* b);
// ghost positions and weights from their sources (the ghosts of the last rebuild)
int update_ghosts(mrmd_ctx* ctx, mrmd_batch* b);
// ghosts, list and the force kernel at the current positions (the kernel's
// epilogue also applies the post-force kick to the velocities)
int eval_forces(mrmd_ctx* ctx, mrmd_batch* b);
int snap_alloc(mrmd_ctx* ctx, const mrmd_batch* b, Snap& s);
void snap_free(Snap& s);
int snapshot(mrmd_ctx* ctx, mrmd_batch* b, Snap& sn, bool save);
int refresh_step_flags(mrmd_ctx* ctx, mrmd_batch* b);
}  // namespace mrmd_batch_impl
