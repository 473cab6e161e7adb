// Fused LJ NVE stepper: the examples/02_LennardJones_NVE time loop
// (02_LennardJones_NVE.cpp:135-216) as one device-resident object.
//
// Per step:
//   [post-kick of step s-1 + pre-kick/drift of step s + force zeroing]  one kernel
//   rebuild (every K steps): mapIntoDomain, cell sort, ghosts, list
//   or ghost position update
//   (mixed) FP32 split coordinates of local + ghost atoms
//   pair force (FP64: half list + atomics; mixed: full list, no atomics)
//   (FP64) ghost force fold-back
// and the final post-kick when a run ends.  The kick arithmetic is the
// reference's (two kicks with the same force, then the drift), so fusing
// post(s-1) with pre(s) changes no bit.  The K-1 steps between rebuilds
// are captured once per rebuild and replayed as one CUDA graph.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "integrate_impl.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"
#include "lj_tile.cuh"
#include "ghost_impl.cuh"
#include "nlist_impl.cuh"
#include "reduce_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int TB = 256;
// Per-step record: LJ energy, LJ virial, kinetic energy, momentum x, y, z.
constexpr int REC = 6;

// Kinetic energy (analysis/KineticEnergy.hpp:26-39) and the velocity sum of
// getSystemMomentum (analysis/SystemMomentum.cpp:21-48) of one atom.
__device__ __forceinline__ void observe_add(double (&o)[4], const double4& v, double m)
{
    o[0] += 0.5 * (m * (v.x * v.x + v.y * v.y + v.z * v.z));
    o[1] += v.x;
    o[2] += v.y;
    o[3] += v.z;
}

// Tile-kernel records (A, B) of one position.
__device__ __forceinline__ void split_store(const double4& x, const SplitParams& sp, float4* __restrict__ recA,
                                            float2* __restrict__ recB, int64_t i)
{
    float4 a;
    float2 b;
    tile_split(x, sp, a, b);
    recA[i] = a;
    recB[i] = b;
}

// OBS: the velocities after the post-kick are the full-step velocities of
// the previous step; their kinetic energy and momentum go to rec[2..5] of
// that step's record (deterministic grid sum).  SPLIT: the new positions'
// split coordinates are written too (the mixed form between rebuilds).
// dtfm[i] = (dt / 2) / mass[i], divided once per sort (kick_factors), the
// same FP64 quotient VelocityVerlet forms per atom and step.
template <bool OBS, bool SPLIT>
__global__ void k_fused_kick_drift(double4* __restrict__ pos, double4* __restrict__ vel, double4* __restrict__ force,
                                   const double* __restrict__ mass, const double* __restrict__ dtfmOf, int64_t n,
                                   double dt, int postKick, double* partial, unsigned* ticket, double* rec,
                                   SplitParams sp, float4* __restrict__ recA, float2* __restrict__ recB)
{
    double o[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 v = vel[i], x = pos[i];
        const double4 f = force[i];
        const double dtfm = dtfmOf[i];
        if (SPLIT)
        {
            // mixed form: each update rounded once (fused multiply-add), and
            // without a record the previous step's post-kick and this step's
            // pre-kick are one: v + 2 (dt/2m) F.  Kick and drift are the
            // kernel's 6 FP64 operations per atom (GB300's FP64 pipe runs 2
            // per SM and clock); the split below runs on the integer pipe.
            if (OBS)
            {
                if (postKick) kick_fma(v, f, dtfm);
                observe_add(o, v, mass[i]);
                kick_fma(v, f, dtfm);
            }
            else
                kick_fma(v, f, postKick ? twice(dtfm) : dtfm);
            drift_fma(x, v, dt);
        }
        else
        {
            if (postKick) kick(v, f, dtfm);  // VelocityVerlet::postForceIntegrate of the previous step
            if (OBS) observe_add(o, v, mass[i]);
            kick(v, f, dtfm);                // preForceIntegrate
            drift(x, v, dt);
        }
        pos[i] = x;
        vel[i] = v;
        // the mixed form's pair kernel overwrites every local force (no
        // accumulation, ghosts unused): only the FP64 form needs the reset
        if (SPLIT)
            split_store(x, sp, recA, recB, i);
        else
            force[i] = make_double4(0.0, 0.0, 0.0, 0.0);
    }
    if (OBS) grid_sum<4>(o, partial, ticket, rec + 2);
}

__global__ void k_kick_factors(const double* __restrict__ mass, int64_t n, double dtHalf, double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __ddiv_rn(dtHalf, mass[i]);  // action/VelocityVerlet.cpp:35
}

// Ghost position update (the ghost layer's) fused with the ghosts' split
// coordinates.
__global__ void k_ghost_update_split(double4* __restrict__ pos, const int32_t* __restrict__ corr, int64_t nLocal,
                                     int64_t nGhost, double3 L, double3 delta, SplitParams sp,
                                     float4* __restrict__ recA, float2* __restrict__ recB)
{
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nGhost;
         g += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t idx = nLocal + g;
        if (!MRMD_IN_BOUNDS(corr[idx], nLocal)) continue;
        const double4 p = ghost_position(pos[idx], pos[corr[idx]], L, delta);
        pos[idx] = p;
        split_store(p, sp, recA, recB, idx);
    }
}

// The record of the last step of a run: full-step velocities formed on the
// fly (v + dt/2 F/m), nothing stored.
__global__ void k_observe_post(const double4* __restrict__ vel, const double4* __restrict__ force,
                               const double* __restrict__ mass, int64_t n, double dtHalf, int postKick,
                               double* partial, unsigned* ticket, double* rec)
{
    double o[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 v = vel[i];
        const double m = mass[i];
        if (postKick) kick(v, force[i], __ddiv_rn(dtHalf, m));
        observe_add(o, v, m);
    }
    grid_sum<4>(o, partial, ticket, rec + 2);
}

__global__ void k_post_kick(double4* __restrict__ vel, const double4* __restrict__ force,
                            const double* __restrict__ mass, int64_t n, double dtHalf)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 v = vel[i];
        kick(v, force[i], __ddiv_rn(dtHalf, mass[i]));
        vel[i] = v;
    }
}

__global__ void k_gather_i32(const int32_t* __restrict__ src, int32_t* __restrict__ dst,
                             const int32_t* __restrict__ perm, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

__global__ void k_iota(int32_t* p, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

// out[orig[i]] = v[i] (three components) for the first n atoms
__global__ void k_unpermute3(const double4* __restrict__ v, const int32_t* __restrict__ orig, int64_t n,
                             double* __restrict__ out3)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 x = v[i];
        const int64_t o = orig[i];
        out3[3 * o] = x.x;
        out3[3 * o + 1] = x.y;
        out3[3 * o + 2] = x.z;
    }
}

// v[i] = in[orig[i]]
__global__ void k_permute_in3(const double* __restrict__ in3, const int32_t* __restrict__ orig, int64_t n,
                              double4* __restrict__ v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t o = orig[i];
        v[i] = make_double4(in3[3 * o], in3[3 * o + 1], in3[3 * o + 2], 0.0);
    }
}
}  // namespace

struct mrmd_md
{
    mrmd_md_config cfg{};
    mrmd_subdomain sd{};
    mrmd_atoms atoms{};
    mrmd_atoms shadow{};
    mrmd_ghost_layer ghosts{};
    mrmd_nlist list{};           // FP64: half list; mixed: near rows of the split full list
    mrmd_nlist farList{};        // mixed: far rows of the split full list
    double rsplit = 0;           // mixed: pairs beyond it are evaluated in FP32
    mrmd_lj* lj = nullptr;
    CellList sortCells;
    CellGrid grid{};
    int32_t* orig = nullptr;     // original index of each local atom
    int32_t* origTmp = nullptr;
    float4* recA = nullptr;      // mixed: tile-kernel records of local + ghost atoms
    float2* recB = nullptr;
    int64_t splitCap = 0;
    SplitParams sp{};            // mixed: the tile kernel's coordinate split
    TileList tiles;              // mixed: the split list as shared-memory tiles
    TileParams tp{};
    double* dEnergy = nullptr;   // [energyCap][REC] per-step records
    int64_t energyCap = 0;
    double* hEnergy = nullptr;   // pinned
    double* dtfm = nullptr;      // (dt / 2) / mass per local atom, in the current atom order
    double* dPartial = nullptr;  // per-block partial sums of the step observables
    unsigned* dTicket = nullptr;
    int64_t n = 0;
    int64_t steps = 0, rebuilds = 0;
    bool forceValid = false;     // force array holds F(x) of the current positions
    bool needRebuild = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graphSteps = 0;      // steps captured in exec
    int64_t graphLaunches = 0;   // kernels per graph replay
    int64_t graphFirstSlot = -1; // energy slot of the first captured step
};

namespace
{
int kick_factors(mrmd_ctx* ctx, mrmd_md* md)
{
    k_kick_factors<<<grid_for(ctx, md->n, TB), TB, 0, ctx->stream>>>(md->atoms.mass, md->n, 0.5 * md->cfg.dt,
                                                                      md->dtfm);
    return after_launch(ctx, "kick_factors");
}

int md_rebuild(mrmd_ctx* ctx, mrmd_md* md)
{
    mrmd_atoms* a = &md->atoms;
    MRMD_TRY(mrmd_ghost_exchange_real_atoms(ctx, a, &md->sd));
    if (md->cfg.sortAtoms > 0 && md->rebuilds % md->cfg.sortAtoms == 0)
    {
        // Z-order of the cells: a warp's 32 atoms form a compact block, so
        // their neighbours overlap and the pair kernel's gathers hit in L1
        MRMD_TRY(md->sortCells.build(ctx, a->pos, md->n, md->grid, true));
        if (md->shadow.capacity < a->capacity)
        {
            mrmd_atoms_free(ctx, &md->shadow);
            MRMD_TRY(mrmd_atoms_alloc(ctx, &md->shadow, a->capacity));
        }
        a->numGhost = 0;
        MRMD_TRY(permute_atoms(ctx, a, &md->shadow, md->sortCells.sorted, md->n));
        k_gather_i32<<<grid_for(ctx, md->n, TB), TB, 0, ctx->stream>>>(md->orig, md->origTmp, md->sortCells.sorted,
                                                                        md->n);
        MRMD_TRY(after_launch(ctx, "gather_orig"));
        std::swap(md->orig, md->origTmp);
        MRMD_TRY(kick_factors(ctx, md));
    }
    MRMD_TRY(mrmd_ghost_create(ctx, &md->ghosts, a, &md->sd));
    const int64_t nAll = a->numLocal + a->numGhost;
    const bool full = md->cfg.precision == MRMD_PREC_MIXED;
    const double rlist = md->cfg.rc + md->cfg.skin;
    if (full)
    {
        // near rows: closer than r_split + skin / 2 at the rebuild, always in
        // double-float.  A far pair that comes within r_split later is still
        // evaluated in double-float (the pair kernel decides per pair).  A
        // margin of skin / 4 ran the pair kernel 0.9% faster but raised the
        // dilute-lattice error from 1.4e-6 to 2.1e-6 per atom (floored).
        if (md->farList.maxNeighbors == 0) md->farList.maxNeighbors = md->cfg.maxNeighbors;
        MRMD_TRY(build_split_list(ctx, &md->list, &md->farList, a->pos, nAll, 0, a->numLocal, rlist,
                                  md->rsplit + 0.5 * md->cfg.skin, md->grid,
                                  md->cfg.gatherNeighbours ? nullptr : &md->tiles, md->cfg.tileBuild == 0));
        MRMD_TRY(list_total_pairs(ctx, &md->farList));
        md->tp = make_tile_params(md->lj->p0, md->lj->rcSqr, md->rsplit, md->farList.maxNeighbors);
    }
    else
    {
        MRMD_TRY(build_half_list(ctx, &md->list, a->pos, nAll, 0, a->numLocal, rlist, md->grid,
                                 md->list.maxNeighbors > 0 ? md->list.maxNeighbors : md->cfg.maxNeighbors, false));
    }
    MRMD_TRY(list_total_pairs(ctx, &md->list));
    if (full && nAll > md->splitCap)
    {
        dfree(md->recA);
        md->recA = nullptr;
        md->recB = nullptr;
        const int64_t c = nAll + nAll / 8 + 64;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&md->recA), (sizeof(float4) + sizeof(float2)) * (size_t)c));
        md->recB = reinterpret_cast<float2*>(md->recA + c);
        md->splitCap = c;
    }
    md->rebuilds++;
    md->needRebuild = false;
    return MRMD_OK;
}

// Force evaluation of the current positions into atoms.force (zeroed by the
// caller), energy/virial added into ev.
int md_forces(mrmd_ctx* ctx, mrmd_md* md, double* ev, bool splitDone = false)
{
    mrmd_atoms* a = &md->atoms;
    if (md->cfg.precision == MRMD_PREC_MIXED)
    {
        const int64_t nAll = a->numLocal + a->numGhost;
        if (!splitDone) MRMD_TRY(tile_split_coords(ctx, a->pos, nAll, md->sp, md->recA, md->recB));
        return lj_tile_forces(ctx, &md->tiles, &md->list, &md->farList, md->recA, md->recB, a->force, md->tp, ev,
                              nAll, md->cfg.gatherNeighbours != 0);
    }
    MRMD_TRY(lj_apply_fp64(ctx, md->lj, a, &md->list, nullptr, ev));
    return mrmd_ghost_reduce_force(ctx, &md->ghosts, a);
}

// Kick / drift / force reset of one step; prevRec (may be null) receives the
// observables of the previous step when the stepper records them.
// split (mixed form, steps without rebuild): write the split coordinates of
// the new local positions instead of resetting the forces, which the tile
// pair kernel overwrites.
int md_kick_drift(mrmd_ctx* ctx, mrmd_md* md, bool postKick, double* prevRec, bool split = false)
{
    mrmd_atoms* a = &md->atoms;
    const unsigned grid = grid_for(ctx, md->n, TB);
    const bool obs = md->cfg.observe && postKick && prevRec;
#define KD_LAUNCH(O, S)                                                                                         \
    k_fused_kick_drift<O, S><<<grid, TB, 0, ctx->stream>>>(                                                     \
        reinterpret_cast<double4*>(a->pos), reinterpret_cast<double4*>(a->vel),                                 \
        reinterpret_cast<double4*>(a->force), a->mass, md->dtfm, md->n, md->cfg.dt, postKick ? 1 : 0,         \
        md->dPartial, md->dTicket, prevRec, md->sp, md->recA, md->recB)
    if (obs && split) KD_LAUNCH(true, true);
    else if (obs) KD_LAUNCH(true, false);
    else if (split) KD_LAUNCH(false, true);
    else KD_LAUNCH(false, false);
#undef KD_LAUNCH
    return after_launch(ctx, "fused_kick_drift");
}

// One step without rebuild, for capture: kick/drift, ghost update, forces
// into this step's record rec; prevRec (may be null) is the previous step's.
// The mixed form writes the split coordinates inside the kick/drift and
// ghost-update kernels instead of a separate pass over all positions.
int md_plain_step(mrmd_ctx* ctx, mrmd_md* md, double* rec, double* prevRec, bool postKick)
{
    mrmd_atoms* a = &md->atoms;
    const bool mixed = md->cfg.precision == MRMD_PREC_MIXED;
    MRMD_TRY(md_kick_drift(ctx, md, postKick, prevRec, mixed));
    if (!mixed)
    {
        MRMD_TRY(mrmd_ghost_update(ctx, &md->ghosts, a, &md->sd));
        return md_forces(ctx, md, rec);
    }
    const mrmd_ghost_layer* g = &md->ghosts;
    if (g->numLocal != a->numLocal || g->numGhost != a->numGhost)
        return set_error(ctx, MRMD_ERR_STATE, "ghost layer does not match atoms");
    if (a->numGhost > 0)
    {
        const mrmd_subdomain& sd = md->sd;
        k_ghost_update_split<<<grid_for(ctx, a->numGhost, TB), TB, 0, ctx->stream>>>(
            reinterpret_cast<double4*>(a->pos), g->correspondingRealAtom, a->numLocal, a->numGhost,
            make_double3(sd.diameter[0], sd.diameter[1], sd.diameter[2]),
            make_double3(0.1 * sd.diameter[0], 0.1 * sd.diameter[1], 0.1 * sd.diameter[2]), md->sp, md->recA,
            md->recB);
        MRMD_TRY(after_launch(ctx, "ghost_update_split"));
    }
    return md_forces(ctx, md, rec, true);
}

int ensure_energy(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps)
{
    if (nsteps + 1 <= md->energyCap) return MRMD_OK;
    cudaStreamSynchronize(ctx->stream);
    dfree(md->dEnergy);
    if (md->hEnergy) cudaFreeHost(md->hEnergy);
    md->dEnergy = nullptr;
    md->hEnergy = nullptr;
    const int64_t c = nsteps + 64;
    MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&md->dEnergy), sizeof(double) * REC * (size_t)c));
    MRMD_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&md->hEnergy), sizeof(double) * REC * (size_t)c));
    md->energyCap = c;
    // any captured graph referenced the old buffer
    if (md->exec)
    {
        cudaGraphExecDestroy(md->exec);
        md->exec = nullptr;
    }
    return MRMD_OK;
}

void drop_graph(mrmd_md* md)
{
    if (md->exec) cudaGraphExecDestroy(md->exec);
    if (md->graph) cudaGraphDestroy(md->graph);
    md->exec = nullptr;
    md->graph = nullptr;
    md->graphSteps = 0;
}

// Capture `count` plain steps writing energies into slots [slot0, slot0+count).
int capture_steps(mrmd_ctx* ctx, mrmd_md* md, int64_t count, int64_t slot0)
{
    cudaGraph_t g = nullptr;
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    MRMD_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = MRMD_OK;
    const int64_t launches0 = ctx->launches;
    for (int64_t k = 0; k < count && rc == MRMD_OK; ++k)
        rc = md_plain_step(ctx, md, md->dEnergy + REC * (slot0 + k), md->dEnergy + REC * (slot0 + k - 1), true);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    // captured kernels run when the graph is launched: count them there
    md->graphLaunches = ctx->launches - launches0;
    ctx->launches = launches0;
    ctx->sync = oldSync;
    if (rc != MRMD_OK)
    {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    MRMD_TRY(check_cuda(ctx, e, "end capture"));
    if (md->exec && md->graphSteps == count)
    {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(md->exec, g, &info) == cudaSuccess)
        {
            if (md->graph) cudaGraphDestroy(md->graph);
            md->graph = g;
            md->graphFirstSlot = slot0;
            return MRMD_OK;
        }
        cudaGetLastError();
    }
    drop_graph(md);
    md->graph = g;
    MRMD_CUDA(ctx, cudaGraphInstantiate(&md->exec, g, 0));
    md->graphSteps = count;
    md->graphFirstSlot = slot0;
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_md_create(mrmd_ctx* ctx, mrmd_md** out, const mrmd_md_config* cfg, int64_t n, const double* pos3,
                   const double* vel3, const double* mass)
{
    if (!ctx || !out || !cfg || !pos3 || !vel3 || n <= 0) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(cfg->rc > 0 && cfg->skin >= 0 && cfg->dt > 0 && cfg->rebuildInterval >= 1, ctx, "bad config");
    MRMD_CHECK_ARG(cfg->precision == MRMD_PREC_FP64 || cfg->precision == MRMD_PREC_MIXED, ctx, "bad precision");
    MRMD_CHECK_ARG(cfg->splitRadius >= 0.0, ctx, "splitRadius must be >= 0");
    MRMD_CHECK_ARG(n < INT32_MAX / 2, ctx, "too many atoms");
    *out = nullptr;
    mrmd_md* md = new mrmd_md();
    md->cfg = *cfg;
    if (md->cfg.maxNeighbors <= 0) md->cfg.maxNeighbors = md->cfg.precision == MRMD_PREC_MIXED ? 112 : 64;
    md->n = n;
    const double rlist = cfg->rc + cfg->skin;
    const double ghost3[3] = {rlist, rlist, rlist};
    int rc = mrmd_subdomain_init(&md->sd, cfg->boxMin, cfg->boxMax, ghost3);
    for (int d = 0; d < 3 && rc == MRMD_OK; ++d)
        if (!(md->sd.diameter[d] > rlist)) rc = set_error(ctx, MRMD_ERR_ARG, "box must exceed the list radius");
    if (rc == MRMD_OK)
    {
        // mixed form: cells of half the list radius (5^3 cells searched: 42%
        // fewer candidates than 3^3 cells of the full radius)
        md->grid = make_grid(md->sd.minGhostCorner, md->sd.maxGhostCorner, rlist,
                             cfg->precision == MRMD_PREC_MIXED ? 2 : 1);
        if (!tile_split_params(md->sd.minGhostCorner, md->grid.extent * 1.25 + 8.0, rlist, &md->sp))
            rc = set_error(ctx, MRMD_ERR_ARG, "box too large for the mixed form's coordinate split");
    }
    std::vector<double> m((size_t)n, 1.0);
    if (mass)
        for (int64_t i = 0; i < n; ++i) m[(size_t)i] = mass[i];
    std::vector<int64_t> type((size_t)n, 0);
    std::vector<double> rel((size_t)n, 1.0);
    const int64_t cap = n + n / 2 + 1024;
    if (rc == MRMD_OK) rc = mrmd_atoms_alloc(ctx, &md->atoms, cap);
    if (rc == MRMD_OK)
        rc = mrmd_atoms_upload(ctx, &md->atoms, n, 0, pos3, vel3, nullptr, type.data(), m.data(), nullptr, rel.data());
    if (rc == MRMD_OK) rc = mrmd_atoms_set_force(ctx, &md->atoms, cap, 0.0);
    if (rc == MRMD_OK) rc = mrmd_atoms_alloc(ctx, &md->shadow, cap);
    if (rc == MRMD_OK) rc = mrmd_ghost_layer_alloc(ctx, &md->ghosts, cap);
    if (rc == MRMD_OK) rc = mrmd_nlist_init(ctx, &md->list);
    if (rc == MRMD_OK) rc = mrmd_nlist_init(ctx, &md->farList);
    md->rsplit = cfg->splitRadius > 0.0 ? cfg->splitRadius : 1.5 * cfg->sigma;
    if (md->rsplit < 1.05 * cfg->cappingDistance) md->rsplit = 1.05 * cfg->cappingDistance;
    if (rc == MRMD_OK)
    {
        const double c = cfg->cappingDistance, r = cfg->rc, s = cfg->sigma, e = cfg->epsilon;
        rc = mrmd_lj_create(ctx, &md->lj, 1, 1, &c, &r, &s, &e, cfg->shifted);
    }
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&md->orig), sizeof(int32_t) * (size_t)n);
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&md->origTmp), sizeof(int32_t) * (size_t)n);
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&md->dtfm), sizeof(double) * (size_t)n);
    if (rc == MRMD_OK) rc = kick_factors(ctx, md);
    if (rc == MRMD_OK)
    {
        // one partial per block of the fused kernel, then the ticket
        const size_t parts = (size_t)grid_for(ctx, n, TB) * 4;
        rc = dmalloc(ctx, reinterpret_cast<void**>(&md->dPartial), sizeof(double) * parts + 256);
        if (rc == MRMD_OK)
        {
            md->dTicket = reinterpret_cast<unsigned*>(md->dPartial + parts);
            rc = dzero(ctx, md->dTicket, sizeof(unsigned));
        }
    }
    if (rc == MRMD_OK)
    {
        k_iota<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(md->orig, n);
        rc = after_launch(ctx, "iota");
    }
    if (rc == MRMD_OK) rc = ensure_energy(ctx, md, 1024);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "md_create");
    if (rc != MRMD_OK)
    {
        mrmd_md_destroy(ctx, md);
        return rc;
    }
    *out = md;
    return MRMD_OK;
}

int mrmd_md_destroy(mrmd_ctx* ctx, mrmd_md* md)
{
    if (!md) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    drop_graph(md);
    mrmd_atoms_free(ctx, &md->atoms);
    mrmd_atoms_free(ctx, &md->shadow);
    mrmd_ghost_layer_free(ctx, &md->ghosts);
    mrmd_nlist_free(ctx, &md->list);
    mrmd_nlist_free(ctx, &md->farList);
    mrmd_lj_destroy(ctx, md->lj);
    md->sortCells.release();
    md->tiles.release();
    dfree(md->orig);
    dfree(md->origTmp);
    dfree(md->recA);
    dfree(md->dEnergy);
    dfree(md->dPartial);
    dfree(md->dtfm);
    if (md->hEnergy) cudaFreeHost(md->hEnergy);
    delete md;
    return MRMD_OK;
}

}  // extern "C"

namespace
{
// The time loop; out (may be NULL) receives the first `cols` values of every
// step's record, [nsteps][cols].
int md_run(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps, double* out, int cols)
{
    if (!ctx || !md || nsteps < 0) return MRMD_ERR_ARG;
    if (nsteps == 0) return MRMD_OK;
    MRMD_TRY(ensure_energy(ctx, md, nsteps));
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    double* rec = md->dEnergy;
    int rc = check_cuda(ctx, cudaMemsetAsync(rec, 0, sizeof(double) * REC * (size_t)(nsteps + 1), ctx->stream),
                        "energy clear");
    mrmd_atoms* a = &md->atoms;
    const int64_t K = md->cfg.rebuildInterval;
    // make sure the force array holds F(x) before the first kick
    if (rc == MRMD_OK && !md->forceValid)
    {
        rc = md_rebuild(ctx, md);
        if (rc == MRMD_OK) rc = mrmd_atoms_set_force(ctx, a, a->numLocal + a->numGhost, 0.0);
        if (rc == MRMD_OK) rc = md_forces(ctx, md, rec + REC * nsteps);  // scratch slot
        md->forceValid = true;
    }
    // the previous step's record, for the kinetic energy its post-kick yields;
    // none for the first step of a run (the last run's end recorded it)
    auto prev = [&](int64_t slot) { return slot > 0 ? rec + REC * (slot - 1) : nullptr; };
    int64_t s = 0;
    while (rc == MRMD_OK && s < nsteps)
    {
        const int64_t global = md->steps + s;
        if (md->needRebuild || global % K == 0)
        {
            // rebuild step, eager: kick/drift, rebuild, forces
            rc = md_kick_drift(ctx, md, global > 0, prev(s));
            if (rc == MRMD_OK) rc = md_rebuild(ctx, md);
            if (rc == MRMD_OK) rc = mrmd_atoms_set_force(ctx, a, a->numLocal + a->numGhost, 0.0);
            if (rc == MRMD_OK) rc = md_forces(ctx, md, rec + REC * s);
            ++s;
            // the steps up to the next rebuild, as one graph (or eagerly)
            const int64_t nextRebuild = ((md->steps + s + K - 1) / K) * K;
            int64_t count = nextRebuild - (md->steps + s);
            if (count > nsteps - s) count = nsteps - s;
            if (rc == MRMD_OK && count > 0)
            {
                if (md->cfg.useGraph && count == K - 1)
                {
                    rc = capture_steps(ctx, md, count, s);
                    if (rc == MRMD_OK)
                    {
                        if (md->graphFirstSlot != s)
                            rc = set_error(ctx, MRMD_ERR_STATE, "graph slot mismatch");
                        else
                            rc = check_cuda(ctx, cudaGraphLaunch(md->exec, ctx->stream), "graph launch");
                        ctx->launches += md->graphLaunches;
                    }
                }
                else
                {
                    for (int64_t k = 0; k < count && rc == MRMD_OK; ++k)
                        rc = md_plain_step(ctx, md, rec + REC * (s + k), prev(s + k), true);
                }
                s += count;
            }
        }
        else
        {
            rc = md_plain_step(ctx, md, rec + REC * s, prev(s), true);
            ++s;
        }
    }
    md->steps += s;
    // The stored velocities stay half-kicked: the post-kick of the last step
    // is applied by the first fused kernel of the next run (and to a copy by
    // mrmd_md_get_state and here).
    if (rc == MRMD_OK && md->cfg.observe)
    {
        k_observe_post<<<grid_for(ctx, md->n, TB), TB, 0, ctx->stream>>>(
            reinterpret_cast<const double4*>(a->vel), reinterpret_cast<const double4*>(a->force), a->mass, md->n,
            0.5 * md->cfg.dt, md->steps > 0 ? 1 : 0, md->dPartial, md->dTicket, rec + REC * (nsteps - 1));
        rc = after_launch(ctx, "observe_post");
    }
    ctx->sync = oldSync;
    if (rc != MRMD_OK) return rc;
    if (out)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(md->hEnergy, rec, sizeof(double) * REC * (size_t)nsteps,
                                       cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t k = 0; k < nsteps; ++k)
            for (int c = 0; c < cols; ++c) out[k * cols + c] = md->hEnergy[k * REC + c];
    }
    return finish(ctx, "md_run");
}
}  // namespace

extern "C" {

int mrmd_md_run(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps, double* energies)
{
    return md_run(ctx, md, nsteps, energies, 2);
}

int mrmd_md_run_observed(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps, double* records)
{
    if (md && !md->cfg.observe) return set_error(ctx, MRMD_ERR_STATE, "the stepper was created without observe");
    return md_run(ctx, md, nsteps, records, REC);
}

int mrmd_md_get_state(mrmd_ctx* ctx, mrmd_md* md, double* pos3, double* vel3, double* force3)
{
    // Velocities are reported at the end of the last full step: the pending
    // post-kick of the last step is applied to a copy.
    if (!ctx || !md) return MRMD_ERR_ARG;
    mrmd_atoms* a = &md->atoms;
    const int64_t n = md->n;
    double* stage = static_cast<double*>(scratch(ctx, sizeof(double) * 3 * (size_t)n));
    if (!stage) return MRMD_ERR_OOM;
    double* hostOut[3] = {pos3, vel3, force3};
    for (int w = 0; w < 3; ++w)
    {
        if (!hostOut[w]) continue;
        const double* src = w == 0 ? a->pos : (w == 1 ? a->vel : a->force);
        if (w == 1 && md->steps > 0)
        {
            // v(t) = v_half + dt/2 F(t)/m on the shadow velocity buffer
            MRMD_CUDA(ctx, cudaMemcpyAsync(md->shadow.vel, a->vel, sizeof(double) * 4 * (size_t)n,
                                           cudaMemcpyDeviceToDevice, ctx->stream));
            k_post_kick<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(reinterpret_cast<double4*>(md->shadow.vel),
                                                                       reinterpret_cast<const double4*>(a->force),
                                                                       a->mass, n, 0.5 * md->cfg.dt);
            MRMD_TRY(after_launch(ctx, "post_kick"));
            src = md->shadow.vel;
        }
        k_unpermute3<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(src), md->orig, n,
                                                                    stage);
        MRMD_TRY(after_launch(ctx, "unpermute"));
        MRMD_CUDA(ctx, cudaMemcpyAsync(hostOut[w], stage, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return MRMD_OK;
}

int mrmd_md_set_state(mrmd_ctx* ctx, mrmd_md* md, const double* pos3, const double* vel3)
{
    if (!ctx || !md) return MRMD_ERR_ARG;
    mrmd_atoms* a = &md->atoms;
    const int64_t n = md->n;
    double* stage = static_cast<double*>(scratch(ctx, sizeof(double) * 3 * (size_t)n));
    if (!stage) return MRMD_ERR_OOM;
    const double* in[2] = {pos3, vel3};
    for (int w = 0; w < 2; ++w)
    {
        if (!in[w]) continue;
        MRMD_CUDA(ctx, cudaMemcpyAsync(stage, in[w], sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice,
                                       ctx->stream));
        k_permute_in3<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(stage, md->orig, n,
                                                                     reinterpret_cast<double4*>(w == 0 ? a->pos : a->vel));
        MRMD_TRY(after_launch(ctx, "permute_in"));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    md->needRebuild = true;
    md->forceValid = false;
    md->steps = 0;
    return MRMD_OK;
}

int mrmd_md_stats(const mrmd_md* md, int64_t* out5)
{
    if (!md || !out5) return MRMD_ERR_ARG;
    out5[0] = md->steps;
    out5[1] = md->rebuilds;
    out5[2] = md->list.totalPairs + (md->cfg.precision == MRMD_PREC_MIXED ? md->farList.totalPairs : 0);
    out5[3] = md->atoms.numGhost;
    out5[4] = md->list.maxNeighbors + (md->cfg.precision == MRMD_PREC_MIXED ? md->farList.maxNeighbors : 0);
    return MRMD_OK;
}

int mrmd_md_eval(mrmd_ctx* ctx, mrmd_md* md, int what, double* ev2)
{
    if (!ctx || !md || (what != 0 && what != 1)) return MRMD_ERR_ARG;
    mrmd_atoms* a = &md->atoms;
    MRMD_TRY(ensure_energy(ctx, md, 1));
    double* ev = md->dEnergy + REC * (md->energyCap - 1);
    if (what == 1)
    {
        if (md->needRebuild || !md->forceValid) return set_error(ctx, MRMD_ERR_STATE, "no list: run or eval first");
        if (md->cfg.precision == MRMD_PREC_MIXED)
            return lj_tile_forces(ctx, &md->tiles, &md->list, &md->farList, md->recA, md->recB, a->force, md->tp,
                                  ev, a->numLocal + a->numGhost, md->cfg.gatherNeighbours != 0);
        return lj_apply_fp64(ctx, md->lj, a, &md->list, nullptr, ev);
    }
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    int rc = MRMD_OK;
    if (md->needRebuild || !md->forceValid) rc = md_rebuild(ctx, md);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(ev, 0, 2 * sizeof(double), ctx->stream), "ev");
    if (rc == MRMD_OK) rc = mrmd_atoms_set_force(ctx, a, a->numLocal + a->numGhost, 0.0);
    if (rc == MRMD_OK) rc = md_forces(ctx, md, ev);
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    md->forceValid = true;
    MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 40, ev, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ev2)
    {
        ev2[0] = ctx->hostScalars[40];
        ev2[1] = ctx->hostScalars[41];
    }
    return MRMD_OK;
}

const mrmd_atoms* mrmd_md_atoms(const mrmd_md* md) { return md ? &md->atoms : nullptr; }
const mrmd_nlist* mrmd_md_nlist(const mrmd_md* md) { return md ? &md->list : nullptr; }

int mrmd_md_tile_stats(const mrmd_md* md, int64_t* out6)
{
    if (!md || !out6) return MRMD_ERR_ARG;
    const bool mixed = md->cfg.precision == MRMD_PREC_MIXED;
    out6[0] = mixed ? md->tiles.tiles : 0;
    out6[1] = mixed ? md->tiles.maxMembers : 0;
    out6[2] = mixed && md->tiles.valid && !md->cfg.gatherNeighbours ? 1 : 0;
    out6[3] = mixed ? md->tiles.totalMembers : 0;
    out6[4] = mixed ? md->tiles.unfitTiles : 0;
    out6[5] = mixed ? md->tiles.twoPassBuilds : 0;
    return MRMD_OK;
}

}  // extern "C"

namespace
{
// Entries of a list in a 32-row tile layout (element type T, `cap` elements
// per row), with the row counts.
template <typename T>
int download_rows(mrmd_ctx* ctx, const T* dev, const int32_t* devCounts, int64_t rows, int64_t cap,
                  std::vector<int32_t>& counts, std::vector<T>& entries)
{
    counts.assign((size_t)rows, 0);
    entries.assign((size_t)(div_up(rows, 32) * 32 * cap), T{});
    if (rows == 0) return MRMD_OK;
    MRMD_TRY(d2h(ctx, counts.data(), devCounts, sizeof(int32_t) * (size_t)rows));
    if (cap > 0) MRMD_TRY(d2h(ctx, entries.data(), dev, sizeof(T) * entries.size()));
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_md_pair_keys(mrmd_ctx* ctx, mrmd_md* md, int64_t* keys, int64_t cap, int64_t* count)
{
    if (!ctx || !md || !count) return MRMD_ERR_ARG;
    if (md->needRebuild || !md->forceValid) return set_error(ctx, MRMD_ERR_STATE, "no list: run or eval first");
    const mrmd_atoms* a = &md->atoms;
    const int64_t n = a->numLocal, nAll = a->numLocal + a->numGhost;
    std::vector<int32_t> orig((size_t)n), corr((size_t)nAll);
    MRMD_TRY(d2h(ctx, orig.data(), md->orig, sizeof(int32_t) * (size_t)n));
    MRMD_TRY(d2h(ctx, corr.data(), md->ghosts.correspondingRealAtom, sizeof(int32_t) * (size_t)nAll));
    const bool mixed = md->cfg.precision == MRMD_PREC_MIXED;
    const bool tiled = mixed && md->tiles.valid && !md->cfg.gatherNeighbours;
    std::vector<int32_t> members, memberCount;
    if (tiled)
    {
        const int64_t tiles = md->tiles.tiles;
        members.resize((size_t)(tiles * TILE_CAP));
        memberCount.resize((size_t)tiles);
        MRMD_TRY(d2h(ctx, members.data(), md->tiles.members, sizeof(int32_t) * members.size()));
        MRMD_TRY(d2h(ctx, memberCount.data(), md->tiles.memberCount, sizeof(int32_t) * memberCount.size()));
    }
    std::vector<int64_t> out;
    auto add = [&](int64_t i, int64_t j) -> int {
        if (j < 0 || j >= nAll) return set_error(ctx, MRMD_ERR_STATE, "list entry %lld outside the atoms", (long long)j);
        const int64_t r = j < n ? j : corr[(size_t)j];
        if (r < 0 || r >= n) return set_error(ctx, MRMD_ERR_STATE, "ghost %lld without a real atom", (long long)j);
        const int64_t oi = orig[(size_t)i], oj = orig[(size_t)r];
        out.push_back(oi < oj ? (oi << 32) | oj : (oj << 32) | oi);
        return MRMD_OK;
    };
    const mrmd_nlist* lists[2] = {&md->list, mixed ? &md->farList : nullptr};
    for (int w = 0; w < 2; ++w)
    {
        const mrmd_nlist* nl = lists[w];
        if (!nl || nl->rows == 0) continue;
        std::vector<int32_t> counts;
        if (tiled)
        {
            const int64_t nch = w == 0 ? md->tiles.nearChunksPerRow : md->tiles.farChunksPerRow;
            std::vector<uint4> e;
            MRMD_TRY(download_rows(ctx, w == 0 ? md->tiles.nearChunks : md->tiles.farChunks, nl->counts, nl->rows,
                                   nch, counts, e));
            for (int64_t i = 0; i < nl->rows; ++i)
            {
                const int64_t t = i / TILE_ROWS;
                for (int64_t k = 0; k < counts[(size_t)i]; ++k)
                {
                    const uint4 c = e[(size_t)chunk_word(i, k >> 3, nch)];
                    const uint32_t word = (k & 7) < 2 ? c.x : (k & 7) < 4 ? c.y : (k & 7) < 6 ? c.z : c.w;
                    const int64_t slot = (word >> (16 * (k & 1))) & 0xffffu;
                    if (slot >= memberCount[(size_t)t]) return set_error(ctx, MRMD_ERR_STATE, "slot beyond the tile");
                    MRMD_TRY(add(i, members[(size_t)(t * TILE_CAP + slot)]));
                }
            }
        }
        else
        {
            const int64_t lcap = nl->maxNeighbors;
            std::vector<int32_t> e;
            MRMD_TRY(download_rows(ctx, nl->nbrs, nl->counts, nl->rows, lcap, counts, e));
            for (int64_t i = 0; i < nl->rows; ++i)
                for (int64_t k = 0; k < counts[(size_t)i]; ++k)
                    MRMD_TRY(add(i, e[(size_t)((i >> 5) * (lcap << 5) + (k << 5) + (i & 31))]));
        }
    }
    std::sort(out.begin(), out.end());
    *count = (int64_t)out.size();
    if (!keys) return MRMD_OK;
    if (cap < *count) return set_error(ctx, MRMD_ERR_CAPACITY, "pair key capacity %lld < %lld", (long long)cap,
                                       (long long)*count);
    std::memcpy(keys, out.data(), sizeof(int64_t) * out.size());
    return MRMD_OK;
}

}  // extern "C"
