// Fused AdResS LJ <-> ideal-gas stepper for single-site molecules.
//
// MRMD has no AdResS driver; the step composes the reference actions in the
// order their data dependencies require:
//   VelocityVerletLangevinThermostat::preForceIntegrate      (B A O A)
//   every K steps: UpdateMolecules (centres), MultiResGhostLayer::
//     exchangeRealAtoms + createGhostAtoms, molecule half Verlet list
//   else: ghost position update
//   UpdateMolecules (lambda, grad lambda of local + ghost molecules)
//   forces = 0; LJ_IdealGas::run; ContributeMoleculeForceToAtoms;
//   ThermodynamicForce::apply; ghost force fold-back; postForceIntegrate
//   ThermodynamicForce::sample every S steps, ::update every U steps.
// The steps between rebuilds are captured once per rebuild and replayed as
// one CUDA graph.
//
// With unit masses (single-site molecules of the AdResS workload) the same
// step runs on the batched engine with one replica instead (batch.cu: full
// list without the pairs of molecules that stay coarse grained, FP32 far
// pairs in the mixed form, four launches per step in CUDA graphs); the
// composed actions above serve other masses.
#include <cmath>
#include <vector>

#include "batch_impl.cuh"
#include "common.cuh"
#include "lj_mixed.cuh"
#include "nlist_impl.cuh"
#include "stepper_impl.cuh"

using namespace mrmd_impl;

struct mrmd_adress
{
    mrmd_adress_config cfg{};
    mrmd_subdomain sd{};
    mrmd_slab slab{};
    mrmd_atoms atoms{};
    mrmd_molecules mol{};
    mrmd_ghost_layer ghosts{};
    mrmd_nlist list{};
    mrmd_ljig* ljig = nullptr;
    mrmd_tf* tf = nullptr;
    CellGrid grid{};
    float4* split = nullptr;
    int64_t splitCap = 0;
    double* dEnergy = nullptr;
    int64_t energyCap = 0;
    double* dScratch = nullptr;  // [0]: max displacement sink
    int64_t n = 0, steps = 0, rebuilds = 0;
    bool needRebuild = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graphSteps = 0, graphLaunches = 0;
    mrmd_batch* batch = nullptr;  // unit masses: the batched engine runs the step
    mrmd_ctx* ctx = nullptr;      // the context the system was created on
};

namespace
{
int ad_rebuild(mrmd_ctx* ctx, mrmd_adress* s)
{
    mrmd_atoms* a = &s->atoms;
    mrmd_molecules* m = &s->mol;
    a->numGhost = 0;
    m->numGhost = 0;
    MRMD_TRY(mrmd_update_molecules(ctx, m, a, &s->slab));
    MRMD_TRY(mrmd_multires_exchange_real_atoms(ctx, m, a, &s->sd));
    MRMD_TRY(mrmd_multires_ghost_create(ctx, &s->ghosts, m, a, &s->sd));
    const int64_t nM = m->numLocal + m->numGhost;
    const double rlist = s->cfg.rc + s->cfg.skin;
    MRMD_TRY(build_half_list(ctx, &s->list, m->pos, nM, 0, m->numLocal, rlist, s->grid,
                             s->list.maxNeighbors > 0 ? s->list.maxNeighbors : s->cfg.maxNeighbors, false));
    MRMD_TRY(list_total_pairs(ctx, &s->list));
    const int64_t nA = a->numLocal + a->numGhost;
    if (s->cfg.precision == MRMD_PREC_MIXED && nA > s->splitCap)
    {
        cudaStreamSynchronize(ctx->stream);
        dfree(s->split);
        s->split = nullptr;
        const int64_t c = nA + nA / 8 + 64;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&s->split), sizeof(float4) * 2 * (size_t)c));
        s->splitCap = c;
    }
    s->rebuilds++;
    s->needRebuild = false;
    return MRMD_OK;
}

// one step; `rebuild` selects the rebuild branch; energy -> *ev (zeroed at run start)
int ad_step(mrmd_ctx* ctx, mrmd_adress* s, int64_t st, bool rebuild, double* ev)
{
    mrmd_atoms* a = &s->atoms;
    mrmd_molecules* m = &s->mol;
    const mrmd_adress_config& c = s->cfg;
    MRMD_TRY(langevin_pre_async(ctx, a, c.dt, c.gamma, c.temperature, c.seed, (uint64_t)st, nullptr, s->dScratch));
    if (rebuild)
        MRMD_TRY(ad_rebuild(ctx, s));
    else
        MRMD_TRY(mrmd_ghost_update(ctx, &s->ghosts, a, &s->sd));
    MRMD_TRY(mrmd_update_molecules(ctx, m, a, &s->slab));
    MRMD_TRY(mrmd_atoms_set_force(ctx, a, a->numLocal + a->numGhost, 0.0));
    MRMD_TRY(mrmd_molecules_set_force(ctx, m, m->numLocal + m->numGhost, 0.0));
    const float4* hi = nullptr;
    const float4* lo = nullptr;
    if (c.precision == MRMD_PREC_MIXED)
    {
        MRMD_TRY(split_coords(ctx, a->pos, a->numLocal + a->numGhost, split_params_for(&s->list), s->split,
                              s->split + s->splitCap));
        hi = s->split;
        lo = s->split + s->splitCap;
    }
    MRMD_TRY(ljig_run_async(ctx, s->ljig, m, &s->list, a, c.precision, ev, hi, lo));
    MRMD_TRY(mrmd_contribute_molecule_force(ctx, m, a));
    if (c.tfEnabled) MRMD_TRY(mrmd_tf_apply(ctx, s->tf, a, nullptr, 0));
    MRMD_TRY(mrmd_ghost_reduce_force(ctx, &s->ghosts, a));
    MRMD_TRY(mrmd_vv_post(ctx, a, c.dt));
    if (c.tfEnabled && st % c.tfSampleInterval == 0) MRMD_TRY(mrmd_tf_sample(ctx, s->tf, a));
    if (c.tfEnabled && (st + 1) % c.tfUpdateInterval == 0)
        MRMD_TRY(mrmd_tf_update(ctx, s->tf, c.tfSmoothingSigma, c.tfSmoothingRange, nullptr));
    return MRMD_OK;
}

void ad_drop_graph(mrmd_adress* s)
{
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
    s->graphSteps = 0;
}

int ad_capture(mrmd_ctx* ctx, mrmd_adress* s, int64_t st0, int64_t count, int64_t slot0)
{
    cudaGraph_t g = nullptr;
    MRMD_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = ctx->launches;
    int rc = MRMD_OK;
    for (int64_t k = 0; k < count && rc == MRMD_OK; ++k)
        rc = ad_step(ctx, s, st0 + k, false, s->dEnergy + (slot0 + k));
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    s->graphLaunches = ctx->launches - l0;
    ctx->launches = l0;
    if (rc != MRMD_OK)
    {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    MRMD_TRY(check_cuda(ctx, e, "end capture"));
    if (s->exec && s->graphSteps == count)
    {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(s->exec, g, &info) == cudaSuccess)
        {
            if (s->graph) cudaGraphDestroy(s->graph);
            s->graph = g;
            return MRMD_OK;
        }
        cudaGetLastError();
    }
    ad_drop_graph(s);
    s->graph = g;
    MRMD_CUDA(ctx, cudaGraphInstantiate(&s->exec, g, 0));
    s->graphSteps = count;
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_adress_create(mrmd_ctx* ctx, mrmd_adress** out, const mrmd_adress_config* cfg, int64_t n,
                       const double* pos3, const double* vel3, const double* mass)
{
    if (!ctx || !out || !cfg || !pos3 || !vel3 || n <= 0) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(cfg->rc > 0 && cfg->skin >= 0 && cfg->dt > 0 && cfg->rebuildInterval >= 1, ctx, "bad config");
    MRMD_CHECK_ARG(cfg->precision == MRMD_PREC_FP64 || cfg->precision == MRMD_PREC_MIXED, ctx, "bad precision");
    MRMD_CHECK_ARG(!cfg->tfEnabled || (cfg->tfSampleInterval >= 1 && cfg->tfUpdateInterval >= 1), ctx,
                   "bad thermodynamic-force intervals");
    *out = nullptr;
    bool unitMass = cfg->composed == 0;
    for (int64_t i = 0; mass && i < n && unitMass; ++i) unitMass = mass[i] == 1.0;
    if (unitMass)
    {
        mrmd_batch_config bc{};
        bc.rc = cfg->rc;
        bc.skin = cfg->skin;
        bc.sigma = cfg->sigma;
        bc.epsilon = cfg->epsilon;
        bc.cappingDistance = cfg->cappingDistance;
        bc.shifted = cfg->shifted;
        bc.precision = cfg->precision;
        bc.dt = cfg->dt;
        bc.hybridDiameter = cfg->hybridDiameter;
        bc.nu = cfg->nu;
        bc.gamma = cfg->gamma;
        bc.temperature = cfg->temperature;
        bc.tfEnabled = cfg->tfEnabled;
        bc.tfBinWidth = cfg->tfBinWidth;
        bc.tfTargetDensity = cfg->tfTargetDensity;
        bc.tfModulation = cfg->tfModulation;
        bc.tfSmoothingSigma = cfg->tfSmoothingSigma;
        bc.tfSmoothingRange = cfg->tfSmoothingRange;
        bc.tfSampleInterval = cfg->tfSampleInterval;
        bc.tfUpdateInterval = cfg->tfUpdateInterval;
        bc.initialMaxNeighbors = cfg->maxNeighbors > 0 ? cfg->maxNeighbors : 0;
        // cell sort every 5th rebuild; graphs of 5 rebuild intervals; from a
        // million molecules the steps between rebuilds as one persistent
        // launch (4,000,000 molecules: 2.01 against 2.33 ms per step mixed,
        // 5.13 against 5.25 FP64; 34,560: 6% slower)
        bc.tuning.threadsPerRow = 1;
        bc.tuning.blockSize = 128;
        bc.tuning.rebuildInterval = cfg->rebuildInterval;
        bc.tuning.sortEvery = 5;
        bc.tuning.graphSteps = cfg->useGraph ? 5 * cfg->rebuildInterval : 0;
        bc.tuning.listLayout = 0;
        bc.tuning.persistent = cfg->useGraph && n >= 1000000 ? 1 : 0;
        mrmd_replica_desc rd{};
        rd.numMolecules = n;
        for (int d = 0; d < 3; ++d)
        {
            rd.boxMin[d] = cfg->boxMin[d];
            rd.boxMax[d] = cfg->boxMax[d];
            rd.slabCenter[d] = cfg->slabCenter[d];
        }
        rd.atomisticDiameter = cfg->atomisticDiameter;
        rd.seed = cfg->seed;
        mrmd_batch* b = nullptr;
        MRMD_TRY(mrmd_batch_create(ctx, &b, &bc, 1, &rd, pos3, vel3));
        mrmd_adress* s = new mrmd_adress();
        s->cfg = *cfg;
        s->n = n;
        s->batch = b;
        s->ctx = ctx;
        *out = s;
        return MRMD_OK;
    }
    mrmd_adress* s = new mrmd_adress();
    s->cfg = *cfg;
    s->ctx = ctx;
    if (s->cfg.maxNeighbors <= 0) s->cfg.maxNeighbors = 64;
    s->n = n;
    const double rlist = cfg->rc + cfg->skin;
    const double ghost3[3] = {rlist, rlist, rlist};
    int rc = mrmd_subdomain_init(&s->sd, cfg->boxMin, cfg->boxMax, ghost3);
    for (int d = 0; d < 3 && rc == MRMD_OK; ++d)
        if (!(s->sd.diameter[d] > rlist)) rc = set_error(ctx, MRMD_ERR_ARG, "box must exceed the list radius");
    if (rc == MRMD_OK)
    {
        s->grid = make_grid(s->sd.minGhostCorner, s->sd.maxGhostCorner, rlist);
        for (int d = 0; d < 3; ++d) s->slab.center[d] = cfg->slabCenter[d];
        s->slab.atomisticRegionDiameter = cfg->atomisticDiameter;
        s->slab.hybridRegionDiameter = cfg->hybridDiameter;
        s->slab.nu = cfg->nu;
        s->slab.interfaceType = 0;
    }
    const int64_t cap = 2 * n + 1024;  // ghosts of a thin slab box can exceed n/2
    std::vector<double> m((size_t)n, 1.0), rel((size_t)n, 1.0);
    if (mass)
        for (int64_t i = 0; i < n; ++i) m[(size_t)i] = mass[i];
    std::vector<int64_t> type((size_t)n, 0), off((size_t)n), na((size_t)n, 1);
    for (int64_t i = 0; i < n; ++i) off[(size_t)i] = i;
    if (rc == MRMD_OK) rc = mrmd_atoms_alloc(ctx, &s->atoms, cap);
    if (rc == MRMD_OK)
        rc = mrmd_atoms_upload(ctx, &s->atoms, n, 0, pos3, vel3, nullptr, type.data(), m.data(), nullptr, rel.data());
    if (rc == MRMD_OK) rc = mrmd_atoms_set_force(ctx, &s->atoms, cap, 0.0);
    if (rc == MRMD_OK) rc = mrmd_molecules_alloc(ctx, &s->mol, cap);
    if (rc == MRMD_OK)
        rc = mrmd_molecules_upload(ctx, &s->mol, n, 0, pos3, nullptr, nullptr, nullptr, nullptr, off.data(), na.data());
    if (rc == MRMD_OK) rc = mrmd_ghost_layer_alloc(ctx, &s->ghosts, cap);
    if (rc == MRMD_OK) rc = mrmd_nlist_init(ctx, &s->list);
    if (rc == MRMD_OK)
    {
        const double c = cfg->cappingDistance, r = cfg->rc, sg = cfg->sigma, e = cfg->epsilon;
        rc = mrmd_ljig_create(ctx, &s->ljig, 1, &c, &r, &sg, &e, cfg->shifted);
    }
    if (rc == MRMD_OK && cfg->tfEnabled)
    {
        const double td = cfg->tfTargetDensity, mod = cfg->tfModulation;
        rc = mrmd_tf_create(ctx, &s->tf, 1, &td, &s->sd, cfg->tfBinWidth, &mod, 0, 1);
    }
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&s->dScratch), 64 * sizeof(double));
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "adress_create");
    if (rc != MRMD_OK)
    {
        mrmd_adress_destroy(ctx, s);
        return rc;
    }
    *out = s;
    return MRMD_OK;
}

int mrmd_adress_destroy(mrmd_ctx* ctx, mrmd_adress* s)
{
    if (!s) return MRMD_OK;
    if (s->batch)
    {
        const int rc = mrmd_batch_destroy(ctx, s->batch);
        delete s;
        return rc;
    }
    if (ctx) cudaStreamSynchronize(ctx->stream);
    ad_drop_graph(s);
    mrmd_atoms_free(ctx, &s->atoms);
    mrmd_molecules_free(ctx, &s->mol);
    mrmd_ghost_layer_free(ctx, &s->ghosts);
    mrmd_nlist_free(ctx, &s->list);
    mrmd_ljig_destroy(ctx, s->ljig);
    mrmd_tf_destroy(ctx, s->tf);
    dfree(s->split);
    dfree(s->dEnergy);
    dfree(s->dScratch);
    delete s;
    return MRMD_OK;
}

int mrmd_adress_run(mrmd_ctx* ctx, mrmd_adress* s, int64_t nsteps, double* energies)
{
    if (!ctx || !s || nsteps < 0) return MRMD_ERR_ARG;
    if (s->batch) return mrmd_batch_run(ctx, s->batch, nsteps, energies);
    if (nsteps == 0) return MRMD_OK;
    if (nsteps + 1 > s->energyCap)
    {
        cudaStreamSynchronize(ctx->stream);
        dfree(s->dEnergy);
        s->dEnergy = nullptr;
        ad_drop_graph(s);  // graphs reference the old buffer
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&s->dEnergy), sizeof(double) * (size_t)(nsteps + 64)));
        s->energyCap = nsteps + 64;
    }
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    int rc = check_cuda(ctx, cudaMemsetAsync(s->dEnergy, 0, sizeof(double) * (size_t)(nsteps + 1), ctx->stream),
                        "energy clear");
    const int64_t K = s->cfg.rebuildInterval;
    int64_t k = 0;
    while (rc == MRMD_OK && k < nsteps)
    {
        const int64_t st = s->steps + k;
        if (s->needRebuild || st % K == 0)
        {
            rc = ad_step(ctx, s, st, true, s->dEnergy + k);
            ++k;
            const int64_t next = ((s->steps + k + K - 1) / K) * K;
            int64_t count = next - (s->steps + k);
            if (count > nsteps - k) count = nsteps - k;
            if (rc == MRMD_OK && count > 0)
            {
                if (s->cfg.useGraph && count == K - 1)
                {
                    rc = ad_capture(ctx, s, s->steps + k, count, k);
                    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaGraphLaunch(s->exec, ctx->stream), "graph launch");
                    ctx->launches += s->graphLaunches;
                }
                else
                {
                    for (int64_t q = 0; q < count && rc == MRMD_OK; ++q)
                        rc = ad_step(ctx, s, s->steps + k + q, false, s->dEnergy + k + q);
                }
                k += count;
            }
        }
        else
        {
            rc = ad_step(ctx, s, st, false, s->dEnergy + k);
            ++k;
        }
    }
    s->steps += k;
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    if (energies)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(energies, s->dEnergy, sizeof(double) * (size_t)nsteps, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    }
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "adress_run");
}

int mrmd_adress_get_state(mrmd_ctx* ctx, mrmd_adress* s, double* pos3, double* vel3, double* force3)
{
    if (!ctx || !s) return MRMD_ERR_ARG;
    if (s->batch) return mrmd_batch_get_state(ctx, s->batch, pos3, vel3, force3);
    return mrmd_atoms_download(ctx, &s->atoms, s->n, pos3, vel3, force3, nullptr, nullptr, nullptr, nullptr);
}

int mrmd_adress_get_tf(mrmd_ctx* ctx, mrmd_adress* s, double* force, double* density, int64_t* numBins)
{
    if (!ctx || !s) return MRMD_ERR_ARG;
    if (s->batch)
    {
        if (!s->cfg.tfEnabled) return MRMD_ERR_ARG;
        int64_t offsets[2] = {0, 0};
        MRMD_TRY(mrmd_batch_get_tf(ctx, s->batch, force, density, offsets));
        if (numBins) *numBins = offsets[1];
        return MRMD_OK;
    }
    if (!s->tf) return MRMD_ERR_ARG;
    if (numBins) mrmd_tf_shape(s->tf, numBins, nullptr, nullptr);
    if (force) MRMD_TRY(mrmd_tf_get_force(ctx, s->tf, force));
    if (density) MRMD_TRY(mrmd_tf_get_density(ctx, s->tf, density, nullptr));
    return MRMD_OK;
}

int mrmd_adress_set_tf(mrmd_ctx* ctx, mrmd_adress* s, const double* force)
{
    if (!ctx || !s || !force) return MRMD_ERR_ARG;
    if (s->batch) return s->cfg.tfEnabled ? mrmd_batch_set_tf(ctx, s->batch, force) : MRMD_ERR_ARG;
    if (!s->tf) return MRMD_ERR_ARG;
    return mrmd_tf_set_force(ctx, s->tf, force);
}

int mrmd_adress_stats(const mrmd_adress* s, int64_t* out4)
{
    if (!s || !out4) return MRMD_ERR_ARG;
    if (s->batch)
    {
        int64_t b10[10];
        MRMD_TRY(mrmd_batch_stats(s->ctx, s->batch, b10));
        out4[0] = b10[0];
        out4[1] = b10[1];
        out4[2] = b10[2];
        out4[3] = b10[3];
        return MRMD_OK;
    }
    out4[0] = s->steps;
    out4[1] = s->rebuilds;
    out4[2] = s->list.totalPairs;
    out4[3] = s->mol.numGhost;
    return MRMD_OK;
}

}  // extern "C"
