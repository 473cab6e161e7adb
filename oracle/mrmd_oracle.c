/*
 * mrmd_oracle.c -- CPU FP64 restatement of MRMD's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed CPU
 * baseline.  Nothing in the product path links or loads this file.
 * Citations are path:line inside the MRMD source tree (v0.2.0).
 */
#include "mrmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

int orc_set_threads(int n)
{
    int old = g_threads;
    g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
    return old;
}

int orc_get_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------ domain ---- */

void orc_subdomain_init(orc_subdomain* sd, const double* minCorner, const double* maxCorner,
                        const double* ghost)
{
    for (int d = 0; d < 3; ++d)
    {
        sd->minCorner[d] = minCorner[d];
        sd->maxCorner[d] = maxCorner[d];
        sd->ghostLayerThickness[d] = ghost[d];
        sd->minGhostCorner[d] = minCorner[d] - ghost[d];
        sd->maxGhostCorner[d] = maxCorner[d] + ghost[d];
        sd->minInnerCorner[d] = minCorner[d] + ghost[d];
        sd->maxInnerCorner[d] = maxCorner[d] - ghost[d];
        sd->diameter[d] = maxCorner[d] - minCorner[d];
        sd->diameterWithGhostLayer[d] = maxCorner[d] - minCorner[d] + 2.0 * ghost[d];
    }
}

/* -------------------------------------------------------------- preds --- */

static int in_symmetric_slab(const orc_pred* p, double coord)
{
    /* util/IsInSymmetricSlab.hpp:33-41 */
    double dx = coord - p->center;
    double absDx = fabs(dx);
    return (absDx >= p->slabMin - p->tolerance && absDx <= p->slabMax + p->tolerance);
}

static int pred_coord(const orc_pred* p, double c)
{
    if (p == NULL) return 1;
    switch (p->kind)
    {
        case ORC_PRED_ALWAYS: return 1;
        case ORC_PRED_IN_SLAB: return in_symmetric_slab(p, c);
        case ORC_PRED_IN_OPEN_INTERVAL: return c > p->slabMin && c < p->slabMax;
        default: return 1;
    }
}

int orc_pred_eval1(const orc_pred* p, double x, double y, double z)
{
    if (p == NULL) return 1;
    double v[3] = {x, y, z};
    return pred_coord(p, v[p->axis]);
}

int orc_pred_eval2(const orc_pred* p, double x1, double y1, double z1, double x2, double y2,
                   double z2)
{
    if (p == NULL || p->kind == ORC_PRED_ALWAYS) return 1;
    double a[3] = {x1, y1, z1};
    double b[3] = {x2, y2, z2};
    int ia = in_symmetric_slab(p, a[p->axis]);
    int ib = in_symmetric_slab(p, b[p->axis]);
    if (p->kind == ORC_PRED_EITHER_IN_SLAB) return ia || ib;
    if (p->kind == ORC_PRED_BOTH_IN_SLAB) return ia && ib;
    return 1;
}

/* ----------------------------------------------------------------- LJ --- */

void orc_lj_force_energy(const orc_lj_params* t, double distSqr, int64_t typeIdx, double* ff,
                         double* e)
{
    /* action/LennardJones.hpp:52-78 */
    const orc_lj_params* p = &t[typeIdx];
    if (distSqr >= p->cappingDistanceSqr)
    {
        double frac2 = 1.0 / distSqr;
        double frac6 = frac2 * frac2 * frac2;
        *ff = frac6 * (p->ff1 * frac6 - p->ff2) * frac2;
        *e = frac6 * (p->ef1 * frac6 - p->ef2) - p->shift;
        return;
    }
    double dist = sqrt(distSqr);
    *ff = p->cappingCoeff / dist;
    *e = p->energyAtCappingPoint - (dist - p->cappingDistance) * p->cappingCoeff - p->shift;
}

void orc_lj_init(orc_lj_params* out, int64_t numTypes, const double* cap, const double* rc,
                 const double* sigma, const double* epsilon, int isShifted)
{
    /* action/LennardJones.cpp:81-116 */
    for (int64_t t = 0; t < numTypes * numTypes; ++t)
    {
        double sig2 = sigma[t] * sigma[t];
        double sig6 = sig2 * sig2 * sig2;
        memset(&out[t], 0, sizeof(orc_lj_params));
        out[t].ff1 = 48.0 * epsilon[t] * sig6 * sig6;
        out[t].ff2 = 24.0 * epsilon[t] * sig6;
        out[t].ef1 = 4.0 * epsilon[t] * sig6 * sig6;
        out[t].ef2 = 4.0 * epsilon[t] * sig6;
        out[t].rcSqr = rc[t] * rc[t];
        out[t].cappingDistance = cap[t];
    }
    /* operator(), action/LennardJones.cpp:61-79 */
    for (int64_t t = 0; t < numTypes * numTypes; ++t)
    {
        double capDist = out[t].cappingDistance;
        out[t].cappingDistance = 0.0;
        out[t].cappingDistanceSqr = 0.0;
        double ff, e;
        orc_lj_force_energy(out, capDist * capDist, t, &ff, &e);
        out[t].cappingCoeff = ff * capDist;
        out[t].energyAtCappingPoint = e;
        out[t].cappingDistance = capDist;
        out[t].cappingDistanceSqr = capDist * capDist;
        if (isShifted)
        {
            orc_lj_force_energy(out, out[t].rcSqr, t, &ff, &e);
            out[t].shift = e;
        }
    }
}

void orc_lj_apply(const orc_lj_params* table, int64_t numTypesIndex, double rcSqr,
                  orc_atoms* atoms, const int32_t* counts, const int32_t* nbrs, int64_t cap,
                  const orc_pred* pred, double* energyOut, double* virialOut)
{
    /* action/LennardJones.hpp:135-206: one task per local atom, register
     * i-force, atomic j-force (atomic_access_slice), energy/virial reduce. */
    double* pos = atoms->pos;
    double* force = atoms->force;
    const int64_t* type = atoms->type;
    const int64_t n = atoms->numLocal;
    double energy = 0.0, virial = 0.0;
    const int usePred = (pred != NULL && pred->kind != ORC_PRED_ALWAYS);

#pragma omp parallel for schedule(static) reduction(+ : energy, virial) if (g_threads > 1)
    for (int64_t idx = 0; idx < n; ++idx)
    {
        double posTmp[3] = {pos[3 * idx + 0], pos[3 * idx + 1], pos[3 * idx + 2]};
        double forceTmp[3] = {0.0, 0.0, 0.0};
        const int64_t numNeighbors = counts[idx];
        for (int64_t k = 0; k < numNeighbors; ++k)
        {
            int64_t jdx = nbrs[idx * cap + k];
            const double* pj = &pos[3 * jdx];
            if (usePred &&
                !orc_pred_eval2(pred, posTmp[0], posTmp[1], posTmp[2], pj[0], pj[1], pj[2]))
                continue;
            double dx = posTmp[0] - pj[0];
            double dy = posTmp[1] - pj[1];
            double dz = posTmp[2] - pj[2];
            double distSqr = dx * dx + dy * dy + dz * dz;
            if (distSqr > rcSqr) continue;
            int64_t typeIdx = type[idx] * numTypesIndex + type[jdx];
            double ff, e;
            orc_lj_force_energy(table, distSqr, typeIdx, &ff, &e);
            energy += e;
            virial -= 0.5 * ff * distSqr;
            forceTmp[0] += dx * ff;
            forceTmp[1] += dy * ff;
            forceTmp[2] += dz * ff;
            double fjx = dx * ff, fjy = dy * ff, fjz = dz * ff;
#pragma omp atomic
            force[3 * jdx + 0] -= fjx;
#pragma omp atomic
            force[3 * jdx + 1] -= fjy;
#pragma omp atomic
            force[3 * jdx + 2] -= fjz;
        }
#pragma omp atomic
        force[3 * idx + 0] += forceTmp[0];
#pragma omp atomic
        force[3 * idx + 1] += forceTmp[1];
#pragma omp atomic
        force[3 * idx + 2] += forceTmp[2];
    }
    *energyOut = energy;
    *virialOut = virial;
}

/* -------------------------------------------------------- Coulomb DSF --- */

#define ORC_INV_SQRTPI 0.56418958354775628695 /* 1 / sqrt(pi) */
#define ORC_COULOMB_PREFACTOR 138.935458       /* CoulombDSF.hpp:57 */

double orc_approx_erfc(double x, double* expX2)
{
    /* util/math.hpp:57-70: erfc(x) ~ t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-x^2),
     * t = 1 / (1 + p x) (Abramowitz & Stegun 7.1.26) */
    const double p = 0.3275911;
    const double a1 = 0.254829592;
    const double a2 = -0.284496736;
    const double a3 = 1.421413741;
    const double a4 = -1.453152027;
    const double a5 = 1.061405429;
    double t = 1.0 / (1.0 + p * x);
    *expX2 = exp(-x * x);
    return t * (a1 + t * (a2 + t * (a3 + t * (a4 + t * a5)))) * *expX2;
}

void orc_coulomb_dsf_init(orc_coulomb_dsf* c, double rc, double alpha)
{
    /* CoulombDSF.hpp:76-83 (exact erfc for the shifts) */
    c->alpha = alpha;
    c->rc = rc;
    c->rcSqr = rc * rc;
    double e = erfc(alpha * rc);
    double x = exp(-alpha * alpha * c->rcSqr);
    c->forceShift = -(e / c->rcSqr + 2.0 * ORC_INV_SQRTPI * alpha * x / rc);
    c->energyShift = e / rc;
}

double orc_coulomb_dsf_force(const orc_coulomb_dsf* c, double distSqr, double q1, double q2)
{
    /* CoulombDSF.hpp:52-62 (eq 16), divided by r^2 as the reference returns it */
    double r = sqrt(distSqr);
    double prefac = ORC_COULOMB_PREFACTOR * q1 * q2;
    double expX2;
    double e = orc_approx_erfc(c->alpha * r, &expX2);
    double force = prefac * (e / r + 2.0 * c->alpha * ORC_INV_SQRTPI * expX2 + r * c->forceShift);
    return force / distSqr;
}

double orc_coulomb_dsf_energy(const orc_coulomb_dsf* c, double distSqr, double q1, double q2)
{
    /* CoulombDSF.hpp:64-74 (eq 15) */
    double r = sqrt(distSqr);
    double prefac = ORC_COULOMB_PREFACTOR * q1 * q2;
    double expX2;
    double e = orc_approx_erfc(c->alpha * r, &expX2);
    return prefac * (e / r - c->energyShift - c->forceShift * (r - c->rc));
}

void orc_coulomb_dsf_apply(const orc_coulomb_dsf* c, orc_atoms* atoms, const int32_t* counts,
                           const int32_t* nbrs, int64_t cap, double* energyOut, double* virialOut)
{
    double* pos = atoms->pos;
    double* force = atoms->force;
    const double* q = atoms->charge;
    double energy = 0.0, virial = 0.0;
    for (int64_t idx = 0; idx < atoms->numLocal; ++idx)
    {
        double forceTmp[3] = {0.0, 0.0, 0.0};
        for (int64_t k = 0; k < counts[idx]; ++k)
        {
            int64_t jdx = nbrs[idx * cap + k];
            double dx = pos[3 * idx + 0] - pos[3 * jdx + 0];
            double dy = pos[3 * idx + 1] - pos[3 * jdx + 1];
            double dz = pos[3 * idx + 2] - pos[3 * jdx + 2];
            double distSqr = dx * dx + dy * dy + dz * dz;
            if (distSqr > c->rcSqr) continue;
            double ff = orc_coulomb_dsf_force(c, distSqr, q[idx], q[jdx]);
            energy += orc_coulomb_dsf_energy(c, distSqr, q[idx], q[jdx]);
            virial -= 0.5 * ff * distSqr;
            forceTmp[0] += dx * ff;
            forceTmp[1] += dy * ff;
            forceTmp[2] += dz * ff;
            force[3 * jdx + 0] -= dx * ff;
            force[3 * jdx + 1] -= dy * ff;
            force[3 * jdx + 2] -= dz * ff;
        }
        force[3 * idx + 0] += forceTmp[0];
        force[3 * idx + 1] += forceTmp[1];
        force[3 * idx + 2] += forceTmp[2];
    }
    *energyOut = energy;
    *virialOut = virial;
}

/* -------------------------------------------------------- ghost layer --- */

void orc_map_into_domain(orc_atoms* atoms, const orc_subdomain* sd)
{
    /* communication/PeriodicMapping.cpp:30-58 */
    for (int64_t idx = 0; idx < atoms->numLocal; ++idx)
    {
        for (int dim = 0; dim < 3; ++dim)
        {
            double* x = &atoms->pos[3 * idx + dim];
            if (sd->maxCorner[dim] <= *x)
            {
                *x -= sd->diameter[dim];
                *x = fmax(*x, sd->minCorner[dim]);
            }
            if (*x < sd->minCorner[dim])
            {
                *x += sd->diameter[dim];
                if (sd->maxCorner[dim] <= *x) *x = sd->minCorner[dim];
            }
        }
    }
}

static void atoms_copy(orc_atoms* a, int64_t dst, int64_t src)
{
    /* data/Atoms.hpp:97-110 */
    for (int d = 0; d < 3; ++d)
    {
        a->pos[3 * dst + d] = a->pos[3 * src + d];
        a->vel[3 * dst + d] = a->vel[3 * src + d];
        a->force[3 * dst + d] = a->force[3 * src + d];
    }
    a->type[dst] = a->type[src];
    a->mass[dst] = a->mass[src];
    a->charge[dst] = a->charge[src];
    a->relativeMass[dst] = a->relativeMass[src];
}

/* Count (positive, negative) selections of one axis pass without writing. */
static void ghost_axis_counts(const orc_atoms* a, int64_t nAll, const orc_subdomain* sd, int axis,
                              int64_t* pos, int64_t* neg)
{
    int64_t p = 0, q = 0;
    for (int64_t idx = 0; idx < nAll; ++idx)
    {
        double x = a->pos[3 * idx + axis];
        if (x < sd->minInnerCorner[axis]) ++p;
        if (x >= sd->maxInnerCorner[axis]) ++q;
    }
    *pos = p;
    *neg = q;
}

/* Ghost count of a full XYZ pass, needed to check capacity up front.  Follows
 * the same selection rules as the real pass (positions of earlier ghosts
 * are shifted exactly as they will be). */
static int64_t ghost_total_needed(const orc_atoms* a, const orc_subdomain* sd)
{
    int64_t n = a->numLocal;
    /* simulate on a scratch copy of positions */
    double* p = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1) * 27);
    int64_t capScratch = n * 27;
    memcpy(p, a->pos, sizeof(double) * 3 * (size_t)n);
    int64_t cur = n;
    for (int axis = 0; axis < 3; ++axis)
    {
        int64_t add = cur;
        int64_t np = 0;
        /* positives then negatives, as the real pass */
        for (int64_t idx = 0; idx < cur; ++idx)
            if (p[3 * idx + axis] < sd->minInnerCorner[axis])
            {
                if (add >= capScratch) break;
                memcpy(&p[3 * add], &p[3 * idx], 3 * sizeof(double));
                p[3 * add + axis] += sd->diameter[axis];
                ++add;
                ++np;
            }
        for (int64_t idx = 0; idx < cur; ++idx)
            if (p[3 * idx + axis] >= sd->maxInnerCorner[axis])
            {
                if (add >= capScratch) break;
                memcpy(&p[3 * add], &p[3 * idx], 3 * sizeof(double));
                p[3 * add + axis] -= sd->diameter[axis];
                ++add;
            }
        (void)np;
        cur = add;
    }
    free(p);
    return cur;
}

int64_t orc_create_ghosts_xyz(orc_atoms* a, const orc_subdomain* sd, int64_t* corr)
{
    /* communication/GhostExchange.cpp:171-187 then createGhostAtoms :59-169 per axis */
    int64_t needed = ghost_total_needed(a, sd);
    if (needed > a->capacity) return needed;

    for (int64_t i = 0; i < a->capacity; ++i) corr[i] = -1;
    a->numGhost = 0;
    for (int axis = 0; axis < 3; ++axis)
    {
        int64_t nAll = a->numLocal + a->numGhost;
        int64_t np, nn;
        ghost_axis_counts(a, nAll, sd, axis, &np, &nn);
        /* parallel_scan order: selections keep increasing source index */
        int64_t k = 0;
        for (int64_t idx = 0; idx < nAll; ++idx)
        {
            if (a->pos[3 * idx + axis] < sd->minInnerCorner[axis])
            {
                int64_t dst = nAll + k++;
                atoms_copy(a, dst, idx);
                a->pos[3 * dst + axis] += sd->diameter[axis];
                int64_t realIdx = idx;
                while (corr[realIdx] != -1) realIdx = corr[realIdx];
                corr[dst] = realIdx;
            }
        }
        k = 0;
        for (int64_t idx = 0; idx < nAll; ++idx)
        {
            if (a->pos[3 * idx + axis] >= sd->maxInnerCorner[axis])
            {
                int64_t dst = nAll + np + k++;
                atoms_copy(a, dst, idx);
                a->pos[3 * dst + axis] -= sd->diameter[axis];
                int64_t realIdx = idx;
                while (corr[realIdx] != -1) realIdx = corr[realIdx];
                corr[dst] = realIdx;
            }
        }
        a->numGhost += np + nn;
    }
    return 0;
}

void orc_update_ghosts(orc_atoms* a, const int64_t* corr, const orc_subdomain* sd)
{
    /* communication/UpdateGhostAtoms.cpp:31-68 */
    double* pos = a->pos;
    for (int64_t idx = a->numLocal; idx < a->numLocal + a->numGhost; ++idx)
    {
        int64_t realIdx = corr[idx];
        double dx[3];
        for (int d = 0; d < 3; ++d) dx[d] = pos[3 * idx + d] - pos[3 * realIdx + d];
        for (int d = 0; d < 3; ++d) pos[3 * idx + d] = pos[3 * realIdx + d];
        double delta[3];
        for (int d = 0; d < 3; ++d) delta[d] = 0.1 * sd->diameter[d];
        for (int d = 0; d < 3; ++d)
            if (dx[d] > +delta[d]) pos[3 * idx + d] += sd->diameter[d];
        for (int d = 0; d < 3; ++d)
            if (dx[d] < -delta[d]) pos[3 * idx + d] -= sd->diameter[d];
    }
}

void orc_ghost_to_real(orc_atoms* a, const int64_t* corr)
{
    /* communication/AccumulateForce.cpp:25-47 (serial order of ghost index) */
    for (int64_t idx = a->numLocal; idx < a->numLocal + a->numGhost; ++idx)
    {
        if (corr[idx] == -1) continue;
        int64_t realIdx = corr[idx];
        for (int d = 0; d < 3; ++d)
        {
            a->force[3 * realIdx + d] += a->force[3 * idx + d];
            a->force[3 * idx + d] = 0.0;
        }
    }
}

/* ------------------------------------------------ cells + Verlet list --- */

void orc_cell_grid(const double* gridMin, const double* gridMax, double delta, int64_t* nCells,
                   double* rdx)
{
    for (int d = 0; d < 3; ++d)
    {
        double L = gridMax[d] - gridMin[d];
        int64_t n = (int64_t)floor(L / delta);
        if (n < 1) n = 1;
        nCells[d] = n;
        rdx[d] = (double)n / L;
    }
}

static inline int64_t cell_coord(double x, double mn, double rdx, int64_t n)
{
    int64_t c = (int64_t)floor((x - mn) * rdx);
    if (c < 0) c = 0;
    if (c > n - 1) c = n - 1;
    return c;
}

void orc_cell_index(const double* pos, int64_t n, const double* gridMin, const int64_t* nCells,
                    const double* rdx, int64_t* cellOut)
{
    for (int64_t i = 0; i < n; ++i)
    {
        int64_t cx = cell_coord(pos[3 * i + 0], gridMin[0], rdx[0], nCells[0]);
        int64_t cy = cell_coord(pos[3 * i + 1], gridMin[1], rdx[1], nCells[1]);
        int64_t cz = cell_coord(pos[3 * i + 2], gridMin[2], rdx[2], nCells[2]);
        cellOut[i] = (cx * nCells[1] + cy) * nCells[2] + cz;
    }
}

static inline int lex_above(const double* pi, const double* pj)
{
    /* Cabana 0.7 NeighborDiscriminator<HalfNeighborTag>::isValid: keep the
     * neighbour when it is spatially "higher" in (x, y, z) order. */
    return (pj[0] > pi[0]) ||
           ((pj[0] == pi[0]) && ((pj[1] > pi[1]) || ((pj[1] == pi[1]) && (pj[2] > pi[2]))));
}

int64_t orc_build_half_list(const double* pos, int64_t n, int64_t begin, int64_t end,
                            double rlist, double cellRatio, const double* gridMin,
                            const double* gridMax, int32_t* counts, int32_t* nbrs, int64_t cap)
{
    int64_t nc[3];
    double rdx[3];
    orc_cell_grid(gridMin, gridMax, rlist * cellRatio, nc, rdx);
    int64_t ncell = nc[0] * nc[1] * nc[2];
    int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t* start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t* sorted = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    orc_cell_index(pos, n, gridMin, nc, rdx, cell);
    for (int64_t i = 0; i < n; ++i) start[cell[i] + 1]++;
    for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
    {
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
        memcpy(fill, start, sizeof(int64_t) * (size_t)ncell);
        for (int64_t i = 0; i < n; ++i) sorted[fill[cell[i]]++] = i; /* stable by index */
        free(fill);
    }
    /* stencil reach in cells: ceil(rlist / edge) */
    int64_t reach[3];
    for (int d = 0; d < 3; ++d)
    {
        double edge = 1.0 / rdx[d];
        reach[d] = (int64_t)ceil(rlist / edge);
        if (reach[d] < 1) reach[d] = 1;
    }
    const double rsq = rlist * rlist;
    int64_t maxCount = 0;

#pragma omp parallel for schedule(dynamic, 256) reduction(max : maxCount) if (g_threads > 1)
    for (int64_t i = begin; i < end; ++i)
    {
        const double* pi = &pos[3 * i];
        int64_t ci = cell[i];
        int64_t cz = ci % nc[2];
        int64_t cy = (ci / nc[2]) % nc[1];
        int64_t cx = ci / (nc[1] * nc[2]);
        int64_t cnt = 0;
        for (int64_t ax = cx - reach[0]; ax <= cx + reach[0]; ++ax)
        {
            if (ax < 0 || ax >= nc[0]) continue;
            for (int64_t ay = cy - reach[1]; ay <= cy + reach[1]; ++ay)
            {
                if (ay < 0 || ay >= nc[1]) continue;
                for (int64_t az = cz - reach[2]; az <= cz + reach[2]; ++az)
                {
                    if (az < 0 || az >= nc[2]) continue;
                    int64_t c = (ax * nc[1] + ay) * nc[2] + az;
                    for (int64_t s = start[c]; s < start[c + 1]; ++s)
                    {
                        int64_t j = sorted[s];
                        if (j == i) continue;
                        const double* pj = &pos[3 * j];
                        double dx = pi[0] - pj[0];
                        double dy = pi[1] - pj[1];
                        double dz = pi[2] - pj[2];
                        double d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 > rsq) continue;
                        if (!lex_above(pi, pj)) continue;
                        if (cnt < cap) nbrs[(i - begin) * cap + cnt] = (int32_t)j;
                        ++cnt;
                    }
                }
            }
        }
        counts[i - begin] = (int32_t)(cnt < cap ? cnt : cap);
        if (cnt > maxCount) maxCount = cnt;
    }
    free(cell);
    free(start);
    free(sorted);
    return maxCount;
}

int64_t orc_count_within(const double* pos, int64_t nLocal, int64_t nAll, double cutoff,
                         const double* box, int periodic)
{
    /* tests/LennardJones/LennardJones.cpp:40-70 */
    double rcSqr = cutoff * cutoff;
    int64_t count = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : count) if (g_threads > 1)
    for (int64_t idx = 0; idx < nLocal; ++idx)
    {
        for (int64_t jdx = idx + 1; jdx < nAll; ++jdx)
        {
            double dx = fabs(pos[3 * idx + 0] - pos[3 * jdx + 0]);
            if (periodic && (dx > box[0] * 0.5)) dx -= box[0];
            double dy = fabs(pos[3 * idx + 1] - pos[3 * jdx + 1]);
            if (periodic && (dy > box[1] * 0.5)) dy -= box[1];
            double dz = fabs(pos[3 * idx + 2] - pos[3 * jdx + 2]);
            if (periodic && (dz > box[2] * 0.5)) dz -= box[2];
            double distSqr = dx * dx + dy * dy + dz * dz;
            if (distSqr < rcSqr) ++count;
        }
    }
    return count;
}

/* -------------------------------------------------------- integrators --- */

double orc_vv_pre(orc_atoms* a, double dt)
{
    /* action/VelocityVerlet.cpp:26-67, updateKick/updateDrift UpdateSteps.hpp:25-54 */
    double dtHalf = 0.5 * dt;
    double dtFull = dt;
    double maxDistSqr = 0.0;
#pragma omp parallel for schedule(static) reduction(max : maxDistSqr) if (g_threads > 1)
    for (int64_t idx = 0; idx < a->numLocal; ++idx)
    {
        double* x = &a->pos[3 * idx];
        double* v = &a->vel[3 * idx];
        const double* f = &a->force[3 * idx];
        double dx[3] = {x[0], x[1], x[2]};
        double dtfm = dtHalf / a->mass[idx];
        v[0] += dtfm * f[0];
        v[1] += dtfm * f[1];
        v[2] += dtfm * f[2];
        x[0] += dtFull * v[0];
        x[1] += dtFull * v[1];
        x[2] += dtFull * v[2];
        dx[0] -= x[0];
        dx[1] -= x[1];
        dx[2] -= x[2];
        double distSqr = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (distSqr > maxDistSqr) maxDistSqr = distSqr;
    }
    return sqrt(maxDistSqr);
}

void orc_vv_post(orc_atoms* a, double dt)
{
    /* action/VelocityVerlet.cpp:69-90 */
    double dtHalf = 0.5 * dt;
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (int64_t idx = 0; idx < a->numLocal; ++idx)
    {
        double* v = &a->vel[3 * idx];
        const double* f = &a->force[3 * idx];
        double dtfm = dtHalf / a->mass[idx];
        v[0] += dtfm * f[0];
        v[1] += dtfm * f[1];
        v[2] += dtfm * f[2];
    }
}

double orc_kinetic_energy(const orc_atoms* a)
{
    /* analysis/KineticEnergy.hpp:26-39 */
    double velSqr = 0.0;
    for (int64_t idx = 0; idx < a->numLocal; ++idx)
    {
        const double* v = &a->vel[3 * idx];
        velSqr += a->mass[idx] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    return 0.5 * velSqr;
}

void orc_system_momentum(const orc_atoms* a, double* out3)
{
    /* analysis/SystemMomentum.cpp:21-48: one reduction per component */
    for (int d = 0; d < 3; ++d)
    {
        double sum = 0.0;
        for (int64_t idx = 0; idx < a->numLocal; ++idx) sum += a->vel[3 * idx + d];
        out3[d] = sum;
    }
}

double orc_pressure(const orc_atoms* a, const orc_subdomain* sd)
{
    /* analysis/Pressure.cpp:23-51 */
    double pressure = 0.0;
    for (int64_t idx = 0; idx < a->numLocal + a->numGhost; ++idx)
    {
        const double* v = &a->vel[3 * idx];
        const double* x = &a->pos[3 * idx];
        const double* F = &a->force[3 * idx];
        pressure += a->mass[idx] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        pressure += F[0] * x[0] + F[1] * x[1] + F[2] * x[2];
    }
    const double volume = sd->diameter[0] * sd->diameter[1] * sd->diameter[2];
    return pressure / (3.0 * volume);
}

/* Philox4x32-10 as published by Salmon et al., "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11: multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key
 * increments 0x9E3779B9 / 0xBB67AE85. */
void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out)
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r)
    {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Box-Muller in FP32 with our own ln and sin/cos (the GPU's normal3 in
 * mrmd_gb300/csrc/integrate_impl.cuh, operation for operation): ln(u) =
 * e ln2 + 2 atanh(t), t = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)]; sin/cos of
 * 2 pi u by a quarter-turn reduction and Taylor polynomials on [-pi/4, pi/4].
 * Every step is a correctly rounded float operation or fmaf, so host and
 * device agree bit for bit (the file is built with -ffp-contract=off). */
static float bm_log(float u)
{
    uint32_t bits;
    memcpy(&bits, &u, sizeof bits);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    uint32_t mb = (bits & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, sizeof m);
    if (m > 0x1.6a09e6p+0f)
    {
        m = m * 0.5f;
        e += 1;
    }
    const float t = (m - 1.0f) / (m + 1.0f);
    const float t2 = t * t;
    float p = fmaf(t2, 0x1.c71c72p-4f, 0x1.24924ap-3f);
    p = fmaf(p, t2, 0x1.99999ap-3f);
    p = fmaf(p, t2, 0x1.555556p-2f);
    p = fmaf(p, t2, 1.0f);
    return fmaf((float)e, 0x1.62e430p-1f, 2.0f * (t * p));
}

static void bm_sincos(float u, float* c, float* s)
{
    const float q = rintf(4.0f * u);
    const float x = u - 0.25f * q;
    const float f = x * 0x1.921fb6p+2f;
    const float f2 = f * f;
    float ps = fmaf(f2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = fmaf(ps, f2, 0x1.111112p-7f);
    ps = fmaf(ps, f2, -0x1.555556p-3f);
    const float sn = fmaf(f * f2, ps, f);
    float pc = fmaf(f2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = fmaf(pc, f2, -0x1.6c16c2p-10f);
    pc = fmaf(pc, f2, 0x1.555556p-5f);
    pc = fmaf(pc, f2, -0.5f);
    const float cs = fmaf(pc, f2, 1.0f);
    const int quadrant = ((int)q) & 3;
    *c = quadrant == 0 ? cs : (quadrant == 1 ? -sn : (quadrant == 2 ? -cs : sn));
    *s = quadrant == 0 ? sn : (quadrant == 1 ? cs : (quadrant == 2 ? -sn : -cs));
}

void orc_normal_from_counter(uint64_t seed, uint64_t step, uint64_t atom, double* out3)
{
    uint32_t ctr[4] = {(uint32_t)atom, (uint32_t)(atom >> 32), (uint32_t)step,
                       (uint32_t)(step >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t r[4];
    orc_philox4x32_10(ctr, key, r);
    /* 23-bit uniforms in (0,1), then two Box-Muller pairs */
    float u[4];
    for (int k = 0; k < 4; ++k) u[k] = ((float)(r[k] >> 9) + 0.5f) * 0x1p-23f;
    const float ra = sqrtf(-2.0f * bm_log(u[0]));
    const float rb = sqrtf(-2.0f * bm_log(u[2]));
    float ca, sa, cb, sb;
    bm_sincos(u[1], &ca, &sa);
    bm_sincos(u[3], &cb, &sb);
    out3[0] = (double)(ra * ca);
    out3[1] = (double)(ra * sa);
    out3[2] = (double)(rb * cb);
}

double orc_langevin_pre(orc_atoms* a, double dt, double zeta, double temperature, uint64_t seed,
                        uint64_t step, const orc_pred* pred)
{
    /* action/VelocityVerletLangevinThermostat.hpp:48-121; updateOrnsteinUhlenbeck
     * UpdateSteps.hpp:56-79 */
    double dtHalf = 0.5 * dt;
    double dtFull = dt;
    double maxDistSqr = 0.0;
#pragma omp parallel for schedule(static) reduction(max : maxDistSqr) if (g_threads > 1)
    for (int64_t idx = 0; idx < a->numLocal; ++idx)
    {
        double* x = &a->pos[3 * idx];
        double* v = &a->vel[3 * idx];
        const double* f = &a->force[3 * idx];
        double m = a->mass[idx];
        double dx[3] = {x[0], x[1], x[2]};
        double dtfm = dtHalf / m;
        v[0] += dtfm * f[0];
        v[1] += dtfm * f[1];
        v[2] += dtfm * f[2];
        x[0] += dtHalf * v[0];
        x[1] += dtHalf * v[1];
        x[2] += dtHalf * v[2];
        if (orc_pred_eval1(pred, x[0], x[1], x[2]))
        {
            double g[3];
            orc_normal_from_counter(seed, step, (uint64_t)idx, g);
            double dtm = dtFull / m;
            double damping = exp(-zeta * dtm);
            double sigma = sqrt(temperature / m * (1.0 - exp(-2.0 * zeta * dtm)));
            v[0] *= damping;
            v[1] *= damping;
            v[2] *= damping;
            v[0] += sigma * g[0];
            v[1] += sigma * g[1];
            v[2] += sigma * g[2];
        }
        x[0] += dtHalf * v[0];
        x[1] += dtHalf * v[1];
        x[2] += dtHalf * v[2];
        dx[0] -= x[0];
        dx[1] -= x[1];
        dx[2] -= x[2];
        double distSqr = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        if (distSqr > maxDistSqr) maxDistSqr = distSqr;
    }
    return sqrt(maxDistSqr);
}

/* ------------------------------------------------------------- AdResS --- */

void orc_slab_init(orc_slab* s, const double* center, double atomisticRegionDiameter,
                   double hybridRegionDiameter, int64_t nu, int32_t interfaceType)
{
    /* weighting_function/Slab.hpp:189-200 */
    s->center[0] = center[0];
    s->center[1] = center[1];
    s->center[2] = center[2];
    s->atomisticRegionHalfDiameter = 0.5 * atomisticRegionDiameter;
    s->hybridRegionDiameter = hybridRegionDiameter;
    s->exponent = 2 * nu;
    s->interfaceType = interfaceType;
    s->pad = 0;
}

static double pow_int(double x, int64_t n)
{
    /* util/math.hpp:31-46 */
    double ww = x;
    double yy = 1.0;
    for (int64_t nn = (n > 0) ? n : -n; nn != 0; nn >>= 1)
    {
        if ((nn & 1) == 1) yy *= ww;
        ww *= ww;
    }
    return (n > 0) ? yy : 1.0 / yy;
}

void orc_slab_eval(const orc_slab* s, double x, double y, double z, double* out)
{
    /* Slab::operator(), weighting_function/Slab.hpp:161-187; out = {lambda,
     * modulatedLambda, gradX, gradY, gradZ} */
    (void)y;
    (void)z;
    const double pi = 3.141592653589793238462643383279502884;
    double dx = x - s->center[0];
    double absDx = fabs(dx);
    if (absDx < s->atomisticRegionHalfDiameter)
    {
        out[0] = 1.0;
        out[1] = 1.0;
        out[2] = out[3] = out[4] = 0.0;
    }
    else if (absDx > s->atomisticRegionHalfDiameter + s->hybridRegionDiameter)
    {
        out[0] = out[1] = 0.0;
        out[2] = out[3] = out[4] = 0.0;
    }
    else if (s->interfaceType == 1)
    {
        out[0] = 1.0;
        out[1] = 1.0;
        out[2] = out[3] = out[4] = 0.0;
    }
    else
    {
        /* setSmoothWeightInHY, Slab.hpp:96-120 */
        double arg = pi / (2.0 * s->hybridRegionDiameter) * (absDx - s->atomisticRegionHalfDiameter);
        double base = cos(arg);
        out[0] = base * base;
        out[1] = pow_int(base, s->exponent);
        double factor = -pi / (2.0 * s->hybridRegionDiameter) * (double)s->exponent * sin(arg) *
                        pow_int(base, s->exponent - 1) / absDx;
        out[2] = factor * dx;
        out[3] = 0.0;
        out[4] = 0.0;
    }
}

void orc_update_molecules(orc_molecules* mol, const orc_atoms* atoms, const orc_slab* slab)
{
    /* action/UpdateMolecules.hpp:39-69 */
    for (int64_t m = 0; m < mol->numLocal + mol->numGhost; ++m)
    {
        int64_t s = mol->atomsOffset[m], e = s + mol->numAtoms[m];
        double* p = &mol->pos[3 * m];
        p[0] = p[1] = p[2] = 0.0;
        for (int64_t a = s; a < e; ++a)
        {
            p[0] += atoms->pos[3 * a + 0] * atoms->relativeMass[a];
            p[1] += atoms->pos[3 * a + 1] * atoms->relativeMass[a];
            p[2] += atoms->pos[3 * a + 2] * atoms->relativeMass[a];
        }
        double w[5];
        orc_slab_eval(slab, p[0], p[1], p[2], w);
        mol->lambda[m] = w[0];
        mol->modulatedLambda[m] = w[1];
        mol->gradLambda[3 * m + 0] = w[2];
        mol->gradLambda[3 * m + 1] = w[3];
        mol->gradLambda[3 * m + 2] = w[4];
    }
}

void orc_contribute_molecule_force(const orc_molecules* mol, orc_atoms* atoms)
{
    /* action/ContributeMoleculeForceToAtoms.cpp:23-48 */
    for (int64_t m = 0; m < mol->numLocal + mol->numGhost; ++m)
    {
        int64_t s = mol->atomsOffset[m], e = s + mol->numAtoms[m];
        for (int64_t a = s; a < e; ++a)
            for (int d = 0; d < 3; ++d)
                atoms->force[3 * a + d] += atoms->relativeMass[a] * mol->force[3 * m + d];
    }
}

/* CheckRegion.hpp:25-38 with REGION_CHECK_EPSILON = 0 */
static inline int is_at(double l) { return l >= 1.0; }
static inline int is_cg(double l) { return l <= 0.0; }
static inline int is_hy(double l) { return !is_at(l) && !is_cg(l); }

static inline int64_t comp_bin(double lambda)
{
    /* MultiHistogram(0,1,200).getBin, data/MultiHistogram.hpp:60-66 */
    const double binSize = (1.0 - 0.0) / (double)ORC_LJIG_BINS;
    const double inv = 1.0 / binSize;
    int64_t bin = (int64_t)floor((lambda - 0.0) * inv);
    if (bin < 0) bin = -1;
    if (bin >= ORC_LJIG_BINS) bin = -1;
    return bin;
}

void orc_update_mean_compensation_energy(double* energy, double* counter, double* mean,
                                         int64_t numBins, int64_t numHist, double factor)
{
    /* action/LJ_IdealGas.cpp:21-50 */
    for (int64_t b = 0; b < numBins; ++b)
        for (int64_t h = 0; h < numHist; ++h)
        {
            int64_t k = b * numHist + h;
            if (counter[k] < 0.5) continue;
            double e = energy[k] / counter[k];
            mean[k] = (factor * mean[k] + e) / (factor + 1.0);
            energy[k] = 0.0;
            counter[k] = 0.0;
        }
}

double orc_ljig_run(orc_ljig* s, orc_molecules* mol, const int32_t* counts, const int32_t* nbrs,
                    int64_t cap, orc_atoms* atoms)
{
    /* action/LJ_IdealGas.cpp:227-260 with the molecule functor :52-225 */
    const int sampling = (s->runCounter % s->samplingInterval) == 0;
    const int64_t nt = s->numTypes;
    double* apos = atoms->pos;
    double* afor = atoms->force;
    const int64_t* atype = atoms->type;
    double sumEnergy = 0.0;

    /* one task per local molecule (parallel_reduce); shared updates are
     * atomic as the reference's atomic_access_slice / ScatterView */
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : sumEnergy) if (g_threads > 1)
    for (int64_t alpha = 0; alpha < mol->numLocal; ++alpha)
    {
        double forceTmpAlpha[3] = {0.0, 0.0, 0.0};
        const double modLamA = mol->modulatedLambda[alpha];
        int64_t binAlpha = -1;
        if (is_hy(modLamA)) binAlpha = comp_bin(mol->lambda[alpha]);
        const double gA[3] = {mol->gradLambda[3 * alpha + 0], mol->gradLambda[3 * alpha + 1],
                              mol->gradLambda[3 * alpha + 2]};
        const int64_t sA = mol->atomsOffset[alpha];
        const int64_t eA = sA + mol->numAtoms[alpha];
        const int64_t numNeighbors = counts[alpha];
        for (int64_t k = 0; k < numNeighbors; ++k)
        {
            const int64_t beta = nbrs[alpha * cap + k];
            double forceTmpBeta[3] = {0.0, 0.0, 0.0};
            const double modLamB = mol->modulatedLambda[beta];
            const double gB[3] = {mol->gradLambda[3 * beta + 0], mol->gradLambda[3 * beta + 1],
                                  mol->gradLambda[3 * beta + 2]};
            const double weighting = 0.5 * (modLamA + modLamB);
            if (is_cg(modLamA) && is_cg(modLamB)) continue;
            const int64_t sB = mol->atomsOffset[beta];
            const int64_t eB = sB + mol->numAtoms[beta];
            for (int64_t idx = sA; idx < eA; ++idx)
            {
                double posTmp[3] = {apos[3 * idx + 0], apos[3 * idx + 1], apos[3 * idx + 2]};
                double forceTmpIdx[3] = {0.0, 0.0, 0.0};
                for (int64_t jdx = sB; jdx < eB; ++jdx)
                {
                    const double dx = posTmp[0] - apos[3 * jdx + 0];
                    const double dy = posTmp[1] - apos[3 * jdx + 1];
                    const double dz = posTmp[2] - apos[3 * jdx + 2];
                    const double distSqr = dx * dx + dy * dy + dz * dz;
                    if (distSqr > s->rcSqr) continue;
                    int64_t typeIdx = atype[idx] * nt + atype[jdx];
                    double ff, e;
                    orc_lj_force_energy(s->table, distSqr, typeIdx, &ff, &e);
                    double ffactor = ff * weighting;
                    forceTmpIdx[0] += dx * ffactor;
                    forceTmpIdx[1] += dy * ffactor;
                    forceTmpIdx[2] += dz * ffactor;
                    const double fjx = dx * ffactor, fjy = dy * ffactor, fjz = dz * ffactor;
#pragma omp atomic
                    afor[3 * jdx + 0] -= fjx;
#pragma omp atomic
                    afor[3 * jdx + 1] -= fjy;
#pragma omp atomic
                    afor[3 * jdx + 2] -= fjz;
                    sumEnergy += e * weighting;
                    double Vij = 0.5 * e;
                    if (is_hy(modLamA) || is_hy(modLamB))
                    {
                        forceTmpAlpha[0] += -Vij * gA[0];
                        forceTmpAlpha[1] += -Vij * gA[1];
                        forceTmpAlpha[2] += -Vij * gA[2];
                        forceTmpBeta[0] += -Vij * gB[0];
                        forceTmpBeta[1] += -Vij * gB[1];
                        forceTmpBeta[2] += -Vij * gB[2];
                        if (sampling)
                        {
                            int64_t binBeta = -1;
                            if (is_hy(modLamB)) binBeta = comp_bin(mol->lambda[beta]);
                            if (is_hy(modLamA) && binAlpha != -1)
                            {
#pragma omp atomic
                                s->compensationEnergy[binAlpha * nt + atype[idx]] += Vij;
                            }
                            if (is_hy(modLamB) && binBeta != -1)
                            {
#pragma omp atomic
                                s->compensationEnergy[binBeta * nt + atype[jdx]] += Vij;
                            }
                        }
                    }
                }
#pragma omp atomic
                afor[3 * idx + 0] += forceTmpIdx[0];
#pragma omp atomic
                afor[3 * idx + 1] += forceTmpIdx[1];
#pragma omp atomic
                afor[3 * idx + 2] += forceTmpIdx[2];
            }
#pragma omp atomic
            mol->force[3 * beta + 0] += forceTmpBeta[0];
#pragma omp atomic
            mol->force[3 * beta + 1] += forceTmpBeta[1];
#pragma omp atomic
            mol->force[3 * beta + 2] += forceTmpBeta[2];
        }
        if (sampling)
        {
            for (int64_t a = sA; a < eA; ++a)
                if (is_hy(modLamA) && binAlpha != -1)
                {
#pragma omp atomic
                    s->compensationEnergyCounter[binAlpha * nt + atype[a]] += 1.0;
                }
        }
        if (is_hy(modLamA) && binAlpha != -1)
        {
            double me = s->meanCompensationEnergy[binAlpha * nt + atype[sA]];
            forceTmpAlpha[0] += me * gA[0];
            forceTmpAlpha[1] += me * gA[1];
            forceTmpAlpha[2] += me * gA[2];
        }
#pragma omp atomic
        mol->force[3 * alpha + 0] += forceTmpAlpha[0];
#pragma omp atomic
        mol->force[3 * alpha + 1] += forceTmpAlpha[1];
#pragma omp atomic
        mol->force[3 * alpha + 2] += forceTmpAlpha[2];
    }

    if (s->runCounter % s->updateInterval == 0)
        orc_update_mean_compensation_energy(s->compensationEnergy, s->compensationEnergyCounter,
                                            s->meanCompensationEnergy, ORC_LJIG_BINS, nt, 10.0);
    ++s->runCounter;
    return sumEnergy;
}

void orc_multires_map_into_domain(const orc_subdomain* sd, orc_molecules* mol, orc_atoms* atoms)
{
    /* communication/MultiResRealAtomsExchange.cpp:23-73 */
    for (int64_t m = 0; m < mol->numLocal; ++m)
    {
        for (int dim = 0; dim < 3; ++dim)
        {
            double* mx = &mol->pos[3 * m + dim];
            int64_t s = mol->atomsOffset[m], e = s + mol->numAtoms[m];
            if (sd->maxCorner[dim] <= *mx)
            {
                *mx -= sd->diameter[dim];
                for (int64_t a = s; a < e; ++a) atoms->pos[3 * a + dim] -= sd->diameter[dim];
            }
            if (*mx < sd->minCorner[dim])
            {
                *mx += sd->diameter[dim];
                for (int64_t a = s; a < e; ++a) atoms->pos[3 * a + dim] += sd->diameter[dim];
            }
        }
    }
}

static void molecules_copy(orc_molecules* m, int64_t dst, int64_t src)
{
    /* data/Molecules.hpp:97-110 */
    for (int d = 0; d < 3; ++d)
    {
        m->pos[3 * dst + d] = m->pos[3 * src + d];
        m->force[3 * dst + d] = m->force[3 * src + d];
        m->gradLambda[3 * dst + d] = m->gradLambda[3 * src + d];
    }
    m->lambda[dst] = m->lambda[src];
    m->modulatedLambda[dst] = m->modulatedLambda[src];
    m->atomsOffset[dst] = m->atomsOffset[src];
    m->numAtoms[dst] = m->numAtoms[src];
}

int64_t orc_multires_create_ghosts_xyz(orc_molecules* mol, orc_atoms* atoms,
                                       const orc_subdomain* sd, int64_t* corr)
{
    /* communication/MultiResPeriodicGhostExchange.cpp:250-265 then :60-248 per axis */
    /* capacity check on molecule centres (atoms follow their molecule) */
    {
        int64_t nm = mol->numLocal, na = atoms->numLocal;
        double* mx = (double*)malloc(sizeof(double) * 3 * (size_t)(nm > 0 ? nm : 1) * 27);
        int64_t* mn = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nm > 0 ? nm : 1) * 27);
        memcpy(mx, mol->pos, sizeof(double) * 3 * (size_t)nm);
        memcpy(mn, mol->numAtoms, sizeof(int64_t) * (size_t)nm);
        int64_t cur = nm, curA = na;
        for (int axis = 0; axis < 3; ++axis)
        {
            int64_t add = cur;
            for (int64_t i = 0; i < cur && add < nm * 27; ++i)
                if (mx[3 * i + axis] >= sd->maxInnerCorner[axis])
                {
                    memcpy(&mx[3 * add], &mx[3 * i], 3 * sizeof(double));
                    mx[3 * add + axis] -= sd->diameter[axis];
                    mn[add] = mn[i];
                    curA += mn[i];
                    ++add;
                }
            for (int64_t i = 0; i < cur && add < nm * 27; ++i)
                if (mx[3 * i + axis] < sd->minInnerCorner[axis])
                {
                    memcpy(&mx[3 * add], &mx[3 * i], 3 * sizeof(double));
                    mx[3 * add + axis] += sd->diameter[axis];
                    mn[add] = mn[i];
                    curA += mn[i];
                    ++add;
                }
            cur = add;
        }
        free(mx);
        free(mn);
        if (cur > mol->capacity) return cur;
        if (curA > atoms->capacity) return curA;
    }

    for (int64_t i = 0; i < atoms->capacity; ++i) corr[i] = -1;
    mol->numGhost = 0;
    atoms->numGhost = 0;
    for (int axis = 0; axis < 3; ++axis)
    {
        int64_t nM = mol->numLocal + mol->numGhost;
        int64_t nA = atoms->numLocal + atoms->numGhost;
        /* counts of the scan (:79-126) */
        int64_t posM = 0, posA = 0, negM = 0, negA = 0;
        for (int64_t i = 0; i < nM; ++i)
        {
            double x = mol->pos[3 * i + axis];
            if (x < sd->minInnerCorner[axis])
            {
                negM++;
                negA += mol->numAtoms[i];
            }
            if (x >= sd->maxInnerCorner[axis])
            {
                posM++;
                posA += mol->numAtoms[i];
            }
        }
        /* positive items (x >= maxInner, shifted by -L) come first (:150-190) */
        int64_t km = 0, ka = 0;
        for (int64_t i = 0; i < nM; ++i)
        {
            if (!(mol->pos[3 * i + axis] >= sd->maxInnerCorner[axis])) continue;
            int64_t s = mol->atomsOffset[i];
            int64_t size = mol->numAtoms[i];
            int64_t dstM = nM + km;
            int64_t dstA = nA + ka;
            molecules_copy(mol, dstM, i);
            mol->pos[3 * dstM + axis] -= sd->diameter[axis];
            mol->atomsOffset[dstM] = dstA;
            mol->numAtoms[dstM] = size;
            for (int64_t a = 0; a < size; ++a)
            {
                atoms_copy(atoms, dstA + a, s + a);
                atoms->pos[3 * (dstA + a) + axis] -= sd->diameter[axis];
                int64_t realIdx = s + a;
                while (corr[realIdx] != -1) realIdx = corr[realIdx];
                corr[dstA + a] = realIdx;
            }
            km++;
            ka += size;
        }
        /* then negative items (x < minInner, shifted by +L) (:192-234) */
        km = 0;
        ka = 0;
        for (int64_t i = 0; i < nM; ++i)
        {
            if (!(mol->pos[3 * i + axis] < sd->minInnerCorner[axis])) continue;
            int64_t s = mol->atomsOffset[i];
            int64_t size = mol->numAtoms[i];
            int64_t dstM = nM + posM + km;
            int64_t dstA = nA + posA + ka;
            molecules_copy(mol, dstM, i);
            mol->pos[3 * dstM + axis] += sd->diameter[axis];
            mol->atomsOffset[dstM] = dstA;
            mol->numAtoms[dstM] = size;
            for (int64_t a = 0; a < size; ++a)
            {
                atoms_copy(atoms, dstA + a, s + a);
                atoms->pos[3 * (dstA + a) + axis] += sd->diameter[axis];
                int64_t realIdx = s + a;
                while (corr[realIdx] != -1) realIdx = corr[realIdx];
                corr[dstA + a] = realIdx;
            }
            km++;
            ka += size;
        }
        mol->numGhost += posM + negM;
        atoms->numGhost += posA + negA;
    }
    return 0;
}

/* ------------------------------------------------------------ histograms - */

void orc_hist_init(orc_hist* h, double min, double max, int64_t numBins, int64_t numHist,
                   double* data)
{
    /* data/MultiHistogram.hpp:31-47 */
    h->min = min;
    h->max = max;
    h->numBins = numBins;
    h->numHist = numHist;
    h->binSize = (max - min) / (double)numBins;
    h->inverseBinSize = 1.0 / h->binSize;
    h->data = data;
}

int64_t orc_hist_get_bin(const orc_hist* h, double val)
{
    int64_t bin = (int64_t)floor((val - h->min) * h->inverseBinSize);
    if (bin < 0) bin = -1;
    if (bin >= h->numBins) bin = -1;
    return bin;
}

double orc_hist_bin_position(const orc_hist* h, int64_t bin)
{
    return h->min + ((double)bin + 0.5) * h->binSize;
}

void orc_hist_scale(orc_hist* h, double f)
{
    for (int64_t k = 0; k < h->numBins * h->numHist; ++k) h->data[k] *= f;
}

void orc_hist_scale_per_hist(orc_hist* h, const double* f)
{
    for (int64_t b = 0; b < h->numBins; ++b)
        for (int64_t j = 0; j < h->numHist; ++j) h->data[b * h->numHist + j] *= f[j];
}

void orc_hist_make_symmetric(orc_hist* h)
{
    int64_t maxIdx = h->numBins - 1;
    for (int64_t i = 0; i < h->numBins / 2; ++i)
        for (int64_t j = 0; j < h->numHist; ++j)
        {
            double val = 0.5 * (h->data[i * h->numHist + j] + h->data[(maxIdx - i) * h->numHist + j]);
            h->data[i * h->numHist + j] = val;
            h->data[(maxIdx - i) * h->numHist + j] = val;
        }
}

void orc_hist_gradient(const orc_hist* in, orc_hist* out, int periodic)
{
    const double inverseSpacing = in->inverseBinSize;
    const double inverseDoubleSpacing = 0.5 * in->inverseBinSize;
    const int64_t nb = in->numBins, nh = in->numHist;
    const double* d = in->data;
    for (int64_t i = 0; i < nb; ++i)
        for (int64_t j = 0; j < nh; ++j)
        {
            double g;
            if (i == 0)
                g = periodic ? (d[(i + 1) * nh + j] - d[(nb - 1) * nh + j]) * inverseDoubleSpacing
                             : (d[(i + 1) * nh + j] - d[i * nh + j]) * inverseSpacing;
            else if (i == nb - 1)
                g = periodic ? (d[0 * nh + j] - d[(i - 1) * nh + j]) * inverseDoubleSpacing
                             : (d[i * nh + j] - d[(i - 1) * nh + j]) * inverseSpacing;
            else
                g = (d[(i + 1) * nh + j] - d[(i - 1) * nh + j]) * inverseDoubleSpacing;
            out->data[i * nh + j] = g;
        }
}

void orc_hist_smoothen(const orc_hist* in, orc_hist* out, double sigma, double range,
                       int periodic)
{
    const double inverseSigma = 1.0 / sigma;
    const int64_t delta = (int64_t)(int)(range * sigma * in->inverseBinSize);
    const int64_t nb = in->numBins, nh = in->numHist;
    for (int64_t b = 0; b < nb; ++b)
        for (int64_t h = 0; h < nh; ++h)
        {
            double normalization = 0.0;
            double acc = 0.0;
            int64_t jMin = b - delta, jMax = b + delta;
            if (!periodic)
            {
                if (jMin < 0) jMin = 0;
                if (jMax > nb - 1) jMax = nb - 1;
            }
            for (int64_t j = jMin; j <= jMax; ++j)
            {
                int64_t m = j;
                if (periodic)
                {
                    if (m < 0) m += nb;
                    if (m >= nb) m -= nb;
                }
                double t = (double)(b - j) * in->binSize * inverseSigma;
                const double eFunc = exp(-(t * t));
                normalization += eFunc;
                acc += in->data[m * nh + h] * eFunc;
            }
            out->data[b * nh + h] = acc / normalization;
        }
}

void orc_hist_replace_if(orc_hist* h, const orc_pred* pred1d, int invert, double newValue)
{
    /* data/MultiHistogram.hpp:180-194 */
    for (int64_t b = 0; b < h->numBins; ++b)
    {
        double x = orc_hist_bin_position(h, b);
        int hit = pred_coord(pred1d, x);
        if (invert ? !hit : hit)
            for (int64_t j = 0; j < h->numHist; ++j) h->data[b * h->numHist + j] = newValue;
    }
}

void orc_cumulative_moving_average(orc_hist* avg, const orc_hist* cur, double factor)
{
    for (int64_t k = 0; k < avg->numBins * avg->numHist; ++k)
        avg->data[k] = (factor * avg->data[k] + cur->data[k]) / (factor + 1.0);
}

void orc_axial_density_profile(const orc_atoms* atoms, int64_t n, orc_hist* h, int axis)
{
    /* analysis/AxialDensityProfile.cpp:21-51 */
    for (int64_t i = 0; i < n; ++i)
    {
        int64_t bin = orc_hist_get_bin(h, atoms->pos[3 * i + axis]);
        if (bin == -1) continue;
        h->data[bin * h->numHist + atoms->type[i]] += 1.0;
    }
}

int64_t orc_tf_num_bins(const orc_subdomain* sd, double requestedBinWidth)
{
    return (int64_t)ceil(sd->diameter[0] / requestedBinWidth);
}

void orc_tf_init(orc_tf* tf, const orc_subdomain* sd, int64_t numBins, int64_t numTypes,
                 double* forceData, double* densityData, double* forceFactor,
                 const double* targetDensity, const double* modulation, int enforceSymmetry,
                 int usePeriodicity)
{
    /* action/ThermodynamicForce.cpp:25-57 */
    orc_hist_init(&tf->force, sd->minCorner[0], sd->maxCorner[0], numBins, numTypes, forceData);
    orc_hist_init(&tf->density, sd->minCorner[0], sd->maxCorner[0], numBins, numTypes, densityData);
    tf->samples = 0;
    tf->binVolume = sd->diameter[1] * sd->diameter[2] * tf->density.binSize;
    tf->forceFactor = forceFactor;
    for (int64_t t = 0; t < numTypes; ++t) forceFactor[t] = modulation[t] / targetDensity[t];
    tf->enforceSymmetry = enforceSymmetry;
    tf->usePeriodicity = usePeriodicity;
}

void orc_tf_sample(orc_tf* tf, const orc_atoms* atoms)
{
    /* .cpp:74-86: temporary histogram then += (same FP result as adding counts) */
    int64_t nbh = tf->density.numBins * tf->density.numHist;
    double* tmp = (double*)calloc((size_t)(nbh > 0 ? nbh : 1), sizeof(double));
    orc_hist h;
    orc_hist_init(&h, tf->density.min, tf->density.max, tf->density.numBins, tf->density.numHist,
                  tmp);
    orc_axial_density_profile(atoms, atoms->numLocal, &h, 0);
    for (int64_t k = 0; k < nbh; ++k) tf->density.data[k] += tmp[k];
    free(tmp);
    tf->samples++;
}

void orc_tf_apply(const orc_tf* tf, orc_atoms* atoms, const orc_pred* pred)
{
    /* .hpp:98-122 */
    for (int64_t i = 0; i < atoms->numLocal; ++i)
    {
        double x = atoms->pos[3 * i + 0];
        if (!orc_pred_eval1(pred, atoms->pos[3 * i], atoms->pos[3 * i + 1], atoms->pos[3 * i + 2]))
            continue;
        int64_t bin = orc_hist_get_bin(&tf->force, x);
        if (bin != -1) atoms->force[3 * i + 0] += tf->force.data[bin * tf->force.numHist + atoms->type[i]];
    }
}

void orc_tf_apply_interpolated(const orc_tf* tf, orc_atoms* atoms, const orc_pred* pred)
{
    /* .hpp:154-216 */
    const orc_hist* fh = &tf->force;
    for (int64_t i = 0; i < atoms->numLocal; ++i)
    {
        double xPos = atoms->pos[3 * i + 0];
        if (!orc_pred_eval1(pred, atoms->pos[3 * i], atoms->pos[3 * i + 1], atoms->pos[3 * i + 2]))
            continue;
        int64_t bin = orc_hist_get_bin(fh, xPos);
        if (bin == -1) continue;
        int64_t t = atoms->type[i];
        double binStart = fh->min + (double)bin * fh->binSize;
        double fracInBin = (xPos - binStart) * fh->inverseBinSize;
        int64_t l, r;
        double factor;
        if (fracInBin < 0.5)
        {
            l = bin - 1;
            r = bin;
            factor = fracInBin + 0.5;
        }
        else
        {
            l = bin;
            r = bin + 1;
            factor = fracInBin - 0.5;
        }
        if (l >= 0 && r < fh->numBins)
        {
            double a = fh->data[l * fh->numHist + t];
            double b = fh->data[r * fh->numHist + t];
            atoms->force[3 * i + 0] += a + (b - a) * factor; /* util/interpolation.hpp:34-37 */
        }
        else
            atoms->force[3 * i + 0] += fh->data[bin * fh->numHist + t];
    }
}

int orc_tf_update(orc_tf* tf, double smoothingSigma, double smoothingIntensity,
                  const orc_pred* pred1d, double* scratch)
{
    /* .hpp:124-152 */
    if (tf->samples <= 0) return -1;
    if (tf->enforceSymmetry) orc_hist_make_symmetric(&tf->density);
    double normalizationFactor = 1.0 / (tf->binVolume * (double)tf->samples);
    orc_hist_scale(&tf->density, normalizationFactor);
    int64_t nbh = tf->density.numBins * tf->density.numHist;
    orc_hist smooth, grad;
    orc_hist_init(&smooth, tf->density.min, tf->density.max, tf->density.numBins,
                  tf->density.numHist, scratch);
    orc_hist_init(&grad, tf->density.min, tf->density.max, tf->density.numBins, tf->density.numHist,
                  scratch + nbh);
    orc_hist_smoothen(&tf->density, &smooth, smoothingSigma, smoothingIntensity, tf->usePeriodicity);
    orc_hist_gradient(&smooth, &grad, tf->usePeriodicity);
    orc_hist_scale_per_hist(&grad, tf->forceFactor);
    /* replace_if_bin_position(grad, x -> !pred(x), 0), ThermodynamicForce.hpp:144-145 */
    if (pred1d != NULL) orc_hist_replace_if(&grad, pred1d, 1, 0.0);
    for (int64_t k = 0; k < nbh; ++k) tf->force.data[k] -= grad.data[k];
    for (int64_t k = 0; k < nbh; ++k) tf->density.data[k] = 0.0;
    tf->samples = 0;
    return 0;
}

void orc_tf_mu(const orc_tf* tf, double* muLeft, double* muRight)
{
    /* .cpp:98-130 */
    const orc_hist* f = &tf->force;
    for (int64_t t = 0; t < f->numHist; ++t)
    {
        double l = 0.0, r = 0.0;
        for (int64_t i = 0; i < f->numBins / 2; ++i) l += f->data[i * f->numHist + t];
        for (int64_t i = f->numBins / 2; i < f->numBins; ++i) r += f->data[i * f->numHist + t];
        muLeft[t] = l * f->binSize;
        muRight[t] = r * f->binSize;
    }
}
