/*
 * mrmd_oracle.h -- CPU FP64 restatement of MRMD's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in mrmd_gb300/ and the timed CPU baseline of bench.py.  It is
 * never linked into, loaded by, or called from the product library.
 *
 * Every function restates one reference routine (MRMD 0.2.0, Kokkos/Cabana)
 * with the same arithmetic order per atom / per pair; the citation is given at
 * each declaration as path:line inside the MRMD source tree.  The Cabana 0.7
 * pieces that the reference calls but does not contain (linked-cell binning,
 * half Verlet list discriminator) are restated from Cabana's published
 * algorithm and pinned by the reference's own golden counts
 * (tests/LennardJones/LennardJones.cpp:30-38).
 *
 * Storage is array-of-structs with three doubles per vector, which is the
 * reference's layout at VECTOR_LENGTH=1 (data/Atoms.hpp:47-54).
 *
 * Build: see oracle/Makefile (plain gcc, -ffp-contract=off so that x86 and
 * aarch64 hosts produce identical bits).
 */
#ifndef MRMD_ORACLE_H
#define MRMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- domain -- */

/* data/Subdomain.hpp:41-62 */
typedef struct {
    double minCorner[3];
    double maxCorner[3];
    double ghostLayerThickness[3];
    double minGhostCorner[3];
    double maxGhostCorner[3];
    double minInnerCorner[3];
    double maxInnerCorner[3];
    double diameter[3];
    double diameterWithGhostLayer[3];
} orc_subdomain;

void orc_subdomain_init(orc_subdomain* sd, const double* minCorner, const double* maxCorner,
                        const double* ghostLayerThickness);

/* data/Atoms.hpp:47-53, 120-121.  Arrays are caller-owned with `capacity`
 * entries; pos/vel/force are [capacity][3]. */
typedef struct {
    double* pos;
    double* vel;
    double* force;
    int64_t* type;
    double* mass;
    double* charge;
    double* relativeMass;
    int64_t numLocal;
    int64_t numGhost;
    int64_t capacity;
} orc_atoms;

/* data/Molecules.hpp:41-47, 120-121.  pos/force/gradLambda are [capacity][3]. */
typedef struct {
    double* pos;
    double* force;
    double* lambda;
    double* modulatedLambda;
    double* gradLambda;
    int64_t* atomsOffset;
    int64_t* numAtoms;
    int64_t numLocal;
    int64_t numGhost;
    int64_t capacity;
} orc_molecules;

/* Number of OpenMP threads used by the parallel restatements (1 = serial,
 * bitwise-reproducible order).  Returns the previous value. */
int orc_set_threads(int n);
int orc_get_max_threads(void);

/* -------------------------------------------------------------- LJ (a1) -- */

/* impl::CappedLennardJonesPotential::PrecomputedValues, action/LennardJones.hpp:27-39 */
typedef struct {
    double ff1, ff2, ef1, ef2;
    double rcSqr;
    double cappingDistance, cappingDistanceSqr, cappingCoeff;
    double shift, energyAtCappingPoint;
} orc_lj_params;

/* Constructor + per-type precompute, action/LennardJones.cpp:61-116.
 * All vectors have numTypes*numTypes entries. */
void orc_lj_init(orc_lj_params* out, int64_t numTypes, const double* cappingDistance,
                 const double* rc, const double* sigma, const double* epsilon, int isShifted);

/* computeForceAndEnergy, action/LennardJones.hpp:52-78 */
void orc_lj_force_energy(const orc_lj_params* table, double distSqr, int64_t typeIdx,
                         double* forceFactor, double* energy);

/* Two-position predicates used with apply_if (datatypes.hpp:214-222).  The
 * in-tree callers use util::IsInSymmetricSlab (util/IsInSymmetricSlab.hpp:24-64)
 * combined with || or && (examples/04_LennardJones_IdealGas_LocalCap:206-227). */
enum {
    ORC_PRED_ALWAYS = 0,
    ORC_PRED_EITHER_IN_SLAB = 1, /* slab(x1) || slab(x2) */
    ORC_PRED_BOTH_IN_SLAB = 2,   /* slab(x1) && slab(x2) */
    ORC_PRED_IN_SLAB = 3,        /* one-position form: slab(x)        */
    ORC_PRED_IN_OPEN_INTERVAL = 4 /* one-position form: lo < x[axis] < hi */
};
typedef struct {
    int32_t kind;
    int32_t axis;
    double center;
    double slabMin;
    double slabMax;
    double tolerance;
} orc_pred;

int orc_pred_eval1(const orc_pred* p, double x, double y, double z);
int orc_pred_eval2(const orc_pred* p, double x1, double y1, double z1, double x2, double y2,
                   double z2);

/* LennardJones::apply_if, action/LennardJones.hpp:135-206.  `numTypesIndex`
 * is the multiplier used for typeIdx (the reference fixes it to 1,
 * action/LennardJones.cpp:52).  counts[i], nbrs[i*cap + n] is the half list.
 * Forces accumulate; energy and virial are returned for this call only. */
void orc_lj_apply(const orc_lj_params* table, int64_t numTypesIndex, double rcSqr,
                  orc_atoms* atoms, const int32_t* counts, const int32_t* nbrs, int64_t cap,
                  const orc_pred* pred, double* energy, double* virial);

/* ------------------------------------------------- ghost layer (a7) -- */

/* PeriodicMapping::mapIntoDomain, communication/PeriodicMapping.cpp:30-58 */
void orc_map_into_domain(orc_atoms* atoms, const orc_subdomain* sd);

/* GhostExchange::createGhostAtomsXYZ, communication/GhostExchange.cpp:59-181.
 * corr has `atoms->capacity` entries.  Returns 0, or the capacity needed
 * (>0) when the arrays are too small (nothing is modified in that case). */
int64_t orc_create_ghosts_xyz(orc_atoms* atoms, const orc_subdomain* sd, int64_t* corr);

/* UpdateGhostAtoms::updateOnlyPos, communication/UpdateGhostAtoms.cpp:31-68 */
void orc_update_ghosts(orc_atoms* atoms, const int64_t* corr, const orc_subdomain* sd);

/* AccumulateForce::ghostToReal, communication/AccumulateForce.cpp:25-47 */
void orc_ghost_to_real(orc_atoms* atoms, const int64_t* corr);

/* ------------------------------------------ cells + Verlet list (a4,a5) -- */

/* Cartesian cell grid over [gridMin, gridMax): n = max(1, floor(L/delta)) cells
 * per axis, edge L/n >= delta, cell = clamp(floor((x-min)*rdx), 0, n-1).
 * Fills nCells[3] and rdx[3]. */
void orc_cell_grid(const double* gridMin, const double* gridMax, double delta, int64_t* nCells,
                   double* rdx);

/* Linear cell id (ix*ny + iy)*nz + iz of each of the first n positions. */
void orc_cell_index(const double* pos, int64_t n, const double* gridMin, const int64_t* nCells,
                    const double* rdx, int64_t* cellOut);

/* Half Verlet list (Cabana 0.7 VerletList<HalfNeighborTag, VerletLayout2D>):
 * lists for particles [begin,end), candidates from all n particles, keep j
 * with j != i, |x_i-x_j|^2 <= rlist^2 and x_j lexicographically above x_i
 * in (x, y, z).  Writes counts[end-begin] and nbrs[(i-begin)*cap + k] as long
 * as k < cap.  Returns the largest count (the caller retries if > cap). */
int64_t orc_build_half_list(const double* pos, int64_t n, int64_t begin, int64_t end,
                            double rlist, double cellRatio, const double* gridMin,
                            const double* gridMax, int32_t* counts, int32_t* nbrs, int64_t cap);

/* countWithinCutoff, tests/LennardJones/LennardJones.cpp:40-70 (strict <). */
int64_t orc_count_within(const double* pos, int64_t nLocal, int64_t nAll, double cutoff,
                         const double* box, int periodic);

/* -------------------------------------------------- integrators (a8,a9) -- */

/* VelocityVerlet::preForceIntegrate, action/VelocityVerlet.cpp:26-67 */
double orc_vv_pre(orc_atoms* atoms, double dt);
/* VelocityVerlet::postForceIntegrate, action/VelocityVerlet.cpp:69-90 */
void orc_vv_post(orc_atoms* atoms, double dt);

/* --------------------------------------------------------- Coulomb DSF -- */
/* impl::CoulombDSF (action/CoulombDSF.hpp:39-83): damped shifted force
 * Coulomb (Fennell & Gezelter; DOI 10.1140/epjst/e2016-60151-6, eqs 15-16),
 * with util::approxErfc (util/math.hpp:57-76, Abramowitz & Stegun 7.1.26). */
typedef struct {
    double alpha, rc, rcSqr, forceShift, energyShift;
} orc_coulomb_dsf;

void orc_coulomb_dsf_init(orc_coulomb_dsf* c, double rc, double alpha);
double orc_approx_erfc(double x, double* expX2);
double orc_coulomb_dsf_force(const orc_coulomb_dsf* c, double distSqr, double q1, double q2);
double orc_coulomb_dsf_energy(const orc_coulomb_dsf* c, double distSqr, double q1, double q2);
/* The half-list loop of LennardJones::apply (action/LennardJones.hpp:135-206)
 * with the DSF pair function and the atoms' charges (cutoff rc). */
void orc_coulomb_dsf_apply(const orc_coulomb_dsf* c, orc_atoms* atoms, const int32_t* counts,
                           const int32_t* nbrs, int64_t cap, double* energyOut, double* virialOut);

/* ------------------------------------------------------------ analysis -- */
/* analysis::getKineticEnergy (analysis/KineticEnergy.hpp:26-39):
 * 0.5 * sum over local atoms of m (vx^2 + vy^2 + vz^2), serial in index order. */
double orc_kinetic_energy(const orc_atoms* atoms);
/* analysis::getSystemMomentum (analysis/SystemMomentum.cpp:21-48): the sum
 * of the local atoms' velocities per component (no mass factor). */
void orc_system_momentum(const orc_atoms* atoms, double* out3);
/* analysis::getPressure (analysis/Pressure.cpp:23-51): sum over local AND
 * ghost atoms of m v.v + F.x, divided by 3 * subdomain volume. */
double orc_pressure(const orc_atoms* atoms, const orc_subdomain* sd);

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), key (k0,k1), counter c[4]. */
void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
/* Standard normal pair from one Philox block (Box-Muller). */
void orc_normal_from_counter(uint64_t seed, uint64_t step, uint64_t atom, double* out3);

/* VelocityVerletLangevinThermostat::preForceIntegrate_apply_if,
 * action/VelocityVerletLangevinThermostat.hpp:48-121 with the noise of
 * atom idx at this step drawn by orc_normal_from_counter(seed, step, idx). */
double orc_langevin_pre(orc_atoms* atoms, double dt, double zeta, double temperature,
                        uint64_t seed, uint64_t step, const orc_pred* pred);

/* ------------------------------------------------- AdResS (a3,a13,a14) -- */

/* weighting_function::Slab, weighting_function/Slab.hpp:27-201 */
typedef struct {
    double center[3];
    double atomisticRegionHalfDiameter;
    double hybridRegionDiameter;
    int64_t exponent;      /* 2*nu */
    int32_t interfaceType; /* 0 smooth, 1 abrupt */
    int32_t pad;
} orc_slab;

void orc_slab_init(orc_slab* s, const double* center, double atomisticRegionDiameter,
                   double hybridRegionDiameter, int64_t nu, int32_t interfaceType);
void orc_slab_eval(const orc_slab* s, double x, double y, double z, double* out5);

/* UpdateMolecules::update, action/UpdateMolecules.hpp:24-70 */
void orc_update_molecules(orc_molecules* mol, const orc_atoms* atoms, const orc_slab* slab);
/* ContributeMoleculeForceToAtoms::update, action/ContributeMoleculeForceToAtoms.cpp:23-48 */
void orc_contribute_molecule_force(const orc_molecules* mol, orc_atoms* atoms);

/* LJ_IdealGas state, action/LJ_IdealGas.hpp:34-104 (200 compensation bins on [0,1)) */
#define ORC_LJIG_BINS 200
typedef struct {
    orc_lj_params* table; /* numTypes*numTypes entries, caller-owned */
    int64_t numTypes;
    double rcSqr;
    double* compensationEnergy;        /* [200][numTypes] */
    double* compensationEnergyCounter; /* [200][numTypes] */
    double* meanCompensationEnergy;    /* [200][numTypes] */
    int64_t runCounter;
    int64_t samplingInterval; /* 200 */
    int64_t updateInterval;   /* 20000 */
} orc_ljig;

/* LJ_IdealGas::run, action/LJ_IdealGas.cpp:227-260 (molecule loop :52-225). */
double orc_ljig_run(orc_ljig* s, orc_molecules* mol, const int32_t* counts, const int32_t* nbrs,
                    int64_t cap, orc_atoms* atoms);

/* updateMeanCompensationEnergy, action/LJ_IdealGas.cpp:21-50 */
void orc_update_mean_compensation_energy(double* energy, double* counter, double* mean,
                                         int64_t numBins, int64_t numHist, double factor);

/* MultiResGhostLayer, communication/MultiResRealAtomsExchange.cpp:23-73 and
 * communication/MultiResPeriodicGhostExchange.cpp:60-277.  Returns 0 or the
 * needed capacity (atoms or molecules) when too small; corrAtom has
 * atoms->capacity entries. */
void orc_multires_map_into_domain(const orc_subdomain* sd, orc_molecules* mol, orc_atoms* atoms);
int64_t orc_multires_create_ghosts_xyz(orc_molecules* mol, orc_atoms* atoms,
                                       const orc_subdomain* sd, int64_t* corrAtom);

/* ---------------------------------------------- histograms (a10-a12) -- */

/* data::MultiHistogram, data/MultiHistogram.hpp:29-92; data is [numBins][numHist]. */
typedef struct {
    double min, max;
    int64_t numBins, numHist;
    double binSize, inverseBinSize;
    double* data;
} orc_hist;

void orc_hist_init(orc_hist* h, double min, double max, int64_t numBins, int64_t numHist,
                   double* data);
int64_t orc_hist_get_bin(const orc_hist* h, double val);     /* :60-66 */
double orc_hist_bin_position(const orc_hist* h, int64_t bin); /* :68-74 */
void orc_hist_scale(orc_hist* h, double f);                   /* MultiHistogram.cpp:48-59 */
void orc_hist_scale_per_hist(orc_hist* h, const double* f);   /* :61-74 */
void orc_hist_make_symmetric(orc_hist* h);                    /* :76-90 */
void orc_hist_gradient(const orc_hist* in, orc_hist* out, int periodic);              /* :113-161 */
void orc_hist_smoothen(const orc_hist* in, orc_hist* out, double sigma, double range,
                       int periodic);                                                 /* :163-212 */
/* replace_if_bin_position (.hpp:180-194): bins whose centre satisfies pred (or
 * !pred when invert != 0) are set to newValue. */
void orc_hist_replace_if(orc_hist* h, const orc_pred* pred1d, int invert, double newValue);
void orc_cumulative_moving_average(orc_hist* avg, const orc_hist* cur, double factor); /* :92-111 */

/* analysis::getAxialDensityProfile, analysis/AxialDensityProfile.cpp:21-51;
 * adds counts into h (which must be zero to get the reference's return). */
void orc_axial_density_profile(const orc_atoms* atoms, int64_t n, orc_hist* h, int axis);

/* ThermodynamicForce, action/ThermodynamicForce.hpp:32-96, .cpp:25-96 */
typedef struct {
    orc_hist force;
    orc_hist density;
    int64_t samples;
    double binVolume;
    double* forceFactor; /* [numTypes] = modulation / targetDensity */
    int32_t enforceSymmetry;
    int32_t usePeriodicity;
} orc_tf;

/* Bin count ceil(diameter_x / requestedWidth) as in ThermodynamicForce.cpp:34 */
int64_t orc_tf_num_bins(const orc_subdomain* sd, double requestedBinWidth);
void orc_tf_init(orc_tf* tf, const orc_subdomain* sd, int64_t numBins, int64_t numTypes,
                 double* forceData, double* densityData, double* forceFactor,
                 const double* targetDensity, const double* modulation, int enforceSymmetry,
                 int usePeriodicity);
void orc_tf_sample(orc_tf* tf, const orc_atoms* atoms);                       /* .cpp:74-86 */
void orc_tf_apply(const orc_tf* tf, orc_atoms* atoms, const orc_pred* pred);  /* .hpp:98-122 */
void orc_tf_apply_interpolated(const orc_tf* tf, orc_atoms* atoms,
                               const orc_pred* pred);                        /* .hpp:154-216 */
/* update_if (.hpp:124-152); pred1d==NULL means update() (.cpp:88-91).
 * scratch needs 2*numBins*numTypes doubles.  Returns -1 when no samples. */
int orc_tf_update(orc_tf* tf, double smoothingSigma, double smoothingIntensity,
                  const orc_pred* pred1d, double* scratch);
void orc_tf_mu(const orc_tf* tf, double* muLeft, double* muRight); /* .cpp:98-130 */

#ifdef __cplusplus
}
#endif
#endif
