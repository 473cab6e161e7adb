/*
 * mrmd_gb300.h -- C ABI of the GB300-native MRMD hot path.
 *
 * One process, one GPU (sm_103a).  Every entry point takes plain pointers and
 * sizes, returns an int status (MRMD_OK == 0, negative on error) and never
 * throws.  Device data lives in structs of device pointers that this library
 * allocates (mrmd_atoms_alloc, mrmd_molecules_alloc, ...); the caller owns the
 * structs and frees them through the matching *_free call.
 *
 * Each declaration names the MRMD (v0.2.0) interface it replaces as
 * path:line inside the MRMD source tree.  Entry points are synchronous by
 * default (like the reference's Kokkos::fence() at the end of every action);
 * mrmd_ctx_set_sync(ctx, 0) turns that off so that a caller can capture a
 * step into a CUDA graph on the context stream.
 */
#ifndef MRMD_GB300_H
#define MRMD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status -- */
enum {
    MRMD_OK = 0,
    MRMD_ERR_ARG = -1,            /* invalid argument (null, negative size, bad enum)   */
    MRMD_ERR_OOM = -2,            /* device or pinned allocation failed                 */
    MRMD_ERR_NLIST_OVERFLOW = -3, /* neighbour list capacity exceeded after retries     */
    MRMD_ERR_NONFINITE = -4,      /* NaN/Inf detected in positions or forces            */
    MRMD_ERR_TIMEOUT = -5,        /* a bounded device wait gave up                      */
    MRMD_ERR_CUDA = -6,           /* CUDA runtime error (see mrmd_ctx_last_error)      */
    MRMD_ERR_STATE = -7,          /* call order violated (e.g. no ghosts created yet)   */
    MRMD_ERR_CAPACITY = -8,       /* fixed capacity exceeded (no growth allowed here)   */
    MRMD_ERR_BOUNDS = -9          /* bounds-checked build: an index was out of range    */
};

/* Precision of the pair arithmetic. */
enum {
    MRMD_PREC_FP64 = 0,  /* plain FP64 drop-in: all arithmetic in double              */
    MRMD_PREC_MIXED = 1  /* FP32 pair arithmetic on cell-relative split coordinates,
                            FP64 positions, velocities, force/energy/virial sums     */
};

/* Predicate forms used by apply_if-style calls (datatypes.hpp:196-222).  The
 * slab forms are util::IsInSymmetricSlab (util/IsInSymmetricSlab.hpp:24-64);
 * the interval form is `lo < x[axis] < hi`. */
enum {
    MRMD_PRED_ALWAYS = 0,
    MRMD_PRED_EITHER_IN_SLAB = 1, /* two positions: slab(p1) || slab(p2) */
    MRMD_PRED_BOTH_IN_SLAB = 2,   /* two positions: slab(p1) && slab(p2) */
    MRMD_PRED_IN_SLAB = 3,        /* one position: slab(p)               */
    MRMD_PRED_IN_OPEN_INTERVAL = 4 /* one position: lo < p[axis] < hi    */
};
typedef struct {
    int32_t kind;
    int32_t axis;
    double center;
    double slabMin; /* or `lo` for the interval form */
    double slabMax; /* or `hi` for the interval form */
    double tolerance;
} mrmd_pred;

/* ------------------------------------------------------------ context -- */
typedef struct mrmd_ctx mrmd_ctx;

/* Replaces Kokkos::initialize / ScopeGuard (initialization.cpp:23-44) for the
 * device side: binds `device`, creates the context stream and error word. */
int mrmd_ctx_create(mrmd_ctx** out, int device);
int mrmd_ctx_destroy(mrmd_ctx* ctx);
/* Kokkos::fence() equivalent: waits for the context stream. */
int mrmd_ctx_sync(mrmd_ctx* ctx);
/* 1 (default): every entry point synchronises before returning. */
int mrmd_ctx_set_sync(mrmd_ctx* ctx, int sync);
/* The CUDA stream (cudaStream_t) all kernels of this context run on. */
void* mrmd_ctx_stream(mrmd_ctx* ctx);
const char* mrmd_ctx_last_error(mrmd_ctx* ctx);
/* 1 in the bounds-checked debug build (libmrmd_gb300_bounds.so, compiled with
 * -DMRMD_BOUNDS_CHECK; the counterpart of the reference's
 * Kokkos_ENABLE_DEBUG_BOUNDS_CHECK CI build, .github/workflows/validate.yml:40),
 * 0 otherwise.  In that build every kernel index into a particle, cell or
 * list array is checked first; the first violation is recorded with its
 * source line, the access is skipped and the entry point returns
 * MRMD_ERR_BOUNDS at its next synchronisation. */
int mrmd_bounds_checked(void);
/* Number of kernel launches issued by this context so far. */
int64_t mrmd_ctx_launch_count(mrmd_ctx* ctx);
const char* mrmd_version(void);

/* -------------------------------------------------------------- atoms -- */
/* data::Atoms (data/Atoms.hpp:33-177).  Device layout: pos/vel/force are
 * [capacity][4] doubles (x, y, z, pad) so that one atom is one 32-byte
 * sector; scalars are plain arrays.  type is int32 on the device (the
 * reference's int64 type ids are range-checked at upload). */
typedef struct {
    double* pos;
    double* vel;
    double* force;
    int32_t* type;
    double* mass;
    double* charge;
    double* relativeMass;
    int64_t numLocal;
    int64_t numGhost;
    int64_t capacity;
} mrmd_atoms;

/* GeneralAtoms(numAtoms) constructor (data/Atoms.hpp:123-133): zeroed storage. */
int mrmd_atoms_alloc(mrmd_ctx* ctx, mrmd_atoms* a, int64_t capacity);
int mrmd_atoms_free(mrmd_ctx* ctx, mrmd_atoms* a);
/* GeneralAtoms::resize (data/Atoms.hpp:89-93): grows capacity, keeps content. */
int mrmd_atoms_reserve(mrmd_ctx* ctx, mrmd_atoms* a, int64_t capacity);
/* deep_copy host -> device (data/Atoms.hpp:150-159).  Host arrays are the
 * reference's AoS layout ([n][3] doubles, int64 types); any pointer may be
 * NULL to leave that field untouched.  Sets numLocal/numGhost. */
int mrmd_atoms_upload(mrmd_ctx* ctx, mrmd_atoms* a, int64_t numLocal, int64_t numGhost,
                      const double* pos3, const double* vel3, const double* force3,
                      const int64_t* type, const double* mass, const double* charge,
                      const double* relativeMass);
/* deep_copy device -> host of the first n atoms; NULL pointers are skipped. */
int mrmd_atoms_download(mrmd_ctx* ctx, const mrmd_atoms* a, int64_t n, double* pos3,
                        double* vel3, double* force3, int64_t* type, double* mass,
                        double* charge, double* relativeMass);
/* GeneralAtoms::setForce(val) / Cabana::deep_copy(force, val) for atoms [0, n). */
int mrmd_atoms_set_force(mrmd_ctx* ctx, mrmd_atoms* a, int64_t n, double val);
/* Atoms::permute(LinkedCellList) (data/Atoms.hpp:95): stable counting sort of
 * the local atoms by cell of the grid [gridMin, gridMax) with cells of edge
 * >= delta.  perm_out (device, may be NULL) receives old index per new slot. */
int mrmd_atoms_sort_by_cell(mrmd_ctx* ctx, mrmd_atoms* a, const double* gridMin,
                            const double* gridMax, double delta, int64_t* perm_out);

/* ---------------------------------------------------------- molecules -- */
/* data::Molecules (data/Molecules.hpp:27-176).  pos/force/gradLambda are
 * [capacity][4] doubles on the device. */
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
} mrmd_molecules;

int mrmd_molecules_alloc(mrmd_ctx* ctx, mrmd_molecules* m, int64_t capacity);
int mrmd_molecules_free(mrmd_ctx* ctx, mrmd_molecules* m);
int mrmd_molecules_reserve(mrmd_ctx* ctx, mrmd_molecules* m, int64_t capacity);
int mrmd_molecules_upload(mrmd_ctx* ctx, mrmd_molecules* m, int64_t numLocal, int64_t numGhost,
                          const double* pos3, const double* force3, const double* lambda,
                          const double* modulatedLambda, const double* gradLambda3,
                          const int64_t* atomsOffset, const int64_t* numAtoms);
int mrmd_molecules_download(mrmd_ctx* ctx, const mrmd_molecules* m, int64_t n, double* pos3,
                            double* force3, double* lambda, double* modulatedLambda,
                            double* gradLambda3, int64_t* atomsOffset, int64_t* numAtoms);
/* GeneralMolecules::setForce (data/Molecules.hpp:60). */
int mrmd_molecules_set_force(mrmd_ctx* ctx, mrmd_molecules* m, int64_t n, double val);

/* ------------------------------------------------------- ghost layer -- */
/* data::Subdomain corners (data/Subdomain.hpp:41-62); filled by
 * mrmd_subdomain_init from min/max corner and ghost layer thickness. */
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
} mrmd_subdomain;

int mrmd_subdomain_init(mrmd_subdomain* sd, const double* minCorner, const double* maxCorner,
                        const double* ghostLayerThickness3);

/* communication::GhostLayer / MultiResGhostLayer state: the
 * correspondingRealAtom index of every atom (-1 for real atoms). */
typedef struct {
    int32_t* correspondingRealAtom; /* device, [capacity] */
    int64_t capacity;
    int64_t numLocal; /* atom counts the ghosts were built for */
    int64_t numGhost;
    /* real atom -> its ghosts, CSR sorted by ghost index (device); lets the
     * force fold-back gather in the reference's serial order without atomics */
    int32_t* ghostStart; /* [localCapacity + 1] */
    int32_t* ghostList;  /* [capacity]          */
    int64_t localCapacity;
} mrmd_ghost_layer;

int mrmd_ghost_layer_alloc(mrmd_ctx* ctx, mrmd_ghost_layer* g, int64_t capacity);
int mrmd_ghost_layer_free(mrmd_ctx* ctx, mrmd_ghost_layer* g);
/* GhostLayer::exchangeRealAtoms -> PeriodicMapping::mapIntoDomain
 * (communication/GhostLayer.hpp:35-38, PeriodicMapping.cpp:30-58). */
int mrmd_ghost_exchange_real_atoms(mrmd_ctx* ctx, mrmd_atoms* a, const mrmd_subdomain* sd);
/* GhostLayer::createGhostAtoms -> GhostExchange::createGhostAtomsXYZ
 * (GhostLayer.hpp:40-43, GhostExchange.cpp:59-181).  Same ghost set and
 * order as the reference; grows atoms/ghost-layer capacity when needed. */
int mrmd_ghost_create(mrmd_ctx* ctx, mrmd_ghost_layer* g, mrmd_atoms* a, const mrmd_subdomain* sd);
/* GhostLayer::updateGhostAtoms -> UpdateGhostAtoms::updateOnlyPos
 * (GhostLayer.hpp:45-50, UpdateGhostAtoms.cpp:31-68). */
int mrmd_ghost_update(mrmd_ctx* ctx, const mrmd_ghost_layer* g, mrmd_atoms* a,
                      const mrmd_subdomain* sd);
/* GhostLayer::contributeBackGhostToReal -> AccumulateForce::ghostToReal
 * (GhostLayer.hpp:52-55, AccumulateForce.cpp:25-47). */
int mrmd_ghost_reduce_force(mrmd_ctx* ctx, const mrmd_ghost_layer* g, mrmd_atoms* a);
/* MultiResGhostLayer::exchangeRealAtoms -> realAtomsExchange
 * (MultiResGhostLayer.hpp:36-41, MultiResRealAtomsExchange.cpp:23-73). */
int mrmd_multires_exchange_real_atoms(mrmd_ctx* ctx, mrmd_molecules* m, mrmd_atoms* a,
                                      const mrmd_subdomain* sd);
/* MultiResGhostLayer::createGhostAtoms -> MultiResPeriodicGhostExchange::createGhostAtomsXYZ
 * (MultiResGhostLayer.hpp:43-48, MultiResPeriodicGhostExchange.cpp:60-277). */
int mrmd_multires_ghost_create(mrmd_ctx* ctx, mrmd_ghost_layer* g, mrmd_molecules* m,
                               mrmd_atoms* a, const mrmd_subdomain* sd);
/* Copy the correspondingRealAtom array (first n entries) to the host. */
int mrmd_ghost_layer_download(mrmd_ctx* ctx, const mrmd_ghost_layer* g, int64_t n, int64_t* out);

/* ------------------------------------------------- neighbour list -- */
/* HalfVerletList = Cabana::VerletList<HalfNeighborTag, VerletLayout2D>
 * (datatypes.hpp:184-187).  Layout: counts[rows]; neighbours in tiles of 32
 * rows, entry k of row i at (i / 32) * 32 * maxNeighbors + 32 * k + i % 32,
 * so a warp reading slot k of its 32 rows issues one 128-byte load and a
 * warp's whole list is one compact tile (written without partial sectors). */
typedef struct {
    int32_t* counts;   /* device, [rowsCapacity]                          */
    int32_t* nbrs;     /* device, [ceil(rows / 32) * 32 * maxNeighbors]   */
    int64_t rows;      /* number of list rows (end - begin)               */
    int64_t begin;     /* first particle with a list                      */
    int64_t stride;    /* step between consecutive slots of a row (32)    */
    int64_t maxNeighbors;
    int64_t rowsCapacity;
    int64_t nbrsCapacity; /* allocated int32 entries of nbrs */
    int64_t totalPairs;   /* sum of counts after the last build */
    void* cells;          /* opaque cell-grid scratch owned by the list */
} mrmd_nlist;

int mrmd_nlist_init(mrmd_ctx* ctx, mrmd_nlist* nl);
int mrmd_nlist_free(mrmd_ctx* ctx, mrmd_nlist* nl);
/* HalfVerletList::build(pos, begin, end, r, cell_ratio, gridMin, gridMax,
 * maxNeigh) (call sites examples/02_LennardJones_NVE:156-163,
 * tests/LennardJones/LennardJones.cpp:112-118).  Candidates are positions
 * [0, nPos); a pair (i, j) is kept when |x_i - x_j|^2 <= r^2 and x_j is
 * above x_i in lexicographic (x, y, z) order (Cabana's half-neighbour
 * discriminator).  Capacity grows (and the build reruns) on overflow. */
int mrmd_nlist_build(mrmd_ctx* ctx, mrmd_nlist* nl, const double* pos4, int64_t nPos,
                     int64_t begin, int64_t end, double rlist, double cellRatio,
                     const double* gridMin, const double* gridMax, int64_t maxNeighbors);
/* Copy counts (rows) and neighbours in row-major [rows][cap] form to the host. */
int mrmd_nlist_download(mrmd_ctx* ctx, const mrmd_nlist* nl, int32_t* counts, int32_t* nbrs,
                        int64_t cap);
/* Cell id of each of the first n positions on the grid the list builder uses
 * (cell edge >= delta; id = (ix*ny + iy)*nz + iz).  cells_out is host int64[n]. */
int mrmd_cell_index(mrmd_ctx* ctx, const double* pos4, int64_t n, const double* gridMin,
                    const double* gridMax, double delta, int64_t* cells_out);

/* ------------------------------------------------------ Lennard-Jones -- */
/* impl::CappedLennardJonesPotential::PrecomputedValues (action/LennardJones.hpp:27-39). */
typedef struct {
    double ff1, ff2, ef1, ef2;
    double rcSqr;
    double cappingDistance, cappingDistanceSqr, cappingCoeff;
    double shift, energyAtCappingPoint;
} mrmd_lj_params;

typedef struct mrmd_lj mrmd_lj;
/* LennardJones(cappingDistance, rc, sigma, epsilon, numTypes, isShifted)
 * (action/LennardJones.hpp:127-132, LennardJones.cpp:46-56,81-116): vectors of
 * numTypes^2 entries.  numTypesIndex is the multiplier of type_i in the
 * table index (the reference's LennardJones fixes it to 1,
 * action/LennardJones.cpp:52; LJ_IdealGas uses numTypes, LJ_IdealGas.cpp:139). */
int mrmd_lj_create(mrmd_ctx* ctx, mrmd_lj** out, int64_t numTypes, int64_t numTypesIndex,
                   const double* cappingDistance, const double* rc, const double* sigma,
                   const double* epsilon, int isShifted);
int mrmd_lj_destroy(mrmd_ctx* ctx, mrmd_lj* lj);
int mrmd_lj_get_params(const mrmd_lj* lj, mrmd_lj_params* out, int64_t count);
/* LennardJones::apply / apply_if (LennardJones.cpp:24-33, LennardJones.hpp:135-206):
 * half-list pair force over local atoms [0, a->numLocal) with the list's
 * rows, forces accumulated (i and j, ghosts included), energy and virial
 * of this call returned (either pointer may be NULL). */
int mrmd_lj_apply(mrmd_ctx* ctx, mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                  const mrmd_pred* pred, int precision, double* energy, double* virial);

/* Largest atom count (local + ghost) mrmd_lj_apply_mixed_noalloc accepts. */
#define MRMD_LJ_NOALLOC_MAX_ATOMS 262144

/* No counterpart in the reference.  The mixed-form mrmd_lj_apply for callers
 * that cannot allocate device memory during their step loop (all free
 * memory already belongs to another allocator, or a cudaMalloc and its
 * implied synchronisation are not allowed there): same arguments and
 * results as mrmd_lj_apply(..., MRMD_PREC_MIXED, ...), but its scratch is a
 * fixed array inside the library (8 MiB per GPU, held until exit) and it
 * calls no allocator.  Rejects more than MRMD_LJ_NOALLOC_MAX_ATOMS atoms
 * with MRMD_ERR_CAPACITY.  The first call on a device looks up the array's
 * device address (make it before any stream capture); calls that overlap
 * on the GPU share the array and race. */
int mrmd_lj_apply_mixed_noalloc(mrmd_ctx* ctx, mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                                const mrmd_pred* pred, double* energy, double* virial);

/* ------------------------------------------------------- integrators -- */
/* VelocityVerlet::preForceIntegrate (action/VelocityVerlet.cpp:26-67);
 * returns the max displacement in *maxDisplacement (may be NULL). */
int mrmd_vv_pre(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double* maxDisplacement);
/* VelocityVerlet::postForceIntegrate (action/VelocityVerlet.cpp:69-90). */
int mrmd_vv_post(mrmd_ctx* ctx, mrmd_atoms* a, double dt);
/* VelocityVerletLangevinThermostat::preForceIntegrate(_apply_if)
 * (action/VelocityVerletLangevinThermostat.hpp:33-121).  The reference's
 * XorShift1024 pool is replaced by Philox4x32-10 keyed by (seed, step) with
 * the local atom index as counter, so a run is reproducible. */
int mrmd_langevin_pre(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double zeta, double temperature,
                      uint64_t seed, uint64_t step, const mrmd_pred* pred,
                      double* maxDisplacement);

/* ------------------------------------------------------------ AdResS -- */
/* weighting_function::Slab (weighting_function/Slab.hpp:189-200): center,
 * atomistic region diameter, hybrid width, nu (exponent 2*nu), interface
 * type 0 smooth / 1 abrupt. */
typedef struct {
    double center[3];
    double atomisticRegionDiameter;
    double hybridRegionDiameter;
    int64_t nu;
    int32_t interfaceType;
    int32_t pad;
} mrmd_slab;

/* UpdateMolecules::update<Slab> (action/UpdateMolecules.hpp:24-70). */
int mrmd_update_molecules(mrmd_ctx* ctx, mrmd_molecules* m, const mrmd_atoms* a,
                          const mrmd_slab* slab);
/* ContributeMoleculeForceToAtoms::update (action/ContributeMoleculeForceToAtoms.cpp:23-48). */
int mrmd_contribute_molecule_force(mrmd_ctx* ctx, const mrmd_molecules* m, mrmd_atoms* a);

typedef struct mrmd_ljig mrmd_ljig;
/* LJ_IdealGas(cappingDistance, rc, sigma, epsilon, numTypes, doShift)
 * (action/LJ_IdealGas.hpp:92-103, LJ_IdealGas.cpp:262-292). */
int mrmd_ljig_create(mrmd_ctx* ctx, mrmd_ljig** out, int64_t numTypes,
                     const double* cappingDistance, const double* rc, const double* sigma,
                     const double* epsilon, int doShift);
int mrmd_ljig_destroy(mrmd_ctx* ctx, mrmd_ljig* s);
/* setCompensationEnergySamplingInterval / setCompensationEnergyUpdateInterval
 * (LJ_IdealGas.hpp:73-80). */
int mrmd_ljig_set_intervals(mrmd_ljig* s, int64_t samplingInterval, int64_t updateInterval);
/* LJ_IdealGas::run (LJ_IdealGas.cpp:227-260). */
int mrmd_ljig_run(mrmd_ctx* ctx, mrmd_ljig* s, mrmd_molecules* m, const mrmd_nlist* nl,
                  mrmd_atoms* a, int precision, double* energy);
/* getMeanCompensationEnergy (LJ_IdealGas.hpp:81) and the two sampling
 * histograms, each [200][numTypes] (any pointer may be NULL). */
int mrmd_ljig_get_compensation(mrmd_ctx* ctx, const mrmd_ljig* s, double* mean, double* energy,
                               double* counter, int64_t* runCounter);
int mrmd_ljig_set_compensation(mrmd_ctx* ctx, mrmd_ljig* s, const double* mean);

/* --------------------------------------------------------- Coulomb DSF -- */
/* impl::CoulombDSF (action/CoulombDSF.hpp:39-83): damped shifted force
 * Coulomb, pair function with util::approxErfc (util/math.hpp:57-76). */
typedef struct {
    double alpha, rc, rcSqr, forceShift, energyShift;
} mrmd_coulomb_dsf_params;
/* CoulombDSF(rc, alpha) (CoulombDSF.hpp:76-83): the shifts, with the exact erfc. */
int mrmd_coulomb_dsf_init(mrmd_coulomb_dsf_params* out, double rc, double alpha);
/* computeForce / computeEnergy (CoulombDSF.hpp:52-74) evaluated on the device
 * for n (distSqr, q1, q2) host triples; force is the reference's
 * force / distSqr factor. */
int mrmd_coulomb_dsf_eval(mrmd_ctx* ctx, const mrmd_coulomb_dsf_params* c, int64_t n,
                          const double* distSqr, const double* q1, const double* q2,
                          double* force, double* energy);
/* The pair force on a half list with the atoms' charges, in the loop of
 * LennardJones::apply (action/LennardJones.hpp:135-206): forces added to i
 * and j (ghosts included), energy and virial (-1/2 sum ff r^2) summed. */
int mrmd_coulomb_dsf_apply(mrmd_ctx* ctx, const mrmd_coulomb_dsf_params* c, mrmd_atoms* a,
                           const mrmd_nlist* nl, double* energy, double* virial);

/* ------------------------------------------------------------ analysis -- */
/* Deterministic device sums (fixed grid and order; same bits on every run). */
/* analysis::getKineticEnergy (analysis/KineticEnergy.hpp:26-39): 0.5 sum m v.v
 * over the local atoms. */
int mrmd_kinetic_energy(mrmd_ctx* ctx, const mrmd_atoms* a, double* out);
/* analysis::getSystemMomentum (analysis/SystemMomentum.cpp:21-48): the sum of
 * the local atoms' velocities (the reference applies no mass factor). */
int mrmd_system_momentum(mrmd_ctx* ctx, const mrmd_atoms* a, double* out3);
/* analysis::getPressure (analysis/Pressure.cpp:23-51): sum over local and
 * ghost atoms of m v.v + F.x, divided by 3 * Subdomain::getVolume. */
int mrmd_pressure(mrmd_ctx* ctx, const mrmd_atoms* a, const mrmd_subdomain* sd, double* out);

/* ------------------------------------------------ thermodynamic force -- */
typedef struct mrmd_tf mrmd_tf;
/* ThermodynamicForce(targetDensity[], subdomain, binWidth, modulation[],
 * enforceSymmetry, usePeriodicity) (action/ThermodynamicForce.cpp:25-57). */
int mrmd_tf_create(mrmd_ctx* ctx, mrmd_tf** out, int64_t numTypes, const double* targetDensity,
                   const mrmd_subdomain* sd, double requestedBinWidth,
                   const double* modulation, int enforceSymmetry, int usePeriodicity);
int mrmd_tf_destroy(mrmd_ctx* ctx, mrmd_tf* tf);
/* numBins, binSize, numTypes of the force/density histograms. */
int mrmd_tf_shape(const mrmd_tf* tf, int64_t* numBins, double* binSize, int64_t* numTypes);
/* ThermodynamicForce::sample (ThermodynamicForce.cpp:74-86). */
int mrmd_tf_sample(mrmd_ctx* ctx, mrmd_tf* tf, const mrmd_atoms* a);
/* apply / apply_if (ThermodynamicForce.cpp:93-96, .hpp:98-122) and
 * applyInterpolated_if (.hpp:154-216) when interpolated != 0. */
int mrmd_tf_apply(mrmd_ctx* ctx, const mrmd_tf* tf, mrmd_atoms* a, const mrmd_pred* pred,
                  int interpolated);
/* update / update_if (ThermodynamicForce.cpp:88-91, .hpp:124-152); pred may
 * be NULL (update).  Returns MRMD_ERR_STATE without samples. */
int mrmd_tf_update(mrmd_ctx* ctx, mrmd_tf* tf, double smoothingSigma, double smoothingIntensity,
                   const mrmd_pred* pred);
/* getForce / setForce / getDensityProfile / getNumberOfDensityProfileSamples
 * (.hpp:48-63), host arrays [numBins][numTypes]. */
int mrmd_tf_get_force(mrmd_ctx* ctx, const mrmd_tf* tf, double* out);
int mrmd_tf_set_force(mrmd_ctx* ctx, mrmd_tf* tf, const double* in);
int mrmd_tf_get_density(mrmd_ctx* ctx, const mrmd_tf* tf, double* out, int64_t* samples);
/* getMuLeft / getMuRight (ThermodynamicForce.cpp:98-130), host [numTypes]. */
int mrmd_tf_mu(mrmd_ctx* ctx, const mrmd_tf* tf, double* muLeft, double* muRight);
/* createGrid(getForce()): the bin centres min + (i + 0.5) binSize
 * (data/MultiHistogram.cpp:214-227, MultiHistogram.hpp:68-74), host [numBins]. */
int mrmd_tf_grid(const mrmd_tf* tf, double* grid);

/* ------------------------------------- thermodynamic-force table text -- */
/* The text format of io/DumpThermoForce.cpp and io/RestoreThermoForce.cpp:
 * line 1 the bin centres, then one line of forces per type; values separated
 * by one space, written with std::ostream's default formatting (6 significant
 * digits); every line ends with a newline.  The two table calls are host-only
 * and take ctx only for the error message (it may be NULL). */

/* dumpThermoForce(filename, tf, typeId) (io/DumpThermoForce.cpp:24-40) and
 * dumpThermoForce(filename, tf) (:42-64) over host arrays grid[numBins] and
 * force[numBins][numTypes]; typeId < 0 writes every type. */
int mrmd_tf_write_table(mrmd_ctx* ctx, const char* path, int64_t numBins, const double* grid,
                        int64_t numTypes, const double* force, int64_t typeId);
/* The parser of restoreThermoForce (io/RestoreThermoForce.cpp:34-73): the grid
 * line must hold >= 2 values, there may be at most maxNumForces force lines,
 * each as long as the grid line (MRMD_ERR_ARG otherwise).  Returns the shape
 * and binWidth = grid[1] - grid[0]; grid (numBins) and force
 * ([numBins][numForces], `capacity` doubles) may be NULL to query the shape. */
int mrmd_tf_read_table(mrmd_ctx* ctx, const char* path, int64_t maxNumForces, int64_t* numBins,
                       int64_t* numForces, double* binWidth, double* grid, double* force,
                       int64_t capacity);
/* dumpThermoForce of a device table (io/DumpThermoForce.cpp:24-64). */
int mrmd_tf_dump(mrmd_ctx* ctx, const mrmd_tf* tf, const char* path, int64_t typeId);
/* restoreThermoForce(filename, subdomain, targetDensities, modulations,
 * enforceSymmetry, usePeriodicity, maxNumForces) (io/RestoreThermoForce.cpp:24-90):
 * a new table with the file's bin width, its forces uploaded.  The file must
 * hold numTypes force lines of ceil(diameter / binWidth) values, the extents
 * setForce's deep_copy requires (ThermodynamicForce.hpp:55). */
int mrmd_tf_restore(mrmd_ctx* ctx, mrmd_tf** out, const char* path, const mrmd_subdomain* sd,
                    int64_t numTypes, const double* targetDensity, const double* modulation,
                    int enforceSymmetry, int usePeriodicity, int64_t maxNumForces);

/* ---------------------------------------------- fused LJ NVE stepper -- */
/* The examples/02_LennardJones_NVE time loop (02_LennardJones_NVE.cpp:135-216)
 * as one device-resident object: cell-sorted atoms, ghost layer, half list
 * rebuilt every `rebuildInterval` steps, VV integration fused with force
 * zeroing, and the steps between rebuilds replayed as one CUDA graph. */
typedef struct mrmd_md mrmd_md;
typedef struct {
    double boxMin[3];
    double boxMax[3];
    double rc;
    double skin;
    double sigma;
    double epsilon;
    double cappingDistance;
    int32_t shifted;
    int32_t precision;       /* MRMD_PREC_FP64 or MRMD_PREC_MIXED */
    double dt;
    int64_t rebuildInterval; /* steps between list rebuilds (>= 1) */
    int32_t useGraph;        /* capture the steps between rebuilds as a CUDA graph */
    int32_t sortAtoms;       /* k > 0: permute atoms into cell order at every k-th rebuild; 0: never */
    int64_t maxNeighbors;    /* initial list capacity (grown on overflow) */
    int32_t observe;         /* record kinetic energy and momentum of every step */
    int32_t gatherNeighbours; /* mixed form: 1 = read neighbour records through the cache
                                 from the int32 lists instead of shared-memory tiles */
    double splitRadius;      /* mixed form: pairs beyond it are evaluated in FP32, closer
                                ones in double-float; 0 = 1.5 sigma (at least 1.05 x the
                                capping distance); >= rc: every pair in double-float */
    int32_t tileBuild;       /* mixed form: 0 = the tile list in one pass from the cell list
                                (the int32 rows and their tile form when a tile does not fit);
                                1 = always the int32 rows, then their tile form */
    int32_t reserved0;
} mrmd_md_config;

int mrmd_md_create(mrmd_ctx* ctx, mrmd_md** out, const mrmd_md_config* cfg, int64_t n,
                   const double* pos3, const double* vel3, const double* mass);
int mrmd_md_destroy(mrmd_ctx* ctx, mrmd_md* md);
/* Advance nsteps; energies (may be NULL) receives the LJ energy and virial
 * of every step as [nsteps][2] (read back from pinned memory at the end). */
int mrmd_md_run(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps, double* energies);
/* As mrmd_md_run for a stepper created with observe = 1; records receives
 * [nsteps][6]: LJ energy, LJ virial, kinetic energy (analysis/KineticEnergy.hpp:26-39)
 * and the velocity sum of getSystemMomentum (analysis/SystemMomentum.cpp:21-48)
 * at the end of every step, with full-step velocities.  They are summed on the
 * device inside the step's own kernels (deterministic order); the only host
 * transfer is the one copy of all records at the end of the run. */
int mrmd_md_run_observed(mrmd_ctx* ctx, mrmd_md* md, int64_t nsteps, double* records);
/* Current state in the ORIGINAL atom order (host [n][3] arrays, NULL skips). */
int mrmd_md_get_state(mrmd_ctx* ctx, mrmd_md* md, double* pos3, double* vel3, double* force3);
/* Replace positions/velocities (original order) and force a rebuild. */
int mrmd_md_set_state(mrmd_ctx* ctx, mrmd_md* md, const double* pos3, const double* vel3);
/* Counters: [0] steps, [1] rebuilds, [2] list pairs, [3] ghosts, [4] list
 * capacity (near + far rows for the mixed form). */
int mrmd_md_stats(const mrmd_md* md, int64_t* out5);
/* what = 0: forces of the current positions (rebuilding ghosts and list when
 * the state was replaced), energy/virial into ev2 (host, may be NULL);
 * what = 1: launch only the pair-force kernel on the current list and split
 * coordinates, asynchronously (for timing the kernel alone). */
int mrmd_md_eval(mrmd_ctx* ctx, mrmd_md* md, int what, double* ev2);
/* Access to the internal atoms / list for profiling and tests (the mixed
 * form's list is split by distance; this is its near part). */
const mrmd_atoms* mrmd_md_atoms(const mrmd_md* md);
const mrmd_nlist* mrmd_md_nlist(const mrmd_md* md);
/* Mixed form's tile list: [0] tiles, [1] members of the largest tile,
 * [2] 1 when the pair kernel reads shared-memory tiles, 0 when it gathers
 * through the int32 lists (a tile over capacity, or gatherNeighbours),
 * [3] members of all tiles, [4] tiles of the last rebuild that the one-pass
 * tile build could not fit (the rebuild then made the int32 rows and their
 * tile form), [5] rebuilds so far that needed that second path. */
int mrmd_md_tile_stats(const mrmd_md* md, int64_t* out6);
/* The stepper's current neighbour pairs as canonical keys a * 2^32 + b of
 * unordered pairs of original atom indices (a < b; ghosts mapped to their
 * real atom), one key per list entry as the pair kernel reads it (the mixed
 * form's full list holds every pair twice), sorted.  keys may be NULL to
 * query *count; otherwise cap >= *count entries are written.  For tests and
 * diagnostics. */
int mrmd_md_pair_keys(mrmd_ctx* ctx, mrmd_md* md, int64_t* keys, int64_t cap, int64_t* count);

/* ------------------------------------------ fused AdResS stepper -- */
/* The AdResS LJ <-> ideal-gas step composed from LJ_IdealGas::run
 * (LJ_IdealGas.cpp:227-260), VelocityVerletLangevinThermostat
 * (VelocityVerletLangevinThermostat.hpp:48-121), UpdateMolecules with a Slab
 * (UpdateMolecules.hpp:24-70), ContributeMoleculeForceToAtoms
 * (ContributeMoleculeForceToAtoms.cpp:23-48), MultiResGhostLayer and
 * ThermodynamicForce sample/apply/update (ThermodynamicForce.cpp:74-96),
 * for single-site molecules; the reference has no driver for this step.
 * With unit masses (mass NULL or all 1) the step runs on the batched engine
 * with one replica (mrmd_batch_*: molecule pairs that stay coarse grained
 * until the next rebuild are left out of its full list, the mixed form
 * evaluates far pairs in FP32); other masses run the composed actions. */
typedef struct mrmd_adress mrmd_adress;
typedef struct {
    double boxMin[3];
    double boxMax[3];
    double rc, skin, sigma, epsilon, cappingDistance;
    int32_t shifted;
    int32_t precision;
    double dt;
    int64_t rebuildInterval;
    double slabCenter[3];
    double atomisticDiameter; /* Slab(center, atomisticRegionDiameter, hybridRegionDiameter, nu) */
    double hybridDiameter;
    int64_t nu;
    double gamma;             /* Langevin friction (zeta) and temperature */
    double temperature;
    uint64_t seed;
    int32_t tfEnabled;
    int32_t useGraph;
    double tfBinWidth, tfTargetDensity, tfModulation, tfSmoothingSigma, tfSmoothingRange;
    int64_t tfSampleInterval, tfUpdateInterval;
    int64_t maxNeighbors;
    int32_t composed;         /* 1: run the composed actions even with unit masses */
    int32_t reserved0;
} mrmd_adress_config;

int mrmd_adress_create(mrmd_ctx* ctx, mrmd_adress** out, const mrmd_adress_config* cfg, int64_t n,
                       const double* pos3, const double* vel3, const double* mass);
int mrmd_adress_destroy(mrmd_ctx* ctx, mrmd_adress* s);
/* Advance nsteps; energies (may be NULL): LJ_IdealGas energy of every step. */
int mrmd_adress_run(mrmd_ctx* ctx, mrmd_adress* s, int64_t nsteps, double* energies);
int mrmd_adress_get_state(mrmd_ctx* ctx, mrmd_adress* s, double* pos3, double* vel3, double* force3);
int mrmd_adress_get_tf(mrmd_ctx* ctx, mrmd_adress* s, double* force, double* density, int64_t* numBins);
int mrmd_adress_set_tf(mrmd_ctx* ctx, mrmd_adress* s, const double* force);
/* [0] steps, [1] rebuilds, [2] molecule list pairs (half list of the composed
 * actions; full-list entries of the batched engine), [3] ghost molecules */
int mrmd_adress_stats(const mrmd_adress* s, int64_t* out4);

/* ------------------------------------------ batched AdResS replicas -- */
/* Many independent single-site AdResS systems (the step of mrmd_adress:
 * LJ_IdealGas::run, LJ_IdealGas.cpp:227-260; VelocityVerletLangevinThermostat,
 * VelocityVerletLangevinThermostat.hpp:48-121; UpdateMolecules + Slab,
 * UpdateMolecules.hpp:24-70; MultiResGhostLayer; ThermodynamicForce
 * apply/sample/update, ThermodynamicForce.cpp:74-96) of different sizes and
 * geometries, advanced together: one launch per phase for all replicas,
 * whole rebuild cycles replayed as CUDA graphs.  Each replica's trajectory
 * is bitwise the one it has when run alone with the same tuning (the force
 * of every molecule is summed over a full list in a fixed order). */
typedef struct mrmd_batch mrmd_batch;
typedef struct {
    int64_t numMolecules;
    double boxMin[3];
    double boxMax[3];
    double slabCenter[3];
    double atomisticDiameter;
    uint64_t seed;            /* Langevin noise key of this replica */
} mrmd_replica_desc;

typedef struct {
    int32_t threadsPerRow;    /* lanes sharing one molecule's neighbour row: 1, 2, 4 or 8 */
    int32_t blockSize;        /* pair-kernel block: 64..1024, multiple of 32 */
    int64_t rebuildInterval;  /* steps between list rebuilds */
    int64_t sortEvery;        /* cell-sort the molecules at every k-th rebuild; 0 = never */
    int64_t graphSteps;       /* steps per CUDA graph (0 = no graphs); a multiple of
                                 rebuildInterval * max(sortEvery, 1) */
    int32_t listLayout;       /* 0 = one full row per molecule (mixed form: all pairs in
                                 double-float); 1 = near and far rows, pairs beyond
                                 1.4 sigma in FP32 (mixed form; the FP64 form treats it
                                 as 0); 2 = 8 x 4 cluster pairs: one warp per 8 molecules,
                                 a row of (4-slot j-cluster, 32-bit pair mask) entries,
                                 threadsPerRow 4 (mixed form: pairs beyond 1.4 sigma in
                                 FP32); its clusters are compact only for molecules in
                                 cell order (sortEvery > 0, or given in cell order) */
    int32_t persistent;       /* 1: inside CUDA graphs, the steps between two rebuilds run
                                 as one persistent cooperative launch (its phases
                                 separated by grid barriers with a time limit; a barrier
                                 that times out makes mrmd_batch_run return
                                 MRMD_ERR_TIMEOUT) */
} mrmd_batch_tuning;

typedef struct {
    double rc, skin, sigma, epsilon, cappingDistance;
    int32_t shifted;
    int32_t precision;        /* MRMD_PREC_FP64 or MRMD_PREC_MIXED */
    double dt;
    double hybridDiameter;
    int64_t nu;
    double gamma, temperature;
    int32_t tfEnabled;
    int32_t compFrozen;       /* 1: no drift-compensation sampling or update; the mean
                                 compensation energies keep their set values (zero) */
    double tfBinWidth, tfTargetDensity, tfModulation, tfSmoothingSigma, tfSmoothingRange;
    int64_t tfSampleInterval, tfUpdateInterval;
    int64_t compSamplingInterval; /* LJ_IdealGas intervals; 0 = the reference's 200 */
    int64_t compUpdateInterval;   /* 0 = the reference's 20000 */
    int64_t initialMaxNeighbors;  /* 0 = measured at creation */
    int64_t initialGhostCapacity; /* 0 = measured at creation */
    mrmd_batch_tuning tuning;
} mrmd_batch_config;

/* pos3/vel3: [sum numMolecules][3], replica after replica. */
int mrmd_batch_create(mrmd_ctx* ctx, mrmd_batch** out, const mrmd_batch_config* cfg, int64_t numReplicas,
                      const mrmd_replica_desc* replicas, const double* pos3, const double* vel3);
int mrmd_batch_destroy(mrmd_ctx* ctx, mrmd_batch* b);
/* Advance nsteps; energies (may be NULL): [nsteps][numReplicas] LJ_IdealGas energies. */
int mrmd_batch_run(mrmd_ctx* ctx, mrmd_batch* b, int64_t nsteps, double* energies);
/* State in the input order ([sum n][3] each, NULL skips). */
int mrmd_batch_get_state(mrmd_ctx* ctx, mrmd_batch* b, double* pos3, double* vel3, double* force3);
/* Thermodynamic-force tables and density counts of all replicas, concatenated;
 * binOffsets [numReplicas + 1]. */
int mrmd_batch_get_tf(mrmd_ctx* ctx, mrmd_batch* b, double* force, double* density, int64_t* binOffsets);
int mrmd_batch_set_tf(mrmd_ctx* ctx, mrmd_batch* b, const double* force);
/* Mean drift-compensation energies [numReplicas][200]. */
int mrmd_batch_get_compensation(mrmd_ctx* ctx, mrmd_batch* b, double* mean);
int mrmd_batch_set_compensation(mrmd_ctx* ctx, mrmd_batch* b, const double* mean);
int mrmd_batch_get_tuning(const mrmd_batch* b, mrmd_batch_tuning* t);
int mrmd_batch_set_tuning(mrmd_ctx* ctx, mrmd_batch* b, const mrmd_batch_tuning* t);
/* Time each candidate tuning (list layout, lanes per row, block size, rebuild
 * interval; then the fastest of those with the persistent step kernel, when
 * the tuning has CUDA graphs) on trialSteps steps from the current state
 * (restored after every trial) and set the fastest.  A rebuild interval longer than the configured one is
 * accepted only if no molecule moved skin/2 away from its position at the
 * last rebuild during the trial.  msPerStep (may be NULL) receives
 * [numCandidates] timings (negative = rejected), candidates (may be NULL) the
 * tunings tried (at most 64). */
int mrmd_batch_autotune(mrmd_ctx* ctx, mrmd_batch* b, int64_t trialSteps, mrmd_batch_tuning* best,
                        double* msPerStep, mrmd_batch_tuning* candidates, int64_t* numCandidates);
/* [0] steps, [1] rebuilds, [2] list pairs, [3] ghosts, [4] graph launches,
 * [5] kernel launches, [6] overflow recoveries, [7] list capacity,
 * [8] ghost capacity, [9] flags (1 ghost overflow, 2 list overflow,
 * 4 a molecule moved skin/2 from its position at the last rebuild) */
int mrmd_batch_stats(mrmd_ctx* ctx, mrmd_batch* b, int64_t* out10);
/* The list of the last rebuild: [0] pairs, [1] entries (one per pair in the
 * per-molecule layouts, one per cluster pair in the cluster layout), [2] pair
 * slots per entry (1 or 32); pairs / (entries * slots) is the fraction of
 * the pair kernel's lanes that evaluate a listed pair. */
int mrmd_batch_list_stats(mrmd_ctx* ctx, mrmd_batch* b, int64_t* out3);
/* The list of the last rebuild of one replica as canonical keys a * 2^32 + b
 * of unordered pairs of the replica's molecules (a < b, indices in the
 * replica's input order; ghosts mapped to their source), one key per pair
 * the force kernel evaluates (per-molecule rows: one per entry; cluster
 * layout: one per set mask bit), sorted.  keys may be NULL to query *count;
 * otherwise cap >= *count keys are written.  For tests and diagnostics. */
int mrmd_batch_pair_keys(mrmd_ctx* ctx, mrmd_batch* b, int64_t replica, int64_t* keys, int64_t cap,
                         int64_t* count);
/* The grid barrier of the persistent step kernel on its own: `rounds`
 * barriers of one cooperative launch; block skipBlock (>= 0) never arrives,
 * so the others give up after limitMs and the call returns MRMD_ERR_TIMEOUT
 * (-1: every block arrives, MRMD_OK).  For tests of the time limit. */
int mrmd_grid_sync_selftest(mrmd_ctx* ctx, int32_t rounds, int32_t skipBlock, double limitMs);

/* ------------------------------------------------- differentiation -- */
/* Gradient of a trajectory loss of one AdResS system (the batched engine with
 * one replica) by a hand-written adjoint of the weighted pair force
 * (LJ_IdealGas.cpp:52-225, drift and compensation forces included), of the
 * thermodynamic force (ThermodynamicForce.hpp:98-122) and of the Langevin
 * velocity-Verlet step, with a checkpoint every checkpointInterval steps and
 * recomputation.  The loss is sum_b (rho_b - rho_uniform)^2 of the x-density
 * smoothed by a Gaussian of width lossSigma on lossBins bin centres and
 * averaged over the last `window` steps.  The compensation means are held
 * fixed and the TF table is not updated inside the trajectory; the table and
 * the LJ epsilon and sigma are the parameters.  The reference has no
 * differentiation. */
typedef struct mrmd_diff mrmd_diff;
typedef struct {
    int64_t steps;
    int64_t window;
    int64_t checkpointInterval; /* a multiple of the rebuild interval */
    int64_t lossBins;
    double lossSigma;
} mrmd_diff_config;

int mrmd_diff_create(mrmd_ctx* ctx, mrmd_diff** out, const mrmd_batch_config* cfg, const mrmd_replica_desc* replica,
                     const double* pos3, const double* vel3, const mrmd_diff_config* dc);
int mrmd_diff_destroy(mrmd_ctx* ctx, mrmd_diff* d);
int mrmd_diff_num_bins(const mrmd_diff* d, int64_t* tfBins);
/* Replace the initial state (positions, velocities; forces start at zero). */
int mrmd_diff_set_state(mrmd_ctx* ctx, mrmd_diff* d, const double* pos3, const double* vel3);
/* Run the trajectory with the given TF table (NULL keeps the current one),
 * epsilon and sigma; returns the loss and keeps the checkpoints. */
int mrmd_diff_forward(mrmd_ctx* ctx, mrmd_diff* d, const double* tfTable, double epsilon, double sigma,
                      double* loss);
/* dLoss/dtable [tfBins], dLoss/depsilon, dLoss/dsigma of the last forward. */
int mrmd_diff_backward(mrmd_ctx* ctx, mrmd_diff* d, double* gradTable, double* gradEpsilon, double* gradSigma);
/* One force evaluation at the initial state and its vector-Jacobian product
 * with adjoint3: force3 = F, xbar3 = (dF/dx)^T a, grads = (dF/dtheta)^T a. */
int mrmd_diff_force_vjp(mrmd_ctx* ctx, mrmd_diff* d, const double* tfTable, double epsilon, double sigma,
                        const double* adjoint3, double* force3, double* xbar3, double* gradTable,
                        double* gradEpsilon, double* gradSigma);
/* State at the end of the last forward run (input order). */
int mrmd_diff_get_state(mrmd_ctx* ctx, mrmd_diff* d, double* pos3, double* vel3);

#ifdef __cplusplus
}
#endif
#endif
