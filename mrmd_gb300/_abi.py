"""ctypes binding of the C ABI declared in include/mrmd_gb300.h.

The library is the in-tree ``mrmd_gb300/libmrmd_gb300.so`` built by
``mrmd_gb300/build.py``; there is no fallback: a missing or unloadable
library raises ``MrmdError``.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# MRMD_GB300_BOUNDS_CHECK=1 loads the bounds-checked debug build instead
# (python -m mrmd_gb300.build --bounds-check).
LIB_PATH = os.path.join(_HERE, "libmrmd_gb300_bounds.so" if os.environ.get("MRMD_GB300_BOUNDS_CHECK") == "1"
                        else "libmrmd_gb300.so")

c_double_p = C.POINTER(C.c_double)
c_int64_p = C.POINTER(C.c_int64)
c_int32_p = C.POINTER(C.c_int32)

MRMD_OK = 0
ERRORS = {
    -1: "MRMD_ERR_ARG", -2: "MRMD_ERR_OOM", -3: "MRMD_ERR_NLIST_OVERFLOW", -4: "MRMD_ERR_NONFINITE",
    -5: "MRMD_ERR_TIMEOUT", -6: "MRMD_ERR_CUDA", -7: "MRMD_ERR_STATE", -8: "MRMD_ERR_CAPACITY",
    -9: "MRMD_ERR_BOUNDS",
}
PREC_FP64, PREC_MIXED = 0, 1
PRED_ALWAYS, PRED_EITHER_IN_SLAB, PRED_BOTH_IN_SLAB, PRED_IN_SLAB, PRED_IN_OPEN_INTERVAL = range(5)


class MrmdError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


class Pred(C.Structure):
    _fields_ = [("kind", C.c_int32), ("axis", C.c_int32), ("center", C.c_double),
                ("slabMin", C.c_double), ("slabMax", C.c_double), ("tolerance", C.c_double)]


class AtomsS(C.Structure):
    _fields_ = [("pos", c_double_p), ("vel", c_double_p), ("force", c_double_p),
                ("type", c_int32_p), ("mass", c_double_p), ("charge", c_double_p),
                ("relativeMass", c_double_p), ("numLocal", C.c_int64), ("numGhost", C.c_int64),
                ("capacity", C.c_int64)]


class MoleculesS(C.Structure):
    _fields_ = [("pos", c_double_p), ("force", c_double_p), ("lambda_", c_double_p),
                ("modulatedLambda", c_double_p), ("gradLambda", c_double_p),
                ("atomsOffset", c_int64_p), ("numAtoms", c_int64_p), ("numLocal", C.c_int64),
                ("numGhost", C.c_int64), ("capacity", C.c_int64)]


class SubdomainS(C.Structure):
    _fields_ = [(n, C.c_double * 3) for n in (
        "minCorner", "maxCorner", "ghostLayerThickness", "minGhostCorner", "maxGhostCorner",
        "minInnerCorner", "maxInnerCorner", "diameter", "diameterWithGhostLayer")]


class GhostLayerS(C.Structure):
    _fields_ = [("correspondingRealAtom", c_int32_p), ("capacity", C.c_int64),
                ("numLocal", C.c_int64), ("numGhost", C.c_int64), ("ghostStart", c_int32_p),
                ("ghostList", c_int32_p), ("localCapacity", C.c_int64)]


class NListS(C.Structure):
    _fields_ = [("counts", c_int32_p), ("nbrs", c_int32_p), ("rows", C.c_int64),
                ("begin", C.c_int64), ("stride", C.c_int64), ("maxNeighbors", C.c_int64),
                ("rowsCapacity", C.c_int64), ("nbrsCapacity", C.c_int64),
                ("totalPairs", C.c_int64), ("cells", C.c_void_p)]


class LJParamsS(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "ff1", "ff2", "ef1", "ef2", "rcSqr", "cappingDistance", "cappingDistanceSqr",
        "cappingCoeff", "shift", "energyAtCappingPoint")]


class SlabS(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("atomisticRegionDiameter", C.c_double),
                ("hybridRegionDiameter", C.c_double), ("nu", C.c_int64),
                ("interfaceType", C.c_int32), ("pad", C.c_int32)]


class CoulombDSFS(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha", "rc", "rcSqr", "forceShift", "energyShift")]


class MDConfigS(C.Structure):
    _fields_ = [("boxMin", C.c_double * 3), ("boxMax", C.c_double * 3), ("rc", C.c_double),
                ("skin", C.c_double), ("sigma", C.c_double), ("epsilon", C.c_double),
                ("cappingDistance", C.c_double), ("shifted", C.c_int32),
                ("precision", C.c_int32), ("dt", C.c_double), ("rebuildInterval", C.c_int64),
                ("useGraph", C.c_int32), ("sortAtoms", C.c_int32), ("maxNeighbors", C.c_int64),
                ("observe", C.c_int32), ("gatherNeighbours", C.c_int32), ("splitRadius", C.c_double),
                ("tileBuild", C.c_int32), ("reserved0", C.c_int32)]


class AdResSConfigS(C.Structure):
    _fields_ = [("boxMin", C.c_double * 3), ("boxMax", C.c_double * 3), ("rc", C.c_double),
                ("skin", C.c_double), ("sigma", C.c_double), ("epsilon", C.c_double),
                ("cappingDistance", C.c_double), ("shifted", C.c_int32), ("precision", C.c_int32),
                ("dt", C.c_double), ("rebuildInterval", C.c_int64), ("slabCenter", C.c_double * 3),
                ("atomisticDiameter", C.c_double), ("hybridDiameter", C.c_double), ("nu", C.c_int64),
                ("gamma", C.c_double), ("temperature", C.c_double), ("seed", C.c_uint64),
                ("tfEnabled", C.c_int32), ("useGraph", C.c_int32), ("tfBinWidth", C.c_double),
                ("tfTargetDensity", C.c_double), ("tfModulation", C.c_double),
                ("tfSmoothingSigma", C.c_double), ("tfSmoothingRange", C.c_double),
                ("tfSampleInterval", C.c_int64), ("tfUpdateInterval", C.c_int64),
                ("maxNeighbors", C.c_int64), ("composed", C.c_int32), ("reserved0", C.c_int32)]


class ReplicaS(C.Structure):
    _fields_ = [("numMolecules", C.c_int64), ("boxMin", C.c_double * 3), ("boxMax", C.c_double * 3),
                ("slabCenter", C.c_double * 3), ("atomisticDiameter", C.c_double), ("seed", C.c_uint64)]


class BatchTuningS(C.Structure):
    _fields_ = [("threadsPerRow", C.c_int32), ("blockSize", C.c_int32), ("rebuildInterval", C.c_int64),
                ("sortEvery", C.c_int64), ("graphSteps", C.c_int64), ("listLayout", C.c_int32),
                ("persistent", C.c_int32)]


class BatchConfigS(C.Structure):
    _fields_ = [("rc", C.c_double), ("skin", C.c_double), ("sigma", C.c_double), ("epsilon", C.c_double),
                ("cappingDistance", C.c_double), ("shifted", C.c_int32), ("precision", C.c_int32),
                ("dt", C.c_double), ("hybridDiameter", C.c_double), ("nu", C.c_int64),
                ("gamma", C.c_double), ("temperature", C.c_double), ("tfEnabled", C.c_int32),
                ("compFrozen", C.c_int32), ("tfBinWidth", C.c_double), ("tfTargetDensity", C.c_double),
                ("tfModulation", C.c_double), ("tfSmoothingSigma", C.c_double),
                ("tfSmoothingRange", C.c_double), ("tfSampleInterval", C.c_int64),
                ("tfUpdateInterval", C.c_int64), ("compSamplingInterval", C.c_int64),
                ("compUpdateInterval", C.c_int64), ("initialMaxNeighbors", C.c_int64),
                ("initialGhostCapacity", C.c_int64), ("tuning", BatchTuningS)]


class DiffConfigS(C.Structure):
    _fields_ = [("steps", C.c_int64), ("window", C.c_int64), ("checkpointInterval", C.c_int64),
                ("lossBins", C.c_int64), ("lossSigma", C.c_double)]


P = C.POINTER
_v = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_u64 = C.c_uint64
_d = C.c_double

# name: (restype, argtypes)
SIGNATURES = {
    "mrmd_version": (C.c_char_p, []),
    "mrmd_ctx_create": (_i, [P(_v), _i]),
    "mrmd_ctx_destroy": (_i, [_v]),
    "mrmd_ctx_sync": (_i, [_v]),
    "mrmd_ctx_set_sync": (_i, [_v, _i]),
    "mrmd_ctx_stream": (_v, [_v]),
    "mrmd_ctx_last_error": (C.c_char_p, [_v]),
    "mrmd_bounds_checked": (_i, []),
    "mrmd_ctx_launch_count": (_i64, [_v]),
    "mrmd_atoms_alloc": (_i, [_v, P(AtomsS), _i64]),
    "mrmd_atoms_free": (_i, [_v, P(AtomsS)]),
    "mrmd_atoms_reserve": (_i, [_v, P(AtomsS), _i64]),
    "mrmd_atoms_upload": (_i, [_v, P(AtomsS), _i64, _i64, c_double_p, c_double_p, c_double_p,
                               c_int64_p, c_double_p, c_double_p, c_double_p]),
    "mrmd_atoms_download": (_i, [_v, P(AtomsS), _i64, c_double_p, c_double_p, c_double_p,
                                 c_int64_p, c_double_p, c_double_p, c_double_p]),
    "mrmd_atoms_set_force": (_i, [_v, P(AtomsS), _i64, _d]),
    "mrmd_atoms_sort_by_cell": (_i, [_v, P(AtomsS), c_double_p, c_double_p, _d, c_int64_p]),
    "mrmd_molecules_alloc": (_i, [_v, P(MoleculesS), _i64]),
    "mrmd_molecules_free": (_i, [_v, P(MoleculesS)]),
    "mrmd_molecules_reserve": (_i, [_v, P(MoleculesS), _i64]),
    "mrmd_molecules_upload": (_i, [_v, P(MoleculesS), _i64, _i64, c_double_p, c_double_p,
                                   c_double_p, c_double_p, c_double_p, c_int64_p, c_int64_p]),
    "mrmd_molecules_download": (_i, [_v, P(MoleculesS), _i64, c_double_p, c_double_p, c_double_p,
                                     c_double_p, c_double_p, c_int64_p, c_int64_p]),
    "mrmd_molecules_set_force": (_i, [_v, P(MoleculesS), _i64, _d]),
    "mrmd_subdomain_init": (_i, [P(SubdomainS), c_double_p, c_double_p, c_double_p]),
    "mrmd_ghost_layer_alloc": (_i, [_v, P(GhostLayerS), _i64]),
    "mrmd_ghost_layer_free": (_i, [_v, P(GhostLayerS)]),
    "mrmd_ghost_exchange_real_atoms": (_i, [_v, P(AtomsS), P(SubdomainS)]),
    "mrmd_ghost_create": (_i, [_v, P(GhostLayerS), P(AtomsS), P(SubdomainS)]),
    "mrmd_ghost_update": (_i, [_v, P(GhostLayerS), P(AtomsS), P(SubdomainS)]),
    "mrmd_ghost_reduce_force": (_i, [_v, P(GhostLayerS), P(AtomsS)]),
    "mrmd_multires_exchange_real_atoms": (_i, [_v, P(MoleculesS), P(AtomsS), P(SubdomainS)]),
    "mrmd_multires_ghost_create": (_i, [_v, P(GhostLayerS), P(MoleculesS), P(AtomsS),
                                        P(SubdomainS)]),
    "mrmd_ghost_layer_download": (_i, [_v, P(GhostLayerS), _i64, c_int64_p]),
    "mrmd_nlist_init": (_i, [_v, P(NListS)]),
    "mrmd_nlist_free": (_i, [_v, P(NListS)]),
    "mrmd_nlist_build": (_i, [_v, P(NListS), c_double_p, _i64, _i64, _i64, _d, _d, c_double_p,
                              c_double_p, _i64]),
    "mrmd_nlist_download": (_i, [_v, P(NListS), c_int32_p, c_int32_p, _i64]),
    "mrmd_cell_index": (_i, [_v, c_double_p, _i64, c_double_p, c_double_p, _d, c_int64_p]),
    "mrmd_lj_create": (_i, [_v, P(_v), _i64, _i64, c_double_p, c_double_p, c_double_p,
                            c_double_p, _i]),
    "mrmd_lj_destroy": (_i, [_v, _v]),
    "mrmd_lj_get_params": (_i, [_v, P(LJParamsS), _i64]),
    "mrmd_lj_apply": (_i, [_v, _v, P(AtomsS), P(NListS), P(Pred), _i, c_double_p, c_double_p]),
    "mrmd_lj_apply_mixed_noalloc": (_i, [_v, _v, P(AtomsS), P(NListS), P(Pred), c_double_p, c_double_p]),
    "mrmd_vv_pre": (_i, [_v, P(AtomsS), _d, c_double_p]),
    "mrmd_vv_post": (_i, [_v, P(AtomsS), _d]),
    "mrmd_langevin_pre": (_i, [_v, P(AtomsS), _d, _d, _d, _u64, _u64, P(Pred), c_double_p]),
    "mrmd_update_molecules": (_i, [_v, P(MoleculesS), P(AtomsS), P(SlabS)]),
    "mrmd_contribute_molecule_force": (_i, [_v, P(MoleculesS), P(AtomsS)]),
    "mrmd_ljig_create": (_i, [_v, P(_v), _i64, c_double_p, c_double_p, c_double_p, c_double_p,
                              _i]),
    "mrmd_ljig_destroy": (_i, [_v, _v]),
    "mrmd_ljig_set_intervals": (_i, [_v, _i64, _i64]),
    "mrmd_ljig_run": (_i, [_v, _v, P(MoleculesS), P(NListS), P(AtomsS), _i, c_double_p]),
    "mrmd_ljig_get_compensation": (_i, [_v, _v, c_double_p, c_double_p, c_double_p, c_int64_p]),
    "mrmd_ljig_set_compensation": (_i, [_v, _v, c_double_p]),
    "mrmd_tf_create": (_i, [_v, P(_v), _i64, c_double_p, P(SubdomainS), _d, c_double_p, _i, _i]),
    "mrmd_tf_destroy": (_i, [_v, _v]),
    "mrmd_tf_shape": (_i, [_v, c_int64_p, c_double_p, c_int64_p]),
    "mrmd_tf_sample": (_i, [_v, _v, P(AtomsS)]),
    "mrmd_tf_apply": (_i, [_v, _v, P(AtomsS), P(Pred), _i]),
    "mrmd_tf_update": (_i, [_v, _v, _d, _d, P(Pred)]),
    "mrmd_tf_get_force": (_i, [_v, _v, c_double_p]),
    "mrmd_tf_set_force": (_i, [_v, _v, c_double_p]),
    "mrmd_tf_get_density": (_i, [_v, _v, c_double_p, c_int64_p]),
    "mrmd_tf_mu": (_i, [_v, _v, c_double_p, c_double_p]),
    "mrmd_tf_grid": (_i, [_v, c_double_p]),
    "mrmd_tf_write_table": (_i, [_v, C.c_char_p, _i64, c_double_p, _i64, c_double_p, _i64]),
    "mrmd_tf_read_table": (_i, [_v, C.c_char_p, _i64, c_int64_p, c_int64_p, c_double_p, c_double_p,
                                c_double_p, _i64]),
    "mrmd_tf_dump": (_i, [_v, _v, C.c_char_p, _i64]),
    "mrmd_tf_restore": (_i, [_v, P(_v), C.c_char_p, P(SubdomainS), _i64, c_double_p, c_double_p, _i, _i,
                             _i64]),
    "mrmd_md_create": (_i, [_v, P(_v), P(MDConfigS), _i64, c_double_p, c_double_p, c_double_p]),
    "mrmd_md_destroy": (_i, [_v, _v]),
    "mrmd_md_run": (_i, [_v, _v, _i64, c_double_p]),
    "mrmd_md_run_observed": (_i, [_v, _v, _i64, c_double_p]),
    "mrmd_coulomb_dsf_init": (_i, [P(CoulombDSFS), _d, _d]),
    "mrmd_coulomb_dsf_eval": (_i, [_v, P(CoulombDSFS), _i64, c_double_p, c_double_p, c_double_p, c_double_p,
                                   c_double_p]),
    "mrmd_coulomb_dsf_apply": (_i, [_v, P(CoulombDSFS), P(AtomsS), P(NListS), c_double_p, c_double_p]),
    "mrmd_kinetic_energy": (_i, [_v, P(AtomsS), c_double_p]),
    "mrmd_system_momentum": (_i, [_v, P(AtomsS), c_double_p]),
    "mrmd_pressure": (_i, [_v, P(AtomsS), P(SubdomainS), c_double_p]),
    "mrmd_md_get_state": (_i, [_v, _v, c_double_p, c_double_p, c_double_p]),
    "mrmd_md_set_state": (_i, [_v, _v, c_double_p, c_double_p]),
    "mrmd_md_stats": (_i, [_v, c_int64_p]),
    "mrmd_md_eval": (_i, [_v, _v, _i, c_double_p]),
    "mrmd_adress_create": (_i, [_v, P(_v), P(AdResSConfigS), _i64, c_double_p, c_double_p,
                                c_double_p]),
    "mrmd_adress_destroy": (_i, [_v, _v]),
    "mrmd_adress_run": (_i, [_v, _v, _i64, c_double_p]),
    "mrmd_adress_get_state": (_i, [_v, _v, c_double_p, c_double_p, c_double_p]),
    "mrmd_adress_get_tf": (_i, [_v, _v, c_double_p, c_double_p, c_int64_p]),
    "mrmd_adress_set_tf": (_i, [_v, _v, c_double_p]),
    "mrmd_adress_stats": (_i, [_v, c_int64_p]),
    "mrmd_batch_create": (_i, [_v, P(_v), P(BatchConfigS), _i64, P(ReplicaS), c_double_p, c_double_p]),
    "mrmd_batch_destroy": (_i, [_v, _v]),
    "mrmd_batch_run": (_i, [_v, _v, _i64, c_double_p]),
    "mrmd_batch_get_state": (_i, [_v, _v, c_double_p, c_double_p, c_double_p]),
    "mrmd_batch_get_tf": (_i, [_v, _v, c_double_p, c_double_p, c_int64_p]),
    "mrmd_batch_set_tf": (_i, [_v, _v, c_double_p]),
    "mrmd_batch_get_compensation": (_i, [_v, _v, c_double_p]),
    "mrmd_batch_set_compensation": (_i, [_v, _v, c_double_p]),
    "mrmd_batch_get_tuning": (_i, [_v, P(BatchTuningS)]),
    "mrmd_batch_set_tuning": (_i, [_v, _v, P(BatchTuningS)]),
    "mrmd_batch_autotune": (_i, [_v, _v, _i64, P(BatchTuningS), c_double_p, P(BatchTuningS), c_int64_p]),
    "mrmd_batch_stats": (_i, [_v, _v, c_int64_p]),
    "mrmd_batch_list_stats": (_i, [_v, _v, c_int64_p]),
    "mrmd_diff_create": (_i, [_v, P(_v), P(BatchConfigS), P(ReplicaS), c_double_p, c_double_p,
                              P(DiffConfigS)]),
    "mrmd_diff_destroy": (_i, [_v, _v]),
    "mrmd_diff_num_bins": (_i, [_v, c_int64_p]),
    "mrmd_diff_set_state": (_i, [_v, _v, c_double_p, c_double_p]),
    "mrmd_diff_forward": (_i, [_v, _v, c_double_p, _d, _d, c_double_p]),
    "mrmd_diff_backward": (_i, [_v, _v, c_double_p, c_double_p, c_double_p]),
    "mrmd_diff_force_vjp": (_i, [_v, _v, c_double_p, _d, _d, c_double_p, c_double_p, c_double_p, c_double_p,
                                 c_double_p, c_double_p]),
    "mrmd_diff_get_state": (_i, [_v, _v, c_double_p, c_double_p]),
    "mrmd_md_atoms": (P(AtomsS), [_v]),
    "mrmd_md_nlist": (P(NListS), [_v]),
    "mrmd_md_tile_stats": (_i, [_v, c_int64_p]),
    "mrmd_md_pair_keys": (_i, [_v, _v, c_int64_p, _i64, c_int64_p]),
    "mrmd_batch_pair_keys": (_i, [_v, _v, _i64, c_int64_p, _i64, c_int64_p]),
    "mrmd_grid_sync_selftest": (_i, [_v, C.c_int32, C.c_int32, C.c_double]),
}

_lib = None


def lib():
    """Load the library (raises MrmdError when it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MrmdError(-6, f"{LIB_PATH} is not built (run mrmd_gb300/build.py)")
        try:
            L = C.CDLL(LIB_PATH)
        except OSError as e:  # pragma: no cover - depends on the machine
            raise MrmdError(-6, f"cannot load {LIB_PATH}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(SIGNATURES)
