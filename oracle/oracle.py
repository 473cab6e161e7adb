"""ctypes view of the CPU oracle (oracle/mrmd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker and by ``bench.py``'s CPU-baseline leg.  The product package
``mrmd_gb300`` never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmrmd_oracle.so")

c_double_p = C.POINTER(C.c_double)
c_int64_p = C.POINTER(C.c_int64)
c_int32_p = C.POINTER(C.c_int32)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (plain gcc)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("mrmd_oracle.c", "mrmd_oracle.h")
    ):
        subprocess.run(["make", "-C", _HERE, "-s"], check=True)
    return _LIB_PATH


class Subdomain(C.Structure):
    _fields_ = [(n, C.c_double * 3) for n in (
        "minCorner", "maxCorner", "ghostLayerThickness", "minGhostCorner", "maxGhostCorner",
        "minInnerCorner", "maxInnerCorner", "diameter", "diameterWithGhostLayer")]


class AtomsS(C.Structure):
    _fields_ = [("pos", c_double_p), ("vel", c_double_p), ("force", c_double_p),
                ("type", c_int64_p), ("mass", c_double_p), ("charge", c_double_p),
                ("relativeMass", c_double_p), ("numLocal", C.c_int64), ("numGhost", C.c_int64),
                ("capacity", C.c_int64)]


class MoleculesS(C.Structure):
    _fields_ = [("pos", c_double_p), ("force", c_double_p), ("lambda_", c_double_p),
                ("modulatedLambda", c_double_p), ("gradLambda", c_double_p),
                ("atomsOffset", c_int64_p), ("numAtoms", c_int64_p), ("numLocal", C.c_int64),
                ("numGhost", C.c_int64), ("capacity", C.c_int64)]


class LJParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "ff1", "ff2", "ef1", "ef2", "rcSqr", "cappingDistance", "cappingDistanceSqr",
        "cappingCoeff", "shift", "energyAtCappingPoint")]


class CoulombDSFS(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha", "rc", "rcSqr", "forceShift", "energyShift")]


class Pred(C.Structure):
    _fields_ = [("kind", C.c_int32), ("axis", C.c_int32), ("center", C.c_double),
                ("slabMin", C.c_double), ("slabMax", C.c_double), ("tolerance", C.c_double)]


class SlabS(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("atomisticRegionHalfDiameter", C.c_double),
                ("hybridRegionDiameter", C.c_double), ("exponent", C.c_int64),
                ("interfaceType", C.c_int32), ("pad", C.c_int32)]


class LJIG(C.Structure):
    _fields_ = [("table", C.POINTER(LJParams)), ("numTypes", C.c_int64), ("rcSqr", C.c_double),
                ("compensationEnergy", c_double_p), ("compensationEnergyCounter", c_double_p),
                ("meanCompensationEnergy", c_double_p), ("runCounter", C.c_int64),
                ("samplingInterval", C.c_int64), ("updateInterval", C.c_int64)]


class Hist(C.Structure):
    _fields_ = [("min", C.c_double), ("max", C.c_double), ("numBins", C.c_int64),
                ("numHist", C.c_int64), ("binSize", C.c_double), ("inverseBinSize", C.c_double),
                ("data", c_double_p)]


class TF(C.Structure):
    _fields_ = [("force", Hist), ("density", Hist), ("samples", C.c_int64),
                ("binVolume", C.c_double), ("forceFactor", c_double_p),
                ("enforceSymmetry", C.c_int32), ("usePeriodicity", C.c_int32)]


PRED_ALWAYS, PRED_EITHER_IN_SLAB, PRED_BOTH_IN_SLAB, PRED_IN_SLAB, PRED_IN_OPEN_INTERVAL = range(5)


def _p(a: np.ndarray, t=c_double_p):
    return a.ctypes.data_as(t)


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_subdomain_init.argtypes = [C.POINTER(Subdomain), c_double_p, c_double_p, c_double_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        L.orc_get_max_threads.restype = C.c_int
        L.orc_lj_init.argtypes = [C.POINTER(LJParams), C.c_int64, c_double_p, c_double_p,
                                  c_double_p, c_double_p, C.c_int]
        L.orc_lj_force_energy.argtypes = [C.POINTER(LJParams), C.c_double, C.c_int64, c_double_p,
                                          c_double_p]
        L.orc_lj_apply.argtypes = [C.POINTER(LJParams), C.c_int64, C.c_double, C.POINTER(AtomsS),
                                   c_int32_p, c_int32_p, C.c_int64, C.POINTER(Pred), c_double_p,
                                   c_double_p]
        L.orc_map_into_domain.argtypes = [C.POINTER(AtomsS), C.POINTER(Subdomain)]
        L.orc_create_ghosts_xyz.argtypes = [C.POINTER(AtomsS), C.POINTER(Subdomain), c_int64_p]
        L.orc_create_ghosts_xyz.restype = C.c_int64
        L.orc_update_ghosts.argtypes = [C.POINTER(AtomsS), c_int64_p, C.POINTER(Subdomain)]
        L.orc_ghost_to_real.argtypes = [C.POINTER(AtomsS), c_int64_p]
        L.orc_cell_grid.argtypes = [c_double_p, c_double_p, C.c_double, c_int64_p, c_double_p]
        L.orc_cell_index.argtypes = [c_double_p, C.c_int64, c_double_p, c_int64_p, c_double_p,
                                     c_int64_p]
        L.orc_build_half_list.argtypes = [c_double_p, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                                          C.c_double, c_double_p, c_double_p, c_int32_p,
                                          c_int32_p, C.c_int64]
        L.orc_build_half_list.restype = C.c_int64
        L.orc_count_within.argtypes = [c_double_p, C.c_int64, C.c_int64, C.c_double, c_double_p,
                                       C.c_int]
        L.orc_count_within.restype = C.c_int64
        L.orc_vv_pre.argtypes = [C.POINTER(AtomsS), C.c_double]
        L.orc_vv_pre.restype = C.c_double
        L.orc_vv_post.argtypes = [C.POINTER(AtomsS), C.c_double]
        L.orc_coulomb_dsf_init.argtypes = [C.POINTER(CoulombDSFS), C.c_double, C.c_double]
        L.orc_approx_erfc.argtypes = [C.c_double, c_double_p]
        L.orc_approx_erfc.restype = C.c_double
        for f in ("orc_coulomb_dsf_force", "orc_coulomb_dsf_energy"):
            getattr(L, f).argtypes = [C.POINTER(CoulombDSFS), C.c_double, C.c_double, C.c_double]
            getattr(L, f).restype = C.c_double
        L.orc_coulomb_dsf_apply.argtypes = [C.POINTER(CoulombDSFS), C.POINTER(AtomsS), c_int32_p,
                                            c_int32_p, C.c_int64, c_double_p, c_double_p]
        L.orc_kinetic_energy.argtypes = [C.POINTER(AtomsS)]
        L.orc_kinetic_energy.restype = C.c_double
        L.orc_system_momentum.argtypes = [C.POINTER(AtomsS), c_double_p]
        L.orc_pressure.argtypes = [C.POINTER(AtomsS), C.POINTER(Subdomain)]
        L.orc_pressure.restype = C.c_double
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
        L.orc_normal_from_counter.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, c_double_p]
        L.orc_langevin_pre.argtypes = [C.POINTER(AtomsS), C.c_double, C.c_double, C.c_double,
                                       C.c_uint64, C.c_uint64, C.POINTER(Pred)]
        L.orc_langevin_pre.restype = C.c_double
        L.orc_slab_init.argtypes = [C.POINTER(SlabS), c_double_p, C.c_double, C.c_double,
                                    C.c_int64, C.c_int32]
        L.orc_slab_eval.argtypes = [C.POINTER(SlabS), C.c_double, C.c_double, C.c_double,
                                    c_double_p]
        L.orc_update_molecules.argtypes = [C.POINTER(MoleculesS), C.POINTER(AtomsS),
                                           C.POINTER(SlabS)]
        L.orc_contribute_molecule_force.argtypes = [C.POINTER(MoleculesS), C.POINTER(AtomsS)]
        L.orc_ljig_run.argtypes = [C.POINTER(LJIG), C.POINTER(MoleculesS), c_int32_p, c_int32_p,
                                   C.c_int64, C.POINTER(AtomsS)]
        L.orc_ljig_run.restype = C.c_double
        L.orc_update_mean_compensation_energy.argtypes = [c_double_p, c_double_p, c_double_p,
                                                          C.c_int64, C.c_int64, C.c_double]
        L.orc_multires_map_into_domain.argtypes = [C.POINTER(Subdomain), C.POINTER(MoleculesS),
                                                   C.POINTER(AtomsS)]
        L.orc_multires_create_ghosts_xyz.argtypes = [C.POINTER(MoleculesS), C.POINTER(AtomsS),
                                                     C.POINTER(Subdomain), c_int64_p]
        L.orc_multires_create_ghosts_xyz.restype = C.c_int64
        L.orc_hist_init.argtypes = [C.POINTER(Hist), C.c_double, C.c_double, C.c_int64, C.c_int64,
                                    c_double_p]
        L.orc_hist_get_bin.argtypes = [C.POINTER(Hist), C.c_double]
        L.orc_hist_get_bin.restype = C.c_int64
        L.orc_hist_bin_position.argtypes = [C.POINTER(Hist), C.c_int64]
        L.orc_hist_bin_position.restype = C.c_double
        L.orc_hist_scale.argtypes = [C.POINTER(Hist), C.c_double]
        L.orc_hist_scale_per_hist.argtypes = [C.POINTER(Hist), c_double_p]
        L.orc_hist_make_symmetric.argtypes = [C.POINTER(Hist)]
        L.orc_hist_gradient.argtypes = [C.POINTER(Hist), C.POINTER(Hist), C.c_int]
        L.orc_hist_smoothen.argtypes = [C.POINTER(Hist), C.POINTER(Hist), C.c_double, C.c_double,
                                        C.c_int]
        L.orc_hist_replace_if.argtypes = [C.POINTER(Hist), C.POINTER(Pred), C.c_int, C.c_double]
        L.orc_cumulative_moving_average.argtypes = [C.POINTER(Hist), C.POINTER(Hist), C.c_double]
        L.orc_axial_density_profile.argtypes = [C.POINTER(AtomsS), C.c_int64, C.POINTER(Hist),
                                                C.c_int]
        L.orc_tf_num_bins.argtypes = [C.POINTER(Subdomain), C.c_double]
        L.orc_tf_num_bins.restype = C.c_int64
        L.orc_tf_init.argtypes = [C.POINTER(TF), C.POINTER(Subdomain), C.c_int64, C.c_int64,
                                  c_double_p, c_double_p, c_double_p, c_double_p, c_double_p,
                                  C.c_int, C.c_int]
        L.orc_tf_sample.argtypes = [C.POINTER(TF), C.POINTER(AtomsS)]
        L.orc_tf_apply.argtypes = [C.POINTER(TF), C.POINTER(AtomsS), C.POINTER(Pred)]
        L.orc_tf_apply_interpolated.argtypes = [C.POINTER(TF), C.POINTER(AtomsS), C.POINTER(Pred)]
        L.orc_tf_update.argtypes = [C.POINTER(TF), C.c_double, C.c_double, C.POINTER(Pred),
                                    c_double_p]
        L.orc_tf_update.restype = C.c_int
        L.orc_tf_mu.argtypes = [C.POINTER(TF), c_double_p, c_double_p]
    return _lib


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def max_threads() -> int:
    return lib().orc_get_max_threads()


# ------------------------------------------------------------------ helpers --

def subdomain(min_corner, max_corner, ghost) -> Subdomain:
    if np.isscalar(ghost):
        ghost = (ghost, ghost, ghost)
    sd = Subdomain()
    a = np.asarray(min_corner, dtype=np.float64)
    b = np.asarray(max_corner, dtype=np.float64)
    g = np.asarray(ghost, dtype=np.float64)
    lib().orc_subdomain_init(C.byref(sd), _p(a), _p(b), _p(g))
    return sd


def pred(kind=PRED_ALWAYS, axis=0, center=0.0, slab_min=0.0, slab_max=0.0, tolerance=0.0) -> Pred:
    return Pred(kind, axis, center, slab_min, slab_max, tolerance)


class Atoms:
    """Numpy-backed atoms in the reference's AoS layout (data/Atoms.hpp:47-53)."""

    def __init__(self, capacity: int):
        capacity = max(int(capacity), 1)
        self.pos = np.zeros((capacity, 3))
        self.vel = np.zeros((capacity, 3))
        self.force = np.zeros((capacity, 3))
        self.type = np.zeros(capacity, dtype=np.int64)
        self.mass = np.zeros(capacity)
        self.charge = np.zeros(capacity)
        self.relativeMass = np.zeros(capacity)
        self.numLocal = 0
        self.numGhost = 0

    @property
    def capacity(self) -> int:
        return self.pos.shape[0]

    @classmethod
    def from_positions(cls, pos, capacity=None, mass=1.0):
        pos = np.asarray(pos, dtype=np.float64)
        a = cls(capacity or max(len(pos) * 2, 64))
        a.pos[: len(pos)] = pos
        a.mass[: len(pos)] = mass
        a.relativeMass[: len(pos)] = 1.0
        a.numLocal = len(pos)
        return a

    def grow(self, capacity: int):
        old = self.capacity
        if capacity <= old:
            return
        for name in ("pos", "vel", "force", "type", "mass", "charge", "relativeMass"):
            arr = getattr(self, name)
            new = np.zeros((capacity,) + arr.shape[1:], dtype=arr.dtype)
            new[:old] = arr
            setattr(self, name, new)

    def s(self) -> AtomsS:
        return AtomsS(_p(self.pos), _p(self.vel), _p(self.force), _p(self.type, c_int64_p),
                      _p(self.mass), _p(self.charge), _p(self.relativeMass), self.numLocal,
                      self.numGhost, self.capacity)

    def sync(self, s: AtomsS):
        self.numLocal, self.numGhost = s.numLocal, s.numGhost

    @property
    def n(self) -> int:
        return self.numLocal + self.numGhost


class Molecules:
    """Numpy-backed molecules (data/Molecules.hpp:41-47)."""

    def __init__(self, capacity: int):
        capacity = max(int(capacity), 1)
        self.pos = np.zeros((capacity, 3))
        self.force = np.zeros((capacity, 3))
        self.lambda_ = np.zeros(capacity)
        self.modulatedLambda = np.zeros(capacity)
        self.gradLambda = np.zeros((capacity, 3))
        self.atomsOffset = np.zeros(capacity, dtype=np.int64)
        self.numAtoms = np.zeros(capacity, dtype=np.int64)
        self.numLocal = 0
        self.numGhost = 0

    @property
    def capacity(self) -> int:
        return self.pos.shape[0]

    def grow(self, capacity: int):
        old = self.capacity
        if capacity <= old:
            return
        for name in ("pos", "force", "lambda_", "modulatedLambda", "gradLambda", "atomsOffset",
                     "numAtoms"):
            arr = getattr(self, name)
            new = np.zeros((capacity,) + arr.shape[1:], dtype=arr.dtype)
            new[:old] = arr
            setattr(self, name, new)

    def s(self) -> MoleculesS:
        return MoleculesS(_p(self.pos), _p(self.force), _p(self.lambda_),
                          _p(self.modulatedLambda), _p(self.gradLambda),
                          _p(self.atomsOffset, c_int64_p), _p(self.numAtoms, c_int64_p),
                          self.numLocal, self.numGhost, self.capacity)

    def sync(self, s: MoleculesS):
        self.numLocal, self.numGhost = s.numLocal, s.numGhost


def lj_table(cap, rc, sigma, eps, num_types=1, shifted=False):
    n2 = num_types * num_types
    arr = (LJParams * n2)()

    def v(x):
        return np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (n2,)))

    c, r, s, e = v(cap), v(rc), v(sigma), v(eps)
    lib().orc_lj_init(arr, num_types, _p(c), _p(r), _p(s), _p(e), int(bool(shifted)))
    return arr


def lj_force_energy(table, dist_sqr, type_idx=0):
    ff, e = C.c_double(), C.c_double()
    lib().orc_lj_force_energy(table, float(dist_sqr), int(type_idx), C.byref(ff), C.byref(e))
    return ff.value, e.value


def lj_apply(table, rc_sqr, atoms: Atoms, counts, nbrs, pred_=None, num_types_index=1):
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
    cap = nbrs.shape[1] if nbrs.ndim == 2 else 1
    s = atoms.s()
    E, W = C.c_double(), C.c_double()
    lib().orc_lj_apply(table, num_types_index, float(rc_sqr), C.byref(s), _p(counts, c_int32_p),
                       _p(nbrs, c_int32_p), cap, C.byref(pred_) if pred_ is not None else None,
                       C.byref(E), C.byref(W))
    return E.value, W.value


def map_into_domain(atoms: Atoms, sd: Subdomain):
    s = atoms.s()
    lib().orc_map_into_domain(C.byref(s), C.byref(sd))


def create_ghosts(atoms: Atoms, sd: Subdomain):
    """GhostLayer::createGhostAtoms; returns the correspondingRealAtom array."""
    while True:
        corr = np.full(atoms.capacity, -1, dtype=np.int64)
        s = atoms.s()
        need = lib().orc_create_ghosts_xyz(C.byref(s), C.byref(sd), _p(corr, c_int64_p))
        if need == 0:
            atoms.sync(s)
            return corr
        atoms.grow(int(need * 1.1) + 16)


def update_ghosts(atoms: Atoms, corr, sd: Subdomain):
    s = atoms.s()
    lib().orc_update_ghosts(C.byref(s), _p(corr, c_int64_p), C.byref(sd))


def ghost_to_real(atoms: Atoms, corr):
    s = atoms.s()
    lib().orc_ghost_to_real(C.byref(s), _p(corr, c_int64_p))


def cell_grid(grid_min, grid_max, delta):
    nc = np.zeros(3, dtype=np.int64)
    rdx = np.zeros(3)
    gmin = np.asarray(grid_min, dtype=np.float64)
    gmax = np.asarray(grid_max, dtype=np.float64)
    lib().orc_cell_grid(_p(gmin), _p(gmax), float(delta), _p(nc, c_int64_p), _p(rdx))
    return nc, rdx


def cell_index(pos, grid_min, nc, rdx):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    out = np.zeros(len(pos), dtype=np.int64)
    gmin = np.asarray(grid_min, dtype=np.float64)
    lib().orc_cell_index(_p(pos), len(pos), _p(gmin), _p(np.ascontiguousarray(nc), c_int64_p),
                         _p(np.ascontiguousarray(rdx)), _p(out, c_int64_p))
    return out


def build_half_list(pos, n_all, begin, end, rlist, grid_min, grid_max, cell_ratio=1.0, cap=64):
    """Half Verlet list; returns (counts[end-begin], nbrs[end-begin, cap])."""
    pos = np.ascontiguousarray(pos[:n_all], dtype=np.float64)
    gmin = np.asarray(grid_min, dtype=np.float64)
    gmax = np.asarray(grid_max, dtype=np.float64)
    while True:
        counts = np.zeros(max(end - begin, 1), dtype=np.int32)
        nbrs = np.zeros((max(end - begin, 1), cap), dtype=np.int32)
        mx = lib().orc_build_half_list(_p(pos), n_all, begin, end, float(rlist), float(cell_ratio),
                                       _p(gmin), _p(gmax), _p(counts, c_int32_p),
                                       _p(nbrs, c_int32_p), cap)
        if mx <= cap:
            return counts[: end - begin], nbrs[: end - begin]
        cap = int(mx) + 8


def count_within(pos, n_local, n_all, cutoff, box, periodic):
    pos = np.ascontiguousarray(pos[:n_all], dtype=np.float64)
    b = np.asarray(box, dtype=np.float64)
    return lib().orc_count_within(_p(pos), n_local, n_all, float(cutoff), _p(b), int(periodic))


def vv_pre(atoms: Atoms, dt):
    s = atoms.s()
    return lib().orc_vv_pre(C.byref(s), float(dt))


def vv_post(atoms: Atoms, dt):
    s = atoms.s()
    lib().orc_vv_post(C.byref(s), float(dt))


class CoulombDSF:
    """impl::CoulombDSF (action/CoulombDSF.hpp:39-83)."""

    def __init__(self, rc, alpha):
        self.c = CoulombDSFS()
        lib().orc_coulomb_dsf_init(C.byref(self.c), float(rc), float(alpha))

    def computeForce(self, dist_sqr, q1, q2):
        return lib().orc_coulomb_dsf_force(C.byref(self.c), float(dist_sqr), float(q1), float(q2))

    def computeEnergy(self, dist_sqr, q1, q2):
        return lib().orc_coulomb_dsf_energy(C.byref(self.c), float(dist_sqr), float(q1), float(q2))

    def apply(self, atoms: Atoms, counts, nbrs):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        s = atoms.s()
        E, W = C.c_double(), C.c_double()
        lib().orc_coulomb_dsf_apply(C.byref(self.c), C.byref(s), _p(counts, c_int32_p), _p(nbrs, c_int32_p),
                                    nbrs.shape[1] if nbrs.ndim == 2 else 1, C.byref(E), C.byref(W))
        return E.value, W.value


def approx_erfc(x):
    e = C.c_double()
    return lib().orc_approx_erfc(float(x), C.byref(e))


def kinetic_energy(atoms: Atoms):
    s = atoms.s()
    return lib().orc_kinetic_energy(C.byref(s))


def system_momentum(atoms: Atoms):
    s = atoms.s()
    out = np.zeros(3)
    lib().orc_system_momentum(C.byref(s), _p(out))
    return out


def pressure(atoms: Atoms, sd: Subdomain):
    s = atoms.s()
    return lib().orc_pressure(C.byref(s), C.byref(sd))


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def normal3(seed, step, atom):
    out = np.zeros(3)
    lib().orc_normal_from_counter(seed, step, atom, _p(out))
    return out


def langevin_pre(atoms: Atoms, dt, zeta, temperature, seed, step, pred_=None):
    s = atoms.s()
    return lib().orc_langevin_pre(C.byref(s), float(dt), float(zeta), float(temperature),
                                  int(seed), int(step),
                                  C.byref(pred_) if pred_ is not None else None)


def slab(center, at_diameter, hy_diameter, nu, interface_type=0) -> SlabS:
    s = SlabS()
    c = np.asarray(center, dtype=np.float64)
    lib().orc_slab_init(C.byref(s), _p(c), float(at_diameter), float(hy_diameter), int(nu),
                        int(interface_type))
    return s


def slab_eval(s: SlabS, x, y=0.0, z=0.0):
    out = np.zeros(5)
    lib().orc_slab_eval(C.byref(s), float(x), float(y), float(z), _p(out))
    return out


def update_molecules(mol: Molecules, atoms: Atoms, s: SlabS):
    ms, as_ = mol.s(), atoms.s()
    lib().orc_update_molecules(C.byref(ms), C.byref(as_), C.byref(s))


def contribute_molecule_force(mol: Molecules, atoms: Atoms):
    ms, as_ = mol.s(), atoms.s()
    lib().orc_contribute_molecule_force(C.byref(ms), C.byref(as_))


class LJIdealGas:
    """State of action::LJ_IdealGas (action/LJ_IdealGas.hpp:34-104)."""

    def __init__(self, cap, rc, sigma, eps, shifted, num_types=1):
        self.table = lj_table(cap, rc, sigma, eps, num_types, shifted)
        nb = 200
        self.comp = np.zeros((nb, num_types))
        self.counter = np.zeros((nb, num_types))
        self.mean = np.zeros((nb, num_types))
        rc_max = float(np.max(np.asarray(rc, dtype=np.float64)))
        self.s = LJIG(self.table, num_types, rc_max * rc_max, _p(self.comp), _p(self.counter),
                      _p(self.mean), 0, 200, 20000)

    def run(self, mol: Molecules, counts, nbrs, atoms: Atoms):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        cap = nbrs.shape[1] if nbrs.ndim == 2 else 1
        ms, as_ = mol.s(), atoms.s()
        return lib().orc_ljig_run(C.byref(self.s), C.byref(ms), _p(counts, c_int32_p),
                                  _p(nbrs, c_int32_p), cap, C.byref(as_))


def multires_map_into_domain(sd: Subdomain, mol: Molecules, atoms: Atoms):
    ms, as_ = mol.s(), atoms.s()
    lib().orc_multires_map_into_domain(C.byref(sd), C.byref(ms), C.byref(as_))


def multires_create_ghosts(mol: Molecules, atoms: Atoms, sd: Subdomain):
    while True:
        corr = np.full(atoms.capacity, -1, dtype=np.int64)
        ms, as_ = mol.s(), atoms.s()
        need = lib().orc_multires_create_ghosts_xyz(C.byref(ms), C.byref(as_), C.byref(sd),
                                                    _p(corr, c_int64_p))
        if need == 0:
            mol.sync(ms)
            atoms.sync(as_)
            return corr
        mol.grow(int(need * 1.1) + 16)
        atoms.grow(int(need * 1.1) + 16)


class Histogram:
    """data::MultiHistogram (data/MultiHistogram.hpp:29-92)."""

    def __init__(self, mn, mx, num_bins, num_hist, data=None):
        self.data = np.zeros((num_bins, num_hist)) if data is None else np.ascontiguousarray(
            data, dtype=np.float64)
        self.h = Hist()
        lib().orc_hist_init(C.byref(self.h), float(mn), float(mx), int(num_bins), int(num_hist),
                            _p(self.data))

    def get_bin(self, v):
        return lib().orc_hist_get_bin(C.byref(self.h), float(v))

    def bin_position(self, b):
        return lib().orc_hist_bin_position(C.byref(self.h), int(b))

    def like(self):
        return Histogram(self.h.min, self.h.max, self.h.numBins, self.h.numHist)

    def scale(self, f):
        if np.isscalar(f):
            lib().orc_hist_scale(C.byref(self.h), float(f))
        else:
            f = np.ascontiguousarray(f, dtype=np.float64)
            lib().orc_hist_scale_per_hist(C.byref(self.h), _p(f))

    def make_symmetric(self):
        lib().orc_hist_make_symmetric(C.byref(self.h))

    def gradient(self, periodic=False):
        out = self.like()
        lib().orc_hist_gradient(C.byref(self.h), C.byref(out.h), int(periodic))
        return out

    def smoothen(self, sigma, rng, periodic=False):
        out = self.like()
        lib().orc_hist_smoothen(C.byref(self.h), C.byref(out.h), float(sigma), float(rng),
                                int(periodic))
        return out

    def replace_if(self, p: Pred, value, invert=False):
        lib().orc_hist_replace_if(C.byref(self.h), C.byref(p), int(invert), float(value))


def axial_density_profile(atoms: Atoms, num_types, mn, mx, num_bins, axis=0):
    h = Histogram(mn, mx, num_bins, num_types)
    s = atoms.s()
    lib().orc_axial_density_profile(C.byref(s), atoms.numLocal, C.byref(h.h), int(axis))
    return h


class ThermodynamicForce:
    """action::ThermodynamicForce (action/ThermodynamicForce.hpp:32-96)."""

    def __init__(self, target_density, sd: Subdomain, bin_width, modulation,
                 enforce_symmetry=False, use_periodicity=False):
        td = np.atleast_1d(np.asarray(target_density, dtype=np.float64))
        mod = np.atleast_1d(np.asarray(modulation, dtype=np.float64))
        nt = len(td)
        nb = lib().orc_tf_num_bins(C.byref(sd), float(bin_width))
        self.force = np.zeros((nb, nt))
        self.density = np.zeros((nb, nt))
        self.factor = np.zeros(nt)
        self.scratch = np.zeros(2 * nb * nt)
        self._td, self._mod = td, mod
        self.tf = TF()
        lib().orc_tf_init(C.byref(self.tf), C.byref(sd), nb, nt, _p(self.force), _p(self.density),
                          _p(self.factor), _p(td), _p(mod), int(enforce_symmetry),
                          int(use_periodicity))

    @property
    def samples(self):
        return self.tf.samples

    def sample(self, atoms: Atoms):
        s = atoms.s()
        lib().orc_tf_sample(C.byref(self.tf), C.byref(s))

    def apply(self, atoms: Atoms, pred_=None):
        s = atoms.s()
        lib().orc_tf_apply(C.byref(self.tf), C.byref(s),
                           C.byref(pred_) if pred_ is not None else None)

    def apply_interpolated(self, atoms: Atoms, pred_=None):
        s = atoms.s()
        lib().orc_tf_apply_interpolated(C.byref(self.tf), C.byref(s),
                                        C.byref(pred_) if pred_ is not None else None)

    def update(self, sigma, intensity, pred_=None):
        return lib().orc_tf_update(C.byref(self.tf), float(sigma), float(intensity),
                                   C.byref(pred_) if pred_ is not None else None,
                                   _p(self.scratch))

    def mu(self):
        nt = self.force.shape[1]
        l, r = np.zeros(nt), np.zeros(nt)
        lib().orc_tf_mu(C.byref(self.tf), _p(l), _p(r))
        return l, r


# ------------------------------------------------ thermodynamic-force text --

def tf_grid(min_x, max_x, num_bins):
    """createGrid: bin centres min + (i + 0.5) binSize (data/MultiHistogram.cpp:214-227,
    MultiHistogram.hpp:40-41, 68-74)."""
    bin_size = (max_x - min_x) / num_bins
    return np.array([min_x + (i + 0.5) * bin_size for i in range(num_bins)])


def tf_table_text(grid, force, type_id=None):
    """dumpThermoForce (io/DumpThermoForce.cpp:24-64) through DumpProfile::dumpScalarView
    (io/DumpProfile.cpp:25-35): values joined by one space, each formatted like a
    default std::ostream (printf %g, 6 significant digits), every line ended by a newline."""
    force = np.asarray(force, dtype=np.float64).reshape(len(grid), -1)
    types = range(force.shape[1]) if type_id is None else [type_id]
    lines = [" ".join("%g" % v for v in grid)]
    lines += [" ".join("%g" % v for v in force[:, t]) for t in types]
    return "".join(line + "\n" for line in lines)


def tf_table_parse(text, max_num_forces=10):
    """restoreThermoForce's reader (io/RestoreThermoForce.cpp:34-73): returns
    (grid, force [numBins][numForces], binWidth = grid[1] - grid[0]).  Raises
    ValueError where the reference asserts (fewer than two bins, more than
    max_num_forces lines) and on lines whose length differs from the grid's."""
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    if not lines:
        raise ValueError("empty table")
    grid = [float(w) for w in lines[0].split()]
    if len(grid) < 2:
        raise ValueError("fewer than two bins")
    rows = []
    for line in lines[1:]:
        row = [float(w) for w in line.split()]
        if len(row) != len(grid):
            raise ValueError("ragged force line")
        rows.append(row)
        if len(rows) > max_num_forces:
            raise ValueError("too many force lines")
    force = np.array(rows, dtype=np.float64).T.reshape(len(grid), len(rows))
    return np.array(grid), force, grid[1] - grid[0]


def tf_num_bins(sd: Subdomain, bin_width):
    """ceil(diameter / binWidth), the bin count of ThermodynamicForce's constructor
    (action/ThermodynamicForce.cpp:34)."""
    return int(lib().orc_tf_num_bins(C.byref(sd), float(bin_width)))


# --------------------------------------------------------- canonical pairs --

def canonical_pairs(counts, nbrs, corr, n_local):
    """Sorted unordered pairs of REAL atom ids from a half list whose entries may
    be ghosts (mapped back through correspondingRealAtom)."""
    counts = np.asarray(counts)
    rows = np.repeat(np.arange(len(counts), dtype=np.int64), counts)
    mask = np.arange(nbrs.shape[1])[None, :] < counts[:, None]
    cols = nbrs[mask].astype(np.int64)
    cols = np.where(cols >= n_local, corr[cols], cols)
    a = np.minimum(rows, cols)
    b = np.maximum(rows, cols)
    keys = a * (1 << 32) + b
    keys.sort()
    return keys
