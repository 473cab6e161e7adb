"""mrmd_gb300: GB300-native MRMD hot path (LJ / AdResS) behind MRMD's action API.

The compute lives in ``libmrmd_gb300.so`` (hand-written sm_103a CUDA behind a
C ABI, ``include/mrmd_gb300.h``).  This module is a thin ctypes mirror of
MRMD's C++ classes (``data::Atoms``, ``action::LennardJones``,
``communication::GhostLayer`` ...) with the same names and argument meaning,
used by the tests and by the PyTorch adjoint.  Every call goes to the GPU;
nothing here computes on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import (MrmdError, PRED_ALWAYS, PRED_BOTH_IN_SLAB, PRED_EITHER_IN_SLAB,  # noqa: F401
                   PRED_IN_OPEN_INTERVAL, PRED_IN_SLAB, PREC_FP64, PREC_MIXED)

c_double_p = _abi.c_double_p
c_int64_p = _abi.c_int64_p
c_int32_p = _abi.c_int32_p


def _dp(a):
    return None if a is None else a.ctypes.data_as(c_double_p)


def _ip(a):
    return None if a is None else a.ctypes.data_as(c_int64_p)


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Context:
    """One GPU, one stream (replaces Kokkos::ScopeGuard for the device side)."""

    def __init__(self, device: int = 0):
        self.lib = _abi.lib()
        h = C.c_void_p()
        self.check(self.lib.mrmd_ctx_create(C.byref(h), int(device)), None)
        self.h = h

    def check(self, rc: int, what: str | None = "call"):
        if rc != 0:
            msg = self.lib.mrmd_ctx_last_error(self.h).decode() if getattr(self, "h", None) else what
            raise MrmdError(rc, f"{what}: {msg}")

    def sync(self):
        self.check(self.lib.mrmd_ctx_sync(self.h), "sync")

    def set_sync(self, on: bool):
        self.check(self.lib.mrmd_ctx_set_sync(self.h, int(bool(on))), "set_sync")

    @property
    def launches(self) -> int:
        return int(self.lib.mrmd_ctx_launch_count(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.mrmd_ctx_stream(self.h) or 0)

    def close(self):
        if getattr(self, "h", None):
            self.lib.mrmd_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def pred(kind=PRED_ALWAYS, axis=0, center=0.0, slab_min=0.0, slab_max=0.0, tolerance=0.0):
    return _abi.Pred(kind, axis, center, slab_min, slab_max, tolerance)


def is_in_symmetric_slab(center, slab_min, slab_max, axis=0, tolerance=0.0, kind=PRED_IN_SLAB):
    """util::IsInSymmetricSlab (util/IsInSymmetricSlab.hpp:24-64) as a predicate."""
    c = center[axis] if np.ndim(center) else center
    return pred(kind, axis, float(c), slab_min, slab_max, tolerance)


class Subdomain:
    """data::Subdomain (data/Subdomain.hpp:37-110)."""

    def __init__(self, min_corner, max_corner, ghost_layer_thickness):
        g = ghost_layer_thickness
        if np.isscalar(g):
            g = (g, g, g)
        self.s = _abi.SubdomainS()
        rc = _abi.lib().mrmd_subdomain_init(C.byref(self.s), _dp(_f64(min_corner)),
                                            _dp(_f64(max_corner)), _dp(_f64(g)))
        if rc != 0:
            raise MrmdError(rc, "Subdomain: bad arguments")

    def __getattr__(self, name):
        if name in ("minCorner", "maxCorner", "ghostLayerThickness", "minGhostCorner", "maxGhostCorner",
                    "minInnerCorner", "maxInnerCorner", "diameter", "diameterWithGhostLayer"):
            return np.array(getattr(self.s, name)[:])
        raise AttributeError(name)


class Atoms:
    """data::Atoms (data/Atoms.hpp:33-177) with device SoA storage."""

    def __init__(self, capacity: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.s = _abi.AtomsS()
        self.ctx.check(self.ctx.lib.mrmd_atoms_alloc(self.ctx.h, C.byref(self.s), int(capacity)),
                       "Atoms")

    numLocalAtoms = property(lambda self: self.s.numLocal,
                             lambda self, v: setattr(self.s, "numLocal", int(v)))
    numGhostAtoms = property(lambda self: self.s.numGhost,
                             lambda self, v: setattr(self.s, "numGhost", int(v)))

    @property
    def size(self):
        return self.s.numLocal + self.s.numGhost

    @property
    def capacity(self):
        return self.s.capacity

    def upload(self, n_local, n_ghost=0, pos=None, vel=None, force=None, type=None, mass=None,
               charge=None, relative_mass=None):
        n = n_local + n_ghost
        t = None if type is None else np.ascontiguousarray(type, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_atoms_upload(
            self.ctx.h, C.byref(self.s), int(n_local), int(n_ghost), _dp(_f64(pos, (n, 3))),
            _dp(_f64(vel, (n, 3))), _dp(_f64(force, (n, 3))), _ip(t), _dp(_f64(mass)),
            _dp(_f64(charge)), _dp(_f64(relative_mass))), "Atoms.upload")

    @classmethod
    def from_arrays(cls, pos, vel=None, mass=1.0, type=None, relative_mass=1.0, capacity=None,
                    ctx=None, force=None):
        pos = _f64(pos)
        n = len(pos)
        a = cls(capacity or max(2 * n, 64), ctx)
        a.upload(n, 0, pos=pos, vel=np.zeros((n, 3)) if vel is None else vel,
                 force=np.zeros((n, 3)) if force is None else force,
                 type=np.zeros(n, dtype=np.int64) if type is None else type,
                 mass=np.broadcast_to(np.asarray(mass, dtype=np.float64), (n,)).copy(),
                 charge=np.zeros(n),
                 relative_mass=np.broadcast_to(np.asarray(relative_mass, dtype=np.float64), (n,)).copy())
        return a

    def download(self, n=None):
        n = self.size if n is None else n
        out = {k: np.zeros((n, 3)) for k in ("pos", "vel", "force")}
        out.update(type=np.zeros(n, dtype=np.int64), mass=np.zeros(n), charge=np.zeros(n),
                   relativeMass=np.zeros(n))
        self.ctx.check(self.ctx.lib.mrmd_atoms_download(
            self.ctx.h, C.byref(self.s), int(n), _dp(out["pos"]), _dp(out["vel"]),
            _dp(out["force"]), _ip(out["type"]), _dp(out["mass"]), _dp(out["charge"]),
            _dp(out["relativeMass"])), "Atoms.download")
        return out

    def getPos(self, n=None):
        return self.download(n)["pos"]

    def getVel(self, n=None):
        return self.download(n)["vel"]

    def getForce(self, n=None):
        return self.download(n)["force"]

    def setForce(self, val: float, n=None):
        n = self.size if n is None else n
        self.ctx.check(self.ctx.lib.mrmd_atoms_set_force(self.ctx.h, C.byref(self.s), int(n),
                                                         float(val)), "setForce")

    def sort_by_cell(self, grid_min, grid_max, delta):
        perm = np.zeros(self.s.numLocal, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_atoms_sort_by_cell(
            self.ctx.h, C.byref(self.s), _dp(_f64(grid_min)), _dp(_f64(grid_max)), float(delta),
            _ip(perm)), "sort_by_cell")
        return perm

    def free(self):
        if self.s.pos:
            self.ctx.lib.mrmd_atoms_free(self.ctx.h, C.byref(self.s))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Molecules:
    """data::Molecules (data/Molecules.hpp:27-176)."""

    def __init__(self, capacity: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.s = _abi.MoleculesS()
        self.ctx.check(self.ctx.lib.mrmd_molecules_alloc(self.ctx.h, C.byref(self.s),
                                                         int(capacity)), "Molecules")

    numLocalMolecules = property(lambda self: self.s.numLocal,
                                 lambda self, v: setattr(self.s, "numLocal", int(v)))
    numGhostMolecules = property(lambda self: self.s.numGhost,
                                 lambda self, v: setattr(self.s, "numGhost", int(v)))

    @property
    def size(self):
        return self.s.numLocal + self.s.numGhost

    def upload(self, n_local, n_ghost=0, pos=None, force=None, lambda_=None, modulated_lambda=None,
               grad_lambda=None, atoms_offset=None, num_atoms=None):
        n = n_local + n_ghost
        off = None if atoms_offset is None else np.ascontiguousarray(atoms_offset, dtype=np.int64)
        na = None if num_atoms is None else np.ascontiguousarray(num_atoms, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_molecules_upload(
            self.ctx.h, C.byref(self.s), int(n_local), int(n_ghost), _dp(_f64(pos, (n, 3))),
            _dp(_f64(force, (n, 3))), _dp(_f64(lambda_)), _dp(_f64(modulated_lambda)),
            _dp(_f64(grad_lambda, (n, 3))), _ip(off), _ip(na)), "Molecules.upload")

    def download(self, n=None):
        n = self.size if n is None else n
        out = dict(pos=np.zeros((n, 3)), force=np.zeros((n, 3)), lambda_=np.zeros(n),
                   modulatedLambda=np.zeros(n), gradLambda=np.zeros((n, 3)),
                   atomsOffset=np.zeros(n, dtype=np.int64), numAtoms=np.zeros(n, dtype=np.int64))
        self.ctx.check(self.ctx.lib.mrmd_molecules_download(
            self.ctx.h, C.byref(self.s), int(n), _dp(out["pos"]), _dp(out["force"]),
            _dp(out["lambda_"]), _dp(out["modulatedLambda"]), _dp(out["gradLambda"]),
            _ip(out["atomsOffset"]), _ip(out["numAtoms"])), "Molecules.download")
        return out

    def setForce(self, val: float, n=None):
        n = self.size if n is None else n
        self.ctx.check(self.ctx.lib.mrmd_molecules_set_force(self.ctx.h, C.byref(self.s), int(n),
                                                             float(val)), "setForce")

    def free(self):
        if self.s.pos:
            self.ctx.lib.mrmd_molecules_free(self.ctx.h, C.byref(self.s))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class GhostLayer:
    """communication::GhostLayer (communication/GhostLayer.hpp:28-56)."""

    def __init__(self, ctx: Context | None = None, capacity: int = 1):
        self.ctx = ctx or default_context()
        self.s = _abi.GhostLayerS()
        self.ctx.check(self.ctx.lib.mrmd_ghost_layer_alloc(self.ctx.h, C.byref(self.s),
                                                           int(capacity)), "GhostLayer")

    def exchangeRealAtoms(self, atoms: Atoms, subdomain: Subdomain):
        self.ctx.check(self.ctx.lib.mrmd_ghost_exchange_real_atoms(
            self.ctx.h, C.byref(atoms.s), C.byref(subdomain.s)), "exchangeRealAtoms")

    def createGhostAtoms(self, atoms: Atoms, subdomain: Subdomain):
        self.ctx.check(self.ctx.lib.mrmd_ghost_create(self.ctx.h, C.byref(self.s), C.byref(atoms.s),
                                                      C.byref(subdomain.s)), "createGhostAtoms")

    def updateGhostAtoms(self, atoms: Atoms, subdomain: Subdomain):
        self.ctx.check(self.ctx.lib.mrmd_ghost_update(self.ctx.h, C.byref(self.s), C.byref(atoms.s),
                                                      C.byref(subdomain.s)), "updateGhostAtoms")

    def contributeBackGhostToReal(self, atoms: Atoms):
        self.ctx.check(self.ctx.lib.mrmd_ghost_reduce_force(self.ctx.h, C.byref(self.s),
                                                            C.byref(atoms.s)),
                       "contributeBackGhostToReal")

    def correspondingRealAtom(self, n: int):
        out = np.zeros(n, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_ghost_layer_download(self.ctx.h, C.byref(self.s), int(n),
                                                              _ip(out)), "corr")
        return out

    def __del__(self):
        try:
            self.ctx.lib.mrmd_ghost_layer_free(self.ctx.h, C.byref(self.s))
        except Exception:
            pass


class MultiResGhostLayer(GhostLayer):
    """communication::MultiResGhostLayer (communication/MultiResGhostLayer.hpp:29-61)."""

    def exchangeRealAtoms(self, molecules: Molecules, atoms: Atoms, subdomain: Subdomain):
        self.ctx.check(self.ctx.lib.mrmd_multires_exchange_real_atoms(
            self.ctx.h, C.byref(molecules.s), C.byref(atoms.s), C.byref(subdomain.s)),
            "exchangeRealAtoms")

    def createGhostAtoms(self, molecules: Molecules, atoms: Atoms, subdomain: Subdomain):
        self.ctx.check(self.ctx.lib.mrmd_multires_ghost_create(
            self.ctx.h, C.byref(self.s), C.byref(molecules.s), C.byref(atoms.s),
            C.byref(subdomain.s)), "createGhostAtoms")


class HalfVerletList:
    """HalfVerletList (datatypes.hpp:184-187) built on the GPU."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.s = _abi.NListS()
        self.ctx.check(self.ctx.lib.mrmd_nlist_init(self.ctx.h, C.byref(self.s)), "HalfVerletList")

    def build(self, pos_source, begin, end, cutoff, cell_ratio, grid_min, grid_max, max_neigh=60,
              n_pos=None):
        """pos_source: Atoms (positions of all its atoms) or Molecules."""
        n_pos = pos_source.size if n_pos is None else n_pos
        self.ctx.check(self.ctx.lib.mrmd_nlist_build(
            self.ctx.h, C.byref(self.s), pos_source.s.pos, int(n_pos), int(begin), int(end),
            float(cutoff), float(cell_ratio), _dp(_f64(grid_min)), _dp(_f64(grid_max)),
            int(max_neigh)), "HalfVerletList.build")

    @property
    def total_pairs(self):
        return self.s.totalPairs

    def download(self, cap=None):
        rows = self.s.rows
        counts = np.zeros(max(rows, 1), dtype=np.int32)
        cap = cap or max(int(self.s.maxNeighbors), 1)
        nbrs = np.zeros((max(rows, 1), cap), dtype=np.int32)
        self.ctx.check(self.ctx.lib.mrmd_nlist_download(
            self.ctx.h, C.byref(self.s), counts.ctypes.data_as(c_int32_p),
            nbrs.ctypes.data_as(c_int32_p), int(cap)), "download")
        return counts[:rows], nbrs[:rows]

    def __del__(self):
        try:
            self.ctx.lib.mrmd_nlist_free(self.ctx.h, C.byref(self.s))
        except Exception:
            pass


def cell_index(atoms: Atoms, n, grid_min, grid_max, delta, ctx=None):
    ctx = ctx or atoms.ctx
    out = np.zeros(n, dtype=np.int64)
    ctx.check(ctx.lib.mrmd_cell_index(ctx.h, atoms.s.pos, int(n), _dp(_f64(grid_min)),
                                      _dp(_f64(grid_max)), float(delta), _ip(out)), "cell_index")
    return out


class LennardJones:
    """action::LennardJones (action/LennardJones.hpp:98-133)."""

    def __init__(self, rc, sigma, epsilon, capping_distance=0.0, num_types=1, is_shifted=False,
                 num_types_index=1, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        n2 = num_types * num_types

        def v(x):
            return np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (n2,)))

        self.num_types = num_types
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.mrmd_lj_create(
            self.ctx.h, C.byref(h), int(num_types), int(num_types_index), _dp(v(capping_distance)),
            _dp(v(rc)), _dp(v(sigma)), _dp(v(epsilon)), int(bool(is_shifted))), "LennardJones")
        self.h = h
        self.energy = 0.0
        self.virial = 0.0

    def params(self):
        n2 = self.num_types * self.num_types
        arr = (_abi.LJParamsS * n2)()
        self.ctx.lib.mrmd_lj_get_params(self.h, arr, n2)
        return arr

    def apply_if(self, atoms: Atoms, verlet_list: HalfVerletList, pred_=None, precision=PREC_FP64):
        E, W = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.mrmd_lj_apply(
            self.ctx.h, self.h, C.byref(atoms.s), C.byref(verlet_list.s),
            C.byref(pred_) if pred_ is not None else None, int(precision), C.byref(E), C.byref(W)),
            "LennardJones.apply")
        self.energy, self.virial = E.value, W.value

    def apply(self, atoms: Atoms, verlet_list: HalfVerletList, precision=PREC_FP64):
        self.apply_if(atoms, verlet_list, None, precision)

    def getEnergy(self):
        return self.energy

    def getVirial(self):
        return self.virial

    def __del__(self):
        try:
            self.ctx.lib.mrmd_lj_destroy(self.ctx.h, self.h)
        except Exception:
            pass


class CoulombDSF:
    """impl::CoulombDSF (action/CoulombDSF.hpp:39-83) with a half-list pair force."""

    def __init__(self, rc, alpha, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.c = _abi.CoulombDSFS()
        rc_ = self.ctx.lib.mrmd_coulomb_dsf_init(C.byref(self.c), float(rc), float(alpha))
        if rc_ != 0:
            raise MrmdError(rc_, "CoulombDSF: rc and alpha must be > 0")
        self.energy = self.virial = 0.0

    def _eval(self, dist_sqr, q1, q2):
        d, a, b = np.broadcast_arrays(np.asarray(dist_sqr, dtype=np.float64), np.asarray(q1, dtype=np.float64),
                                      np.asarray(q2, dtype=np.float64))
        shape = d.shape
        d, a, b = (np.ascontiguousarray(x).ravel() for x in (d, a, b))
        f, e = np.zeros(d.size), np.zeros(d.size)
        self.ctx.check(self.ctx.lib.mrmd_coulomb_dsf_eval(self.ctx.h, C.byref(self.c), d.size, _dp(d), _dp(a),
                                                          _dp(b), _dp(f), _dp(e)), "CoulombDSF")
        return f.reshape(shape), e.reshape(shape)

    def computeForce(self, dist_sqr, q1, q2):
        """Force / distSqr, evaluated on the device (scalars or arrays)."""
        f = self._eval(dist_sqr, q1, q2)[0]
        return float(f) if f.ndim == 0 else f

    def computeEnergy(self, dist_sqr, q1, q2):
        e = self._eval(dist_sqr, q1, q2)[1]
        return float(e) if e.ndim == 0 else e

    def apply(self, atoms: Atoms, verlet_list: "HalfVerletList"):
        E, W = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.mrmd_coulomb_dsf_apply(self.ctx.h, C.byref(self.c), C.byref(atoms.s),
                                                           C.byref(verlet_list.s), C.byref(E), C.byref(W)),
                       "CoulombDSF.apply")
        self.energy, self.virial = E.value, W.value
        return self.energy

    def getEnergy(self):
        return self.energy

    def getVirial(self):
        return self.virial


class VelocityVerlet:
    """action::VelocityVerlet (action/VelocityVerlet.hpp:26-31)."""

    @staticmethod
    def preForceIntegrate(atoms: Atoms, dt: float) -> float:
        m = C.c_double()
        atoms.ctx.check(atoms.ctx.lib.mrmd_vv_pre(atoms.ctx.h, C.byref(atoms.s), float(dt),
                                                  C.byref(m)), "preForceIntegrate")
        return m.value

    @staticmethod
    def postForceIntegrate(atoms: Atoms, dt: float):
        atoms.ctx.check(atoms.ctx.lib.mrmd_vv_post(atoms.ctx.h, C.byref(atoms.s), float(dt)),
                        "postForceIntegrate")


class VelocityVerletLangevinThermostat:
    """action::VelocityVerletLangevinThermostat with Philox noise keyed by (seed, step)."""

    def __init__(self, zeta, temperature, seed=1234):
        self.set(zeta, temperature)
        self.seed = seed
        self.step = 0

    def set(self, zeta, temperature):
        self.zeta, self.temperature = float(zeta), float(temperature)

    def preForceIntegrate_apply_if(self, atoms: Atoms, dt, pred_=None, step=None):
        m = C.c_double()
        st = self.step if step is None else step
        atoms.ctx.check(atoms.ctx.lib.mrmd_langevin_pre(
            atoms.ctx.h, C.byref(atoms.s), float(dt), self.zeta, self.temperature, int(self.seed),
            int(st), C.byref(pred_) if pred_ is not None else None, C.byref(m)), "langevin")
        if step is None:
            self.step += 1
        return m.value

    def preForceIntegrate(self, atoms: Atoms, dt, step=None):
        return self.preForceIntegrate_apply_if(atoms, dt, None, step)

    def postForceIntegrate(self, atoms: Atoms, dt):
        VelocityVerlet.postForceIntegrate(atoms, dt)


class Slab:
    """weighting_function::Slab (weighting_function/Slab.hpp:27-201)."""

    def __init__(self, center, atomistic_region_diameter, hybrid_region_diameter, nu,
                 interface_type=0):
        c = (C.c_double * 3)(*[float(x) for x in center])
        self.s = _abi.SlabS(c, float(atomistic_region_diameter), float(hybrid_region_diameter),
                            int(nu), int(interface_type), 0)


class UpdateMolecules:
    @staticmethod
    def update(molecules: Molecules, atoms: Atoms, weight: Slab):
        atoms.ctx.check(atoms.ctx.lib.mrmd_update_molecules(
            atoms.ctx.h, C.byref(molecules.s), C.byref(atoms.s), C.byref(weight.s)),
            "UpdateMolecules")


class ContributeMoleculeForceToAtoms:
    @staticmethod
    def update(molecules: Molecules, atoms: Atoms):
        atoms.ctx.check(atoms.ctx.lib.mrmd_contribute_molecule_force(
            atoms.ctx.h, C.byref(molecules.s), C.byref(atoms.s)), "ContributeMoleculeForceToAtoms")


class LJ_IdealGas:
    """action::LJ_IdealGas (action/LJ_IdealGas.hpp:34-104)."""

    def __init__(self, capping_distance, rc, sigma, epsilon, do_shift, num_types=1,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        n2 = num_types * num_types

        def v(x):
            return np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (n2,)))

        self.num_types = num_types
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.mrmd_ljig_create(
            self.ctx.h, C.byref(h), int(num_types), _dp(v(capping_distance)), _dp(v(rc)),
            _dp(v(sigma)), _dp(v(epsilon)), int(bool(do_shift))), "LJ_IdealGas")
        self.h = h

    def setCompensationEnergySamplingInterval(self, k):
        self._intervals(k, None)

    def setCompensationEnergyUpdateInterval(self, k):
        self._intervals(None, k)

    def _intervals(self, s, u):
        cur = self.compensation()
        self.ctx.check(self.ctx.lib.mrmd_ljig_set_intervals(
            self.h, int(s if s is not None else cur["sampling"]),
            int(u if u is not None else cur["update"])), "intervals")
        self._sampling = s if s is not None else cur["sampling"]
        self._update = u if u is not None else cur["update"]

    def run(self, molecules: Molecules, verlet_list: HalfVerletList, atoms: Atoms,
            precision=PREC_FP64) -> float:
        E = C.c_double()
        self.ctx.check(self.ctx.lib.mrmd_ljig_run(
            self.ctx.h, self.h, C.byref(molecules.s), C.byref(verlet_list.s), C.byref(atoms.s),
            int(precision), C.byref(E)), "LJ_IdealGas.run")
        return E.value

    def compensation(self):
        nb = 200 * self.num_types
        mean, e, c = np.zeros(nb), np.zeros(nb), np.zeros(nb)
        rc = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_ljig_get_compensation(
            self.ctx.h, self.h, _dp(mean), _dp(e), _dp(c), C.byref(rc)), "compensation")
        return dict(mean=mean.reshape(200, -1), energy=e.reshape(200, -1),
                    counter=c.reshape(200, -1), runCounter=rc.value,
                    sampling=getattr(self, "_sampling", 200), update=getattr(self, "_update", 20000))

    def getMeanCompensationEnergy(self):
        return self.compensation()["mean"]

    def __del__(self):
        try:
            self.ctx.lib.mrmd_ljig_destroy(self.ctx.h, self.h)
        except Exception:
            pass


class ThermodynamicForce:
    """action::ThermodynamicForce (action/ThermodynamicForce.hpp:32-96)."""

    def __init__(self, target_density, subdomain: Subdomain, requested_bin_width, modulation,
                 enforce_symmetry=False, use_periodicity=False, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        td = np.atleast_1d(np.asarray(target_density, dtype=np.float64))
        mod = np.atleast_1d(np.asarray(modulation, dtype=np.float64))
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.mrmd_tf_create(
            self.ctx.h, C.byref(h), len(td), _dp(td), C.byref(subdomain.s),
            float(requested_bin_width), _dp(mod), int(bool(enforce_symmetry)),
            int(bool(use_periodicity))), "ThermodynamicForce")
        self._adopt_handle(h)

    @classmethod
    def _adopt(cls, h, ctx: Context):
        """Wrap a table made by the library (restoreThermoForce)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self._adopt_handle(h)
        return self

    def _adopt_handle(self, h):
        self.h = h
        nb, bs, nt = C.c_int64(), C.c_double(), C.c_int64()
        self.ctx.lib.mrmd_tf_shape(h, C.byref(nb), C.byref(bs), C.byref(nt))
        self.num_bins, self.bin_size, self.num_types = nb.value, bs.value, nt.value

    def sample(self, atoms: Atoms):
        self.ctx.check(self.ctx.lib.mrmd_tf_sample(self.ctx.h, self.h, C.byref(atoms.s)), "sample")

    def apply_if(self, atoms: Atoms, pred_=None):
        self.ctx.check(self.ctx.lib.mrmd_tf_apply(self.ctx.h, self.h, C.byref(atoms.s),
                                                  C.byref(pred_) if pred_ is not None else None, 0),
                       "apply")

    def apply(self, atoms: Atoms):
        self.apply_if(atoms, None)

    def applyInterpolated_if(self, atoms: Atoms, pred_=None):
        self.ctx.check(self.ctx.lib.mrmd_tf_apply(self.ctx.h, self.h, C.byref(atoms.s),
                                                  C.byref(pred_) if pred_ is not None else None, 1),
                       "applyInterpolated")

    def update_if(self, sigma, intensity, pred_=None):
        self.ctx.check(self.ctx.lib.mrmd_tf_update(self.ctx.h, self.h, float(sigma),
                                                   float(intensity),
                                                   C.byref(pred_) if pred_ is not None else None),
                       "update")

    def update(self, sigma, intensity):
        self.update_if(sigma, intensity, None)

    def getForce(self):
        out = np.zeros((self.num_bins, self.num_types))
        self.ctx.check(self.ctx.lib.mrmd_tf_get_force(self.ctx.h, self.h, _dp(out)), "getForce")
        return out

    def setForce(self, f):
        f = _f64(f, (self.num_bins, self.num_types))
        self.ctx.check(self.ctx.lib.mrmd_tf_set_force(self.ctx.h, self.h, _dp(f)), "setForce")

    def getDensityProfile(self):
        out = np.zeros((self.num_bins, self.num_types))
        s = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_tf_get_density(self.ctx.h, self.h, _dp(out), C.byref(s)),
                       "getDensityProfile")
        self.samples = s.value
        return out

    def getNumberOfDensityProfileSamples(self):
        self.getDensityProfile()
        return self.samples

    def getGrid(self):
        """createGrid(getForce()): the bin centres."""
        out = np.zeros(self.num_bins)
        self.ctx.check(self.ctx.lib.mrmd_tf_grid(self.h, _dp(out)), "grid")
        return out

    def getMu(self):
        left, right = np.zeros(self.num_types), np.zeros(self.num_types)
        self.ctx.check(self.ctx.lib.mrmd_tf_mu(self.ctx.h, self.h, _dp(left), _dp(right)), "mu")
        return left, right

    def __del__(self):
        try:
            self.ctx.lib.mrmd_tf_destroy(self.ctx.h, self.h)
        except Exception:
            pass


def getKineticEnergy(atoms: Atoms) -> float:
    """analysis::getKineticEnergy (analysis/KineticEnergy.hpp:26-39)."""
    out = C.c_double()
    atoms.ctx.check(atoms.ctx.lib.mrmd_kinetic_energy(atoms.ctx.h, C.byref(atoms.s), C.byref(out)),
                    "getKineticEnergy")
    return out.value


def getMeanKineticEnergy(atoms: Atoms) -> float:
    """analysis::getMeanKineticEnergy (analysis/KineticEnergy.hpp:44-47)."""
    return getKineticEnergy(atoms) / float(atoms.numLocalAtoms)


def getSystemMomentum(atoms: Atoms):
    """analysis::getSystemMomentum (analysis/SystemMomentum.cpp:21-48): the
    velocity sum of the local atoms."""
    out = np.zeros(3)
    atoms.ctx.check(atoms.ctx.lib.mrmd_system_momentum(atoms.ctx.h, C.byref(atoms.s), _dp(out)),
                    "getSystemMomentum")
    return out


def getPressure(atoms: Atoms, subdomain: Subdomain) -> float:
    """analysis::getPressure (analysis/Pressure.cpp:23-51)."""
    out = C.c_double()
    atoms.ctx.check(atoms.ctx.lib.mrmd_pressure(atoms.ctx.h, C.byref(atoms.s), C.byref(subdomain.s),
                                                C.byref(out)), "getPressure")
    return out.value


class LJSystem:
    """Fused device-resident LJ NVE stepper (mrmd_md_*), the examples/02 loop.

    sort_atoms: permute the atoms into Z-order of their cells at every k-th
    list rebuild (True = every rebuild, 0 = never; the order decays slowly,
    so every 4th rebuild is the default).  tile_build (mixed form):
    "one_pass" builds the tile list from the cell list, "two_kernel" the int32
    rows and then their tile form (the same lists)."""

    def __init__(self, pos, vel, box_min, box_max, rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0,
                 capping_distance=0.0, shifted=True, precision=PREC_FP64, dt=0.005,
                 rebuild_interval=10, use_graph=True, sort_atoms=4, max_neighbors=0, mass=None,
                 observe=False, split_radius=0.0, gather_neighbours=False, tile_build="one_pass",
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        pos = _f64(pos)
        vel = _f64(vel)
        self.n = len(pos)
        cfg = _abi.MDConfigS()
        cfg.boxMin = (C.c_double * 3)(*box_min)
        cfg.boxMax = (C.c_double * 3)(*box_max)
        cfg.rc, cfg.skin, cfg.sigma, cfg.epsilon = rc, skin, sigma, epsilon
        cfg.cappingDistance = capping_distance
        cfg.shifted = int(bool(shifted))
        cfg.precision = int(precision)
        cfg.dt = dt
        cfg.rebuildInterval = int(rebuild_interval)
        cfg.useGraph = int(bool(use_graph))
        cfg.sortAtoms = int(sort_atoms)  # True: every rebuild; k: every k-th rebuild
        cfg.maxNeighbors = int(max_neighbors)
        cfg.observe = int(bool(observe))
        cfg.splitRadius = float(split_radius)
        cfg.gatherNeighbours = int(bool(gather_neighbours))
        if tile_build not in ("one_pass", "two_kernel"):
            raise ValueError("tile_build must be 'one_pass' or 'two_kernel'")
        cfg.tileBuild = 1 if tile_build == "two_kernel" else 0
        self.cfg = cfg
        h = C.c_void_p()
        m = None if mass is None else _f64(np.broadcast_to(mass, (self.n,)).copy())
        self.ctx.check(self.ctx.lib.mrmd_md_create(self.ctx.h, C.byref(h), C.byref(cfg), self.n,
                                                   _dp(pos), _dp(vel), _dp(m)), "LJSystem")
        self.h = h

    def run(self, nsteps: int, energies: bool = True):
        e = np.zeros((max(nsteps, 1), 2)) if energies else None
        self.ctx.check(self.ctx.lib.mrmd_md_run(self.ctx.h, self.h, int(nsteps), _dp(e)), "run")
        return e[:nsteps] if energies else None

    def run_observed(self, nsteps: int):
        """Advance nsteps (stepper created with observe=True); returns the
        per-step records [nsteps, 6]: LJ energy, LJ virial, kinetic energy,
        momentum (velocity sum) x, y, z, summed on the device."""
        r = np.zeros((max(nsteps, 1), 6))
        self.ctx.check(self.ctx.lib.mrmd_md_run_observed(self.ctx.h, self.h, int(nsteps), _dp(r)),
                       "run_observed")
        return r[:nsteps]

    def state(self, out=None):
        """(pos, vel, force) in the original atom order; `out` may supply three
        C-contiguous float64 [n, 3] arrays (e.g. pinned) to fill."""
        p, v, f = out if out is not None else (np.zeros((self.n, 3)) for _ in range(3))
        for a in (p, v, f):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == (self.n, 3)
        self.ctx.check(self.ctx.lib.mrmd_md_get_state(self.ctx.h, self.h, _dp(p), _dp(v), _dp(f)),
                       "state")
        return p, v, f

    def set_state(self, pos, vel):
        self.ctx.check(self.ctx.lib.mrmd_md_set_state(self.ctx.h, self.h, _dp(_f64(pos)),
                                                      _dp(_f64(vel))), "set_state")

    def eval_forces(self):
        """Forces of the current positions; returns (energy, virial)."""
        ev = np.zeros(2)
        self.ctx.check(self.ctx.lib.mrmd_md_eval(self.ctx.h, self.h, 0, _dp(ev)), "eval")
        return float(ev[0]), float(ev[1])

    def launch_pair_kernel(self):
        """Enqueue the pair-force kernel alone (asynchronous; for timing)."""
        self.ctx.check(self.ctx.lib.mrmd_md_eval(self.ctx.h, self.h, 1, None), "pair kernel")

    def stats(self):
        out = np.zeros(5, dtype=np.int64)
        self.ctx.lib.mrmd_md_stats(self.h, _ip(out))
        return dict(steps=int(out[0]), rebuilds=int(out[1]), pairs=int(out[2]), ghosts=int(out[3]),
                    list_capacity=int(out[4]))

    def tile_stats(self):
        """Mixed form: tiles, members of the largest tile, whether the pair
        kernel reads shared-memory tiles (True) or gathers through the cache,
        members of all tiles, the tiles the last rebuild's one-pass build could
        not fit, and the rebuilds so far that needed the int32 rows."""
        out = np.zeros(6, dtype=np.int64)
        self.ctx.lib.mrmd_md_tile_stats(self.h, _ip(out))
        return dict(tiles=int(out[0]), max_members=int(out[1]), tiled=bool(out[2]), members=int(out[3]),
                    unfit_tiles=int(out[4]), two_pass_builds=int(out[5]))

    def pair_keys(self):
        """Sorted canonical keys a * 2^32 + b (a < b, original atom indices) of
        every entry of the current list, as the pair kernel reads it."""
        cnt = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_md_pair_keys(self.ctx.h, self.h, None, 0, C.byref(cnt)), "pair_keys")
        keys = np.zeros(max(cnt.value, 1), dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_md_pair_keys(self.ctx.h, self.h, _ip(keys), len(keys), C.byref(cnt)),
                       "pair_keys")
        return keys[: cnt.value]

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.mrmd_md_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AdResSSystem:
    """Fused AdResS LJ <-> ideal-gas stepper for single-site molecules (mrmd_adress_*).
    With unit masses the step runs on the batched engine with one replica;
    composed=True (or other masses) runs the composed actions instead."""

    def __init__(self, pos, vel, box_min, box_max, slab_center, atomistic_diameter,
                 hybrid_diameter, nu=1, rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0,
                 capping_distance=0.0, shifted=True, precision=PREC_FP64, dt=0.005,
                 rebuild_interval=10, gamma=1.0, temperature=1.0, seed=1234, tf=True,
                 tf_bin_width=1.2, tf_target_density=0.5, tf_modulation=1.0, tf_sigma=2.4,
                 tf_range=3.0, tf_sample_interval=1, tf_update_interval=1000, use_graph=True,
                 max_neighbors=0, mass=None, composed=False, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        pos = _f64(pos)
        vel = _f64(vel)
        self.n = len(pos)
        c = _abi.AdResSConfigS()
        c.boxMin = (C.c_double * 3)(*box_min)
        c.boxMax = (C.c_double * 3)(*box_max)
        c.rc, c.skin, c.sigma, c.epsilon = rc, skin, sigma, epsilon
        c.cappingDistance = capping_distance
        c.shifted = int(bool(shifted))
        c.precision = int(precision)
        c.dt = dt
        c.rebuildInterval = int(rebuild_interval)
        c.slabCenter = (C.c_double * 3)(*slab_center)
        c.atomisticDiameter, c.hybridDiameter, c.nu = atomistic_diameter, hybrid_diameter, int(nu)
        c.gamma, c.temperature, c.seed = gamma, temperature, int(seed)
        c.tfEnabled = int(bool(tf))
        c.useGraph = int(bool(use_graph))
        c.tfBinWidth, c.tfTargetDensity, c.tfModulation = tf_bin_width, tf_target_density, tf_modulation
        c.tfSmoothingSigma, c.tfSmoothingRange = tf_sigma, tf_range
        c.tfSampleInterval, c.tfUpdateInterval = int(tf_sample_interval), int(tf_update_interval)
        c.maxNeighbors = int(max_neighbors)
        c.composed = int(bool(composed))
        self.cfg = c
        h = C.c_void_p()
        m = None if mass is None else _f64(np.broadcast_to(mass, (self.n,)).copy())
        self.ctx.check(self.ctx.lib.mrmd_adress_create(self.ctx.h, C.byref(h), C.byref(c), self.n,
                                                       _dp(pos), _dp(vel), _dp(m)), "AdResSSystem")
        self.h = h

    def run(self, nsteps: int, energies: bool = True):
        e = np.zeros(max(nsteps, 1)) if energies else None
        self.ctx.check(self.ctx.lib.mrmd_adress_run(self.ctx.h, self.h, int(nsteps), _dp(e)), "run")
        return e[:nsteps] if energies else None

    def state(self):
        p, v, f = (np.zeros((self.n, 3)) for _ in range(3))
        self.ctx.check(self.ctx.lib.mrmd_adress_get_state(self.ctx.h, self.h, _dp(p), _dp(v), _dp(f)),
                       "state")
        return p, v, f

    def thermodynamic_force(self):
        nb = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_adress_get_tf(self.ctx.h, self.h, None, None, C.byref(nb)), "tf")
        f, d = np.zeros(nb.value), np.zeros(nb.value)
        self.ctx.check(self.ctx.lib.mrmd_adress_get_tf(self.ctx.h, self.h, _dp(f), _dp(d), None), "tf")
        return f, d

    def set_thermodynamic_force(self, f):
        self.ctx.check(self.ctx.lib.mrmd_adress_set_tf(self.ctx.h, self.h, _dp(_f64(f))), "set tf")

    def stats(self):
        out = np.zeros(4, dtype=np.int64)
        self.ctx.lib.mrmd_adress_stats(self.h, _ip(out))
        return dict(steps=int(out[0]), rebuilds=int(out[1]), pairs=int(out[2]), ghost_molecules=int(out[3]))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.mrmd_adress_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Replica:
    """One replica of a batch: molecule count, box, slab centre and width, noise key."""

    def __init__(self, num_molecules, box_min, box_max, slab_center, atomistic_diameter, seed):
        self.num_molecules = int(num_molecules)
        self.box_min = tuple(float(v) for v in box_min)
        self.box_max = tuple(float(v) for v in box_max)
        self.slab_center = tuple(float(v) for v in slab_center)
        self.atomistic_diameter = float(atomistic_diameter)
        self.seed = int(seed)

    def _struct(self):
        r = _abi.ReplicaS()
        r.numMolecules = self.num_molecules
        r.boxMin = (C.c_double * 3)(*self.box_min)
        r.boxMax = (C.c_double * 3)(*self.box_max)
        r.slabCenter = (C.c_double * 3)(*self.slab_center)
        r.atomisticDiameter = self.atomistic_diameter
        r.seed = self.seed
        return r


def _tuning_dict(t):
    return dict(threads_per_row=int(t.threadsPerRow), block_size=int(t.blockSize),
                rebuild_interval=int(t.rebuildInterval), sort_every=int(t.sortEvery),
                graph_steps=int(t.graphSteps), list_layout=int(t.listLayout), persistent=int(t.persistent))


def _tuning_struct(d):
    t = _abi.BatchTuningS()
    t.threadsPerRow = int(d["threads_per_row"])
    t.blockSize = int(d["block_size"])
    t.rebuildInterval = int(d["rebuild_interval"])
    t.sortEvery = int(d["sort_every"])
    t.graphSteps = int(d["graph_steps"])
    t.listLayout = int(d.get("list_layout", 0))
    t.persistent = int(d.get("persistent", 0))
    return t


def grid_sync_selftest(rounds=100, skip_block=-1, limit_ms=50.0, ctx: Context | None = None):
    """The persistent step kernel's grid barrier on its own (mrmd_grid_sync_selftest):
    returns the status, MRMD_ERR_TIMEOUT when a block never arrived (skip_block >= 0)."""
    ctx = ctx or default_context()
    return int(ctx.lib.mrmd_grid_sync_selftest(ctx.h, int(rounds), int(skip_block), float(limit_ms)))


class BatchSystem:
    """Many independent single-site AdResS replicas advanced together (mrmd_batch_*).

    `replicas` is a list of Replica; pos/vel are the replicas' molecules
    concatenated in that order.  Physics parameters are shared, as in
    AdResSSystem; the tuning (lanes per row, block size, rebuild interval,
    sort interval, graph length, list layout) can be set or picked by autotune().
    List layouts: 0 one row per molecule, 1 near and far rows (mixed form),
    2 8 x 4 cluster pairs (threads_per_row 4)."""

    def __init__(self, replicas, pos, vel, hybrid_diameter, nu=1, rc=2.5, skin=0.3, sigma=1.0,
                 epsilon=1.0, capping_distance=0.0, shifted=True, precision=PREC_FP64, dt=0.005,
                 gamma=1.0, temperature=1.0, tf=True, tf_bin_width=1.2, tf_target_density=0.5,
                 tf_modulation=1.0, tf_sigma=2.4, tf_range=3.0, tf_sample_interval=1,
                 tf_update_interval=1000, comp_sampling_interval=0, comp_update_interval=0, comp_frozen=False,
                 threads_per_row=1, block_size=128, rebuild_interval=10, sort_every=5, graph_steps=50,
                 list_layout=0, initial_max_neighbors=0, initial_ghost_capacity=0, persistent=False,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        pos = _f64(pos)
        vel = _f64(vel)
        self.replicas = list(replicas)
        self.sizes = np.array([r.num_molecules for r in self.replicas], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        self.n = int(self.offsets[-1])
        if pos.shape != (self.n, 3) or vel.shape != (self.n, 3):
            raise ValueError("pos/vel must be [sum of replica sizes][3]")
        c = _abi.BatchConfigS()
        c.rc, c.skin, c.sigma, c.epsilon = rc, skin, sigma, epsilon
        c.cappingDistance = capping_distance
        c.shifted = int(bool(shifted))
        c.precision = int(precision)
        c.dt = dt
        c.hybridDiameter, c.nu = hybrid_diameter, int(nu)
        c.gamma, c.temperature = gamma, temperature
        c.tfEnabled = int(bool(tf))
        c.tfBinWidth, c.tfTargetDensity, c.tfModulation = tf_bin_width, tf_target_density, tf_modulation
        c.tfSmoothingSigma, c.tfSmoothingRange = tf_sigma, tf_range
        c.tfSampleInterval, c.tfUpdateInterval = int(tf_sample_interval), int(tf_update_interval)
        c.compSamplingInterval, c.compUpdateInterval = int(comp_sampling_interval), int(comp_update_interval)
        c.compFrozen = int(bool(comp_frozen))
        c.initialMaxNeighbors, c.initialGhostCapacity = int(initial_max_neighbors), int(initial_ghost_capacity)
        c.tuning = _tuning_struct(dict(threads_per_row=threads_per_row, block_size=block_size,
                                       rebuild_interval=rebuild_interval, sort_every=sort_every,
                                       graph_steps=graph_steps, list_layout=list_layout,
                                       persistent=int(bool(persistent))))
        self.cfg = c
        reps = (_abi.ReplicaS * len(self.replicas))(*[r._struct() for r in self.replicas])
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.mrmd_batch_create(self.ctx.h, C.byref(h), C.byref(c), len(self.replicas),
                                                      reps, _dp(pos), _dp(vel)), "BatchSystem")
        self.h = h

    @property
    def num_replicas(self):
        return len(self.replicas)

    def run(self, nsteps: int, energies: bool = True):
        """Advance nsteps; returns the [nsteps][replicas] LJ_IdealGas energies."""
        e = np.zeros((max(nsteps, 1), self.num_replicas)) if energies else None
        self.ctx.check(self.ctx.lib.mrmd_batch_run(self.ctx.h, self.h, int(nsteps), _dp(e)), "run")
        return e[:nsteps] if energies else None

    def state(self):
        p, v, f = (np.zeros((self.n, 3)) for _ in range(3))
        self.ctx.check(self.ctx.lib.mrmd_batch_get_state(self.ctx.h, self.h, _dp(p), _dp(v), _dp(f)), "state")
        return p, v, f

    def replica_slice(self, r):
        return slice(int(self.offsets[r]), int(self.offsets[r + 1]))

    def thermodynamic_force(self):
        """(tables, densities): lists with one array per replica."""
        off = np.zeros(self.num_replicas + 1, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_batch_get_tf(self.ctx.h, self.h, None, None, _ip(off)), "tf")
        f, d = np.zeros(max(int(off[-1]), 1)), np.zeros(max(int(off[-1]), 1))
        self.ctx.check(self.ctx.lib.mrmd_batch_get_tf(self.ctx.h, self.h, _dp(f), _dp(d), None), "tf")
        return ([f[off[r]:off[r + 1]] for r in range(self.num_replicas)],
                [d[off[r]:off[r + 1]] for r in range(self.num_replicas)])

    def set_thermodynamic_force(self, tables):
        self.ctx.check(self.ctx.lib.mrmd_batch_set_tf(self.ctx.h, self.h, _dp(_f64(np.concatenate(tables)))),
                       "set tf")

    def compensation(self):
        m = np.zeros((self.num_replicas, 200))
        self.ctx.check(self.ctx.lib.mrmd_batch_get_compensation(self.ctx.h, self.h, _dp(m)), "compensation")
        return m

    def set_compensation(self, mean):
        m = _f64(np.broadcast_to(mean, (self.num_replicas, 200)).copy())
        self.ctx.check(self.ctx.lib.mrmd_batch_set_compensation(self.ctx.h, self.h, _dp(m)), "set compensation")

    @property
    def tuning(self):
        t = _abi.BatchTuningS()
        self.ctx.lib.mrmd_batch_get_tuning(self.h, C.byref(t))
        return _tuning_dict(t)

    @tuning.setter
    def tuning(self, d):
        t = _tuning_struct({**self.tuning, **d})
        self.ctx.check(self.ctx.lib.mrmd_batch_set_tuning(self.ctx.h, self.h, C.byref(t)), "tuning")

    def autotune(self, trial_steps=50):
        """Time the candidate tunings from the current state and keep the fastest safe one.
        Returns (best, [(candidate, ms_per_step or None if rejected), ...])."""
        best = _abi.BatchTuningS()
        ms = np.zeros(64)
        cands = (_abi.BatchTuningS * 64)()
        n = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_batch_autotune(self.ctx.h, self.h, int(trial_steps), C.byref(best),
                                                        _dp(ms), cands, C.byref(n)), "autotune")
        trials = [(_tuning_dict(cands[k]), float(ms[k]) if ms[k] >= 0 else None) for k in range(n.value)]
        return _tuning_dict(best), trials

    def stats(self):
        out = np.zeros(10, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_batch_stats(self.ctx.h, self.h, _ip(out)), "stats")
        keys = ["steps", "rebuilds", "pairs", "ghost_molecules", "graph_launches", "kernel_launches",
                "recoveries", "list_capacity", "ghost_capacity", "flags"]
        return {k: int(v) for k, v in zip(keys, out)}

    def pair_keys(self, replica: int):
        """Sorted canonical keys a * 2^32 + b (a < b, molecule indices in the
        replica's input order) of every pair the force kernel evaluates in the
        current list of one replica."""
        cnt = C.c_int64()
        self.ctx.check(self.ctx.lib.mrmd_batch_pair_keys(self.ctx.h, self.h, int(replica), None, 0, C.byref(cnt)),
                       "batch_pair_keys")
        keys = np.zeros(max(cnt.value, 1), dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_batch_pair_keys(self.ctx.h, self.h, int(replica), _ip(keys), len(keys),
                                                         C.byref(cnt)), "batch_pair_keys")
        return keys[: cnt.value]

    def list_stats(self):
        """The list of the last rebuild: pairs, entries, pair slots per entry and
        the fraction of the pair kernel's lanes that evaluate a listed pair."""
        out = np.zeros(3, dtype=np.int64)
        self.ctx.check(self.ctx.lib.mrmd_batch_list_stats(self.ctx.h, self.h, _ip(out)), "list_stats")
        pairs, entries, slots = (int(v) for v in out)
        return dict(pairs=pairs, entries=entries, slots_per_entry=slots,
                    lane_efficiency=pairs / (entries * slots) if entries else 0.0)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.mrmd_batch_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DiffSystem:
    """One AdResS system with the adjoint of its trajectory loss (mrmd_diff_*).

    forward(table, epsilon, sigma) runs `steps` steps from the initial state and
    returns the loss: sum_b (rho_b - rho_uniform)^2 of the Gaussian-smoothed
    (loss_sigma, loss_bins) x-density averaged over the last `window` steps.
    backward() returns (dL/dtable, dL/depsilon, dL/dsigma) of that run.  The
    compensation means are held fixed and the TF table is not updated inside
    the trajectory."""

    def __init__(self, replica, pos, vel, hybrid_diameter, steps=500, window=100, checkpoint_interval=25,
                 loss_bins=128, loss_sigma=1.0, nu=1, rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0,
                 capping_distance=0.0, shifted=True, precision=PREC_FP64, dt=0.005, gamma=1.0,
                 temperature=1.0, tf_bin_width=1.2, rebuild_interval=5, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        pos = _f64(pos)
        vel = _f64(vel)
        self.n = len(pos)
        c = _abi.BatchConfigS()
        c.rc, c.skin, c.sigma, c.epsilon = rc, skin, sigma, epsilon
        c.cappingDistance = capping_distance
        c.shifted = int(bool(shifted))
        c.precision = int(precision)
        c.dt = dt
        c.hybridDiameter, c.nu = hybrid_diameter, int(nu)
        c.gamma, c.temperature = gamma, temperature
        c.tfEnabled = 1
        c.tfBinWidth, c.tfTargetDensity, c.tfModulation = tf_bin_width, 0.5, 1.0
        c.tfSmoothingSigma, c.tfSmoothingRange = 1.0, 1.0
        c.tfSampleInterval, c.tfUpdateInterval = 1, int(steps) + 1
        c.tuning = _tuning_struct(dict(threads_per_row=1, block_size=128, rebuild_interval=rebuild_interval,
                                       sort_every=0, graph_steps=0))
        dc = _abi.DiffConfigS(int(steps), int(window), int(checkpoint_interval), int(loss_bins), float(loss_sigma))
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.mrmd_diff_create(self.ctx.h, C.byref(h), C.byref(c), C.byref(replica._struct()),
                                                     _dp(pos), _dp(vel), C.byref(dc)), "DiffSystem")
        self.h = h
        nb = C.c_int64()
        self.ctx.lib.mrmd_diff_num_bins(self.h, C.byref(nb))
        self.num_bins = int(nb.value)

    def set_state(self, pos, vel):
        self.ctx.check(self.ctx.lib.mrmd_diff_set_state(self.ctx.h, self.h, _dp(_f64(pos)), _dp(_f64(vel))),
                       "set_state")

    def forward(self, table, epsilon, sigma):
        loss = C.c_double()
        t = None if table is None else _f64(table)
        self.ctx.check(self.ctx.lib.mrmd_diff_forward(self.ctx.h, self.h, _dp(t), float(epsilon), float(sigma),
                                                      C.byref(loss)), "forward")
        return float(loss.value)

    def backward(self):
        gt = np.zeros(max(self.num_bins, 1))
        ge, gs = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.mrmd_diff_backward(self.ctx.h, self.h, _dp(gt), C.byref(ge), C.byref(gs)),
                       "backward")
        return gt[:self.num_bins], float(ge.value), float(gs.value)

    def force_vjp(self, table, epsilon, sigma, adjoint):
        f, xb = np.zeros((self.n, 3)), np.zeros((self.n, 3))
        gt = np.zeros(max(self.num_bins, 1))
        ge, gs = C.c_double(), C.c_double()
        t = None if table is None else _f64(table)
        self.ctx.check(self.ctx.lib.mrmd_diff_force_vjp(self.ctx.h, self.h, _dp(t), float(epsilon), float(sigma),
                                                        _dp(_f64(adjoint, (self.n, 3))), _dp(f), _dp(xb), _dp(gt),
                                                        C.byref(ge), C.byref(gs)), "force_vjp")
        return f, xb, gt[:self.num_bins], float(ge.value), float(gs.value)

    def state(self):
        p, v = np.zeros((self.n, 3)), np.zeros((self.n, 3))
        self.ctx.check(self.ctx.lib.mrmd_diff_get_state(self.ctx.h, self.h, _dp(p), _dp(v)), "state")
        return p, v

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.mrmd_diff_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def version() -> str:
    return _abi.lib().mrmd_version().decode()
