"""io::dumpThermoForce / io::restoreThermoForce (io/DumpThermoForce.cpp,
io/RestoreThermoForce.cpp) and the host-side table text they use.

The text is the reference's: the bin centres on the first line, one line of
forces per type, values written with C++ stream defaults (6 significant
digits).  ``write_table`` and ``read_table`` run on the host alone (no GPU
context); ``dumpThermoForce`` and ``restoreThermoForce`` move the table
between the file and a device ``ThermodynamicForce``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import Context, MrmdError, Subdomain, ThermodynamicForce, _abi, _dp, _f64, default_context


def _path(filename) -> bytes:
    return os.fsencode(os.fspath(filename))


def write_table(filename, grid, force, type_id=None):
    """The text of dumpThermoForce for host arrays grid [numBins] and
    force [numBins][numTypes]; ``type_id`` None writes every type."""
    grid = _f64(grid)
    force = _f64(force)
    if force.ndim == 1:
        force = force.reshape(-1, 1)
    if force.shape[0] != grid.shape[0]:
        raise MrmdError(-1, "write_table: force and grid differ in the number of bins")
    rc = _abi.lib().mrmd_tf_write_table(None, _path(filename), grid.shape[0], _dp(grid), force.shape[1],
                                        _dp(force), -1 if type_id is None else int(type_id))
    if rc != 0:
        raise MrmdError(rc, f"write_table: cannot write {filename}")


def read_table(filename, max_num_forces=10):
    """The parser of restoreThermoForce: returns (grid, force [numBins][numForces],
    binWidth = grid[1] - grid[0])."""
    lib = _abi.lib()
    nb, nf, bw = C.c_int64(), C.c_int64(), C.c_double()
    rc = lib.mrmd_tf_read_table(None, _path(filename), int(max_num_forces), C.byref(nb), C.byref(nf),
                                C.byref(bw), None, None, 0)
    if rc != 0:
        raise MrmdError(rc, f"read_table: {filename} is not a thermodynamic-force table")
    grid = np.zeros(nb.value)
    force = np.zeros((nb.value, nf.value))
    rc = lib.mrmd_tf_read_table(None, _path(filename), int(max_num_forces), None, None, None, _dp(grid),
                                _dp(force), force.size)
    if rc != 0:
        raise MrmdError(rc, f"read_table: {filename} changed while reading")
    return grid, force, bw.value


def dumpThermoForce(filename, thermodynamic_force: ThermodynamicForce, type_id=None):
    """io::dumpThermoForce (io/DumpThermoForce.cpp:24-64)."""
    tf = thermodynamic_force
    tf.ctx.check(tf.ctx.lib.mrmd_tf_dump(tf.ctx.h, tf.h, _path(filename),
                                        -1 if type_id is None else int(type_id)), "dumpThermoForce")


def restoreThermoForce(filename, subdomain: Subdomain, target_densities=(1.0,), modulations=(1.0,),
                       enforce_symmetry=False, use_periodicity=False, max_num_forces=10,
                       ctx: Context | None = None) -> ThermodynamicForce:
    """io::restoreThermoForce (io/RestoreThermoForce.cpp:24-90)."""
    ctx = ctx or default_context()
    td = np.atleast_1d(np.asarray(target_densities, dtype=np.float64))
    mod = np.atleast_1d(np.asarray(modulations, dtype=np.float64))
    if len(td) != len(mod):
        raise MrmdError(-1, "restoreThermoForce: one modulation per target density")
    h = C.c_void_p()
    ctx.check(ctx.lib.mrmd_tf_restore(ctx.h, C.byref(h), _path(filename), C.byref(subdomain.s), len(td),
                                      _dp(td), _dp(mod), int(bool(enforce_symmetry)),
                                      int(bool(use_periodicity)), int(max_num_forces)), "restoreThermoForce")
    return ThermodynamicForce._adopt(h, ctx)
