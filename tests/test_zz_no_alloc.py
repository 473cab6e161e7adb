"""mrmd_lj_apply_mixed_noalloc: the mixed-form LJ pair force for callers that
cannot allocate device memory inside their step loop (the free memory
belongs to another allocator, or a cudaMalloc and its synchronisation are
not allowed there).  Checked through the C ABI against mrmd_lj_apply in the
mixed form, on two calls in a row (the fixed scratch array keeps the last
call's contents, so the second call must not see the first one's sums)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # the parity tolerance of the other GPU tests


def fcc(cells, rho=0.8442):
    a = (4.0 / rho) ** (1.0 / 3.0)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(cells)] * 3, indexing="ij"), -1).reshape(-1, 3)
    return ((g[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a, a * cells


def test_noalloc_matches_mixed_apply_twice():
    import mrmd_gb300 as M
    from mrmd_gb300 import _abi

    lib = _abi.lib()
    ctx = M.Context(0)
    pos, L = fcc(12)  # 6,912 atoms
    pos = pos + np.random.default_rng(3).normal(0, 0.05, pos.shape)
    rc, skin = 2.5, 0.3
    atoms = M.Atoms.from_arrays(pos, capacity=20000, ctx=ctx)
    sd = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    gl = M.GhostLayer(ctx)
    gl.createGhostAtoms(atoms, sd)
    assert atoms.size <= 262144
    vl = M.HalfVerletList(ctx)
    vl.build(atoms, 0, atoms.numLocalAtoms, rc + skin, 1.0, sd.minGhostCorner, sd.maxGhostCorner, 64)
    lj = M.LennardJones(rc, 1.0, 1.0, is_shifted=True, ctx=ctx)

    atoms.setForce(0.0)
    lj.apply(atoms, vl, precision=M.PREC_MIXED)
    f_ref = atoms.getForce()
    e_ref, w_ref = lj.getEnergy(), lj.getVirial()

    for call in range(2):
        atoms.setForce(0.0)
        e, w = C.c_double(), C.c_double()
        rc_ = lib.mrmd_lj_apply_mixed_noalloc(ctx.h, lj.h, C.byref(atoms.s), C.byref(vl.s), None,
                                              C.byref(e), C.byref(w))
        assert rc_ == 0, lib.mrmd_ctx_last_error(ctx.h)
        f = atoms.getForce()
        scale = np.abs(f_ref).max()
        assert np.abs(f - f_ref).max() <= RTOL * scale, call
        assert abs(e.value - e_ref) <= RTOL * abs(e_ref), call
        assert abs(w.value - w_ref) <= RTOL * abs(w_ref), call


def test_noalloc_rejects_too_many_atoms():
    import mrmd_gb300 as M
    from mrmd_gb300 import _abi

    lib = _abi.lib()
    ctx = M.Context(0)
    big = M.Atoms(262144 + 16, ctx=ctx)
    big.numLocalAtoms = 262144 + 16
    vl = M.HalfVerletList(ctx)
    lj = M.LennardJones(2.5, 1.0, 1.0, ctx=ctx)
    rc_ = lib.mrmd_lj_apply_mixed_noalloc(ctx.h, lj.h, C.byref(big.s), C.byref(vl.s), None, None, None)
    assert rc_ == -8  # MRMD_ERR_CAPACITY
    assert b"exceed the fixed scratch" in lib.mrmd_ctx_last_error(ctx.h)
