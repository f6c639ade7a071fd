"""GPU test of anigpu_assemble_noalloc, the allocation-free assembly entry point for callers
that cannot allocate device memory when they assemble (device memory held by another
allocator, latency-critical loops).  It is called through the C ABI and must give the same
matrix and right-hand side as anigpu_assemble, on two calls in a row (the calls share one
fixed device array that keeps the previous call's contents).  This file sorts last so that a
run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(lib, n, perturb, space=None):
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=perturb, seed=3)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.P2 if space is None else space)
    lib.set_dirichlet(meshgen.boundary_mask(lib.dof_coords().cpu().numpy()))
    return meshgen.aniso_tensors(tets.shape[0], 1.5, 4)


def _call(lib, kind, Dd, precision, vals, rhs):
    import anigpu
    with lib.on_stream():
        return lib.lib.anigpu_assemble_noalloc(lib.h, kind, ctypes.c_void_p(Dd.data_ptr()) if Dd is not None else None,
                                               None, 1.0, 4, precision, ctypes.c_void_p(vals.data_ptr()),
                                               ctypes.c_void_p(rhs.data_ptr()), 1e-100)


@pytest.mark.parametrize("space", ["P1", "P2"])
@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_assemble(lib, precision, space):
    import torch

    import anigpu
    D = _setup(lib, 6, 0.2, getattr(anigpu, space))
    ref_vals, ref_rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, precision)
    dt = torch.float64 if precision == anigpu.F64 else torch.float32
    Dd = torch.tensor(D, device="cuda")
    for call in range(2):
        vals = torch.full((lib.nnz,), 7.0, dtype=dt, device="cuda")  # garbage the call must overwrite
        rhs = torch.full((lib.ndof,), 7.0, dtype=torch.float64, device="cuda")
        rc = _call(lib, anigpu.TENSOR_TET_SYM, Dd, precision, vals, rhs)
        assert rc == 0, lib.lib.anigpu_last_error(lib.h).decode()
        torch.cuda.synchronize()
        tol = 1e-12 if precision == anigpu.F64 else 1e-6
        v, rv = vals.double().cpu().numpy(), ref_vals.double().cpu().numpy()
        assert np.abs(v - rv).max() <= tol * np.abs(rv).max(), call
        r, rr = rhs.cpu().numpy(), ref_rhs.cpu().numpy()
        assert np.abs(r - rr).max() <= tol * np.abs(rr).max(), call


def _soup(lib, nt):
    """nt separate tets (each with its own four vertices) set up as a P1 problem."""
    import anigpu
    from anigpu import meshgen
    XY = meshgen.random_tets(nt, seed=11)
    lib.mesh_upload(XY.reshape(-1, 3), np.arange(4 * nt, dtype=np.int32).reshape(nt, 4))
    lib.problem_setup(anigpu.P1)


@pytest.mark.parametrize("prec_name,limit", [("F64", 262_144), ("F32", 524_288)])
def test_noalloc_limit_is_exact(lib, prec_name, limit):
    """A mesh of exactly the documented number of tets is accepted, one more is rejected."""
    import torch

    import anigpu
    precision = getattr(anigpu, prec_name)
    dt = torch.float64 if precision == anigpu.F64 else torch.float32
    for nt, ok in ((limit, True), (limit + 1, False)):
        _soup(lib, nt)
        vals = torch.empty(lib.nnz, dtype=dt, device="cuda")
        rhs = torch.empty(lib.ndof, dtype=torch.float64, device="cuda")
        rc = _call(lib, anigpu.TENSOR_NULL, None, precision, vals, rhs)
        if ok:
            assert rc == 0, lib.lib.anigpu_last_error(lib.h).decode()
            torch.cuda.synchronize()
            # GRAD.GRAD kills constants: every row of a lone P1 tet sums to zero
            rp, _ = lib.csr_template()
            v = vals.double().cpu().numpy()
            row_sums = np.add.reduceat(v, rp.cpu().numpy()[:-1])
            assert np.abs(row_sums).max() <= (1e-12 if precision == anigpu.F64 else 1e-5) * np.abs(v).max()
        else:
            assert rc == anigpu.ERR_ARG
            assert "fixed scratch" in lib.lib.anigpu_last_error(lib.h).decode()


def test_noalloc_rejects_meshes_above_the_limit(lib):
    import torch

    import anigpu
    _setup(lib, 50, 0.0)  # 750,000 tets > 524,288
    vals = torch.empty(lib.nnz, dtype=torch.float32, device="cuda")
    rhs = torch.empty(lib.ndof, dtype=torch.float64, device="cuda")
    with lib.on_stream():
        rc = lib.lib.anigpu_assemble_noalloc(lib.h, anigpu.TENSOR_NULL, None, None, 1.0, 4, anigpu.F32,
                                             ctypes.c_void_p(vals.data_ptr()), ctypes.c_void_p(rhs.data_ptr()),
                                             1e-100)
    assert rc == anigpu.ERR_ARG
    assert "fixed scratch" in lib.lib.anigpu_last_error(lib.h).decode()
