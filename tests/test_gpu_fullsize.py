"""GPU parity at the benchmark sizes: the P2 anisotropic-diffusion system on 64^3 x 6 perturbed Kuhn
tets (1,572,864 tets, 60.9 M nnz) and the vector-P2 elasticity system on 48^3 x 6 (663,552 tets,
232 M nnz), assembled on the GPU in FP64 and FP32 and by the oracle on all host cores
(oracle.Restated.assemble_problem_mt: the restated assembler split over tets and rows, bitwise equal
to the serial one).  FP64: template bit-exact, values and right-hand side within 1e-12 of the
largest value.  FP32: the error per row against the FP64 oracle (max and median printed) stays
within the FP32 bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _row_errors(rowptr, ref, got):
    n = rowptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    rown = np.sqrt(np.bincount(rows, ref ** 2, minlength=n))
    return np.sqrt(np.bincount(rows, (got - ref) ** 2, minlength=n)) / np.maximum(rown, 1e-300)


def test_p2_aniso_64_matches_oracle(lib, restated):
    import anigpu
    from anigpu import meshgen
    xyz, tets, D6 = meshgen.p2_aniso_workload(64)
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(anigpu.P2)
    mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy())
    lib.set_dirichlet(mask)
    v64, r64, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D6, None, 1.0, 4, anigpu.F64)
    v32, r32, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D6, None, 1.0, 4, anigpu.F32)
    ref = restated.assemble_problem_mt(xyz, tets, 2, 3, D6, 1.0, 4, dirichlet=(mask, None))
    rp, col = lib.csr_template()
    assert np.array_equal(rp.cpu().numpy(), ref["rowptr"])
    assert np.array_equal(col.cpu().numpy(), ref["col"])
    vmax = np.abs(ref["vals"]).max()
    assert np.abs(v64.cpu().numpy() - ref["vals"]).max() <= 1e-12 * vmax
    assert np.abs(r64.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()
    err = _row_errors(ref["rowptr"], ref["vals"], v32.double().cpu().numpy())
    print(f"64^3 P2 FP32 per-row error: max {err.max():.2e} median {np.median(err):.2e}; "
          f"tets redone in FP64 geometry: {meshgen.fp64_redo_count(xyz, tets)}")
    assert err.max() <= 1e-4
    assert np.abs(r32.cpu().numpy() - ref["rhs"]).max() <= 1e-5 * np.abs(ref["rhs"]).max()


def test_elasticity_48_matches_oracle(lib, restated):
    import anigpu
    from anigpu import meshgen
    xyz, tets, LM = meshgen.elasticity_workload(48)
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(anigpu.VEC3_P2)
    coords = lib.dof_coords().cpu().numpy()
    mask = (np.abs(coords[:, 0]) < 1e-12).astype(np.uint8)
    lib.set_dirichlet(mask)
    v64, r64, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.0, 4, anigpu.F64)
    v32, _, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.0, 4, anigpu.F32)
    ref = restated.assemble_problem_mt(xyz, tets, 5, 4, meshgen.lame9(LM[:, 0], LM[:, 1]), 0.0, 4,
                                       dirichlet=(mask, None))
    rp, col = lib.csr_template()
    assert np.array_equal(rp.cpu().numpy(), ref["rowptr"])
    assert np.array_equal(col.cpu().numpy(), ref["col"])
    vmax = np.abs(ref["vals"]).max()
    assert np.abs(v64.cpu().numpy() - ref["vals"]).max() <= 1e-12 * vmax
    err = _row_errors(ref["rowptr"], ref["vals"], v32.double().cpu().numpy())
    print(f"48^3 vector P2 FP32 per-row error: max {err.max():.2e} median {np.median(err):.2e}")
    assert err.max() <= 1e-4
