"""GPU parity of the batched fem3Dtet (anigpu_fem3dtet) against the reference's own
fem3Dtet outputs (tests/golden/golden.npz) and the reference's golden matrices."""
import numpy as np
import pytest

from helpers import KIND_CODE, op_nf_dim, parse_case, point_tensor, ref_tol, rel_err_per_tet


def op_info(code):
    import anigpu
    return anigpu.op_info(code)

pytestmark = pytest.mark.gpu


def _run_case(lib, golden, name, precision):
    import anigpu
    XY = golden["tets_XY"]
    ca, cb, kind, order = parse_case(name)
    nfA, dA = op_nf_dim(ca)
    nfB, dB = op_nf_dim(cb)
    if kind.startswith("point"):
        fn = int(kind[5:])
        q = lib.quadrature_points(order, XY).cpu().numpy()
        D = point_tensor(fn, q, dB, dA)
        A = lib.fem3dtet(ca, cb, XY, D, anigpu.TENSOR_POINT, order, precision)
    else:
        D = golden[f"case_{name}_D"] if f"case_{name}_D" in golden.files else None
        A = lib.fem3dtet(ca, cb, XY, D, KIND_CODE[kind], order, precision)
    return A.double().cpu().numpy()


def test_fem3dtet_f64_matches_reference(lib, golden):
    import anigpu
    worst = 0.0
    for name in golden["case_names"]:
        name = str(name)
        A = _run_case(lib, golden, name, anigpu.F64)
        err = rel_err_per_tet(A, golden[f"case_{name}_A"])
        worst = max(worst, err)
        assert err <= 1e-12, (name, err)
    print("worst FP64 relative error per tet:", worst)


def test_fem3dtet_f32_error_bound(lib, golden):
    import anigpu
    worst = 0.0
    for name in golden["case_names"]:
        name = str(name)
        A = _run_case(lib, golden, name, anigpu.F32)
        err = rel_err_per_tet(A, golden[f"case_{name}_A"])
        worst = max(worst, err)
        assert err <= 2e-5, (name, err)
    print("worst FP32 relative error per tet:", worst)


def _run_sliver(lib, golden, name, precision):
    from helpers import KIND_CODE
    XY = golden["sliver_XY"]
    ca, cb, kind, order = parse_case(name)
    D = golden[f"sliver_{name}_D"] if f"sliver_{name}_D" in golden.files else None
    return lib.fem3dtet(ca, cb, XY, D, KIND_CODE[kind], order, precision).double().cpu().numpy()


def test_fem3dtet_slivers_f64_matches_reference(lib, golden):
    """Badly shaped tets (|det| / (|e1||e2||e3|) from 0.58 down to 1e-6): FP64 within 1e-12 of the
    reference's fem3Dtet."""
    import anigpu
    for name in golden["sliver_case_names"]:
        name = str(name)
        err = rel_err_per_tet(_run_sliver(lib, golden, name, anigpu.F64), golden[f"sliver_{name}_A"])
        assert err <= 1e-12, (name, err)


def test_fem3dtet_slivers_f32_error(lib, golden):
    """The FP32 kernels on the same tets: those with |det| <= 0.05 |e1||e2||e3| take the FP64
    geometry branch; every tet stays within the FP32 bound of 2e-5 relative (Frobenius, per tet)."""
    import anigpu
    XY = golden["sliver_XY"].reshape(-1, 4, 3)
    e = XY[:, 1:] - XY[:, :1]
    ratio = np.abs(np.linalg.det(e)) / np.prod(np.linalg.norm(e, axis=2), axis=1)
    assert (ratio <= 0.05).sum() >= 10 and (ratio > 0.05).sum() >= 5  # both branches are exercised
    worst = 0.0
    for name in golden["sliver_case_names"]:
        name = str(name)
        err = rel_err_per_tet(_run_sliver(lib, golden, name, anigpu.F32), golden[f"sliver_{name}_A"])
        worst = max(worst, err)
        assert err <= 2e-5, (name, err)
    print("worst FP32 relative error per tet on slivers:", worst)


def test_golden_matrices_on_gpu(lib, golden):
    import anigpu
    XY = golden["int_tet_test_tet_onepoint"].reshape(1, 12)
    exp = golden["int_tet_test_onepoint_12x20"] / golden["int_tet_test_onepoint_coef"]
    for order in (5, 6):
        q = lib.quadrature_points(order, XY).cpu().numpy()
        D = point_tensor(0, q, 9, 3)
        A = lib.fem3dtet(32, 42, XY, D, anigpu.TENSOR_POINT, order).cpu().numpy()[0].T
        assert np.linalg.norm(A - exp) <= ref_tol(A)
    exp = golden["int_tet_test_vecp1_12x12"] / golden["int_tet_test_vecp1_coef"]
    for kind, D in ((anigpu.TENSOR_NULL, None), (anigpu.TENSOR_CONST_SCALAR, np.array([1.0])),
                    (anigpu.TENSOR_TET_GENERAL, np.eye(9).reshape(1, 81))):
        A = lib.fem3dtet(42, 42, XY, D, kind, 5).cpu().numpy()[0].T
        assert np.linalg.norm(A - exp) <= ref_tol(A)
    Bp = golden["int_tet_test_rhs_Bp"]
    XYr = golden["int_tet_test_tet_rhs"].reshape(1, 12)
    for k in (1, 2):
        A = lib.fem3dtet(1, 51, XYr, np.array([40.0 * k]), anigpu.TENSOR_CONST_SCALAR, 2).cpu().numpy()[0, 0]
        assert np.linalg.norm(A - k * Bp) <= ref_tol(A)


def test_fem3dtet_large_batch_vs_oracle(lib, restated):
    """A batch larger than the grid (grid-stride loop) against the restated oracle."""
    import anigpu
    from anigpu import meshgen
    XY = meshgen.random_tets(5000, seed=77)
    D6 = meshgen.aniso_tensors(5000, 1.5, 78)
    A = lib.fem3dtet(22, 22, XY, D6, anigpu.TENSOR_TET_SYM, 4).cpu().numpy()
    Ao = restated.fem3dtet(22, 22, 3, 4, XY, D6)
    assert rel_err_per_tet(A, Ao) <= 1e-12


def test_apply_dir_on_gpu(lib, restated):
    import torch
    rng = np.random.default_rng(3)
    nt, n = 7, 10
    A = rng.standard_normal((nt, n, n))
    F = rng.standard_normal((nt, n))
    mask = rng.integers(0, 1 << n, nt).astype(np.int32)
    bc = rng.standard_normal((nt, n))
    Ad = torch.tensor(A, device="cuda")
    Fd = torch.tensor(F, device="cuda")
    lib.apply_dir(Ad, Fd, mask, bc)
    torch.cuda.synchronize()
    for t in range(nt):
        a, f = A[t].copy(), F[t].copy()
        for k in range(n):
            if (mask[t] >> k) & 1:
                restated.apply_dir(a, f, k, bc[t, k])
        assert np.array_equal(Ad[t].cpu().numpy(), a)
        assert np.allclose(Fd[t].cpu().numpy(), f, rtol=0, atol=1e-14)


def test_errors_are_reported(lib):
    import anigpu
    XY = np.zeros((1, 12))
    with pytest.raises(anigpu.AnigpuError) as e:
        lib.fem3dtet(22, 22, XY, None, anigpu.TENSOR_NULL, 21)  # order above 20
    assert e.value.code == anigpu.ERR_UNSUPPORTED
    with pytest.raises(anigpu.AnigpuError) as e:
        lib.fem3dtet(22, 21, XY, None, anigpu.TENSOR_NULL, 2)  # identity of incompatible dims (3 vs 1)
    assert e.value.code == anigpu.ERR_ARG


def test_fem3d_apply_matches_reference(lib, golden):
    """anigpu_fem3d_apply / _apply_x (FP64) against the reference's fem3DapplyL / fem3DapplyX
    outputs for every operator code: within 1e-12 of the largest value per tet."""
    XY = golden["tets_XY"]
    for code in golden["apply_codes"]:
        code = int(code)
        dofs = golden[f"apply_{code}_dofs"]
        got_l = lib.fem3d_apply(code, XY, golden["apply_XYL"], dofs).cpu().numpy()
        got_x = lib.fem3d_apply_x(code, XY, golden["apply_X"], dofs).cpu().numpy()
        for got, ref in ((got_l, golden[f"apply_{code}_L"]), (got_x, golden[f"apply_{code}_X"])):
            assert got.shape == ref.shape
            scale = np.maximum(np.abs(ref).reshape(ref.shape[0], -1).max(axis=1), 1e-300)
            err = np.abs(got - ref).reshape(ref.shape[0], -1).max(axis=1) / scale
            assert err.max() <= 1e-12, (code, err.max())


@pytest.mark.parametrize("space", [1, 2, 5])
def test_eval_solution_matches_oracle_and_reproduces_quadratics(lib, restated, space):
    """anigpu_eval_solution on a set-up problem: IDEN and GRAD of a global vector at the order-4
    quadrature points equal the restated fem3DapplyL on the gathered element DOFs; the P2
    interpolant of a quadratic field reproduces the field and its gradient exactly."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(4, perturb=0.2, seed=3)
    lib.mesh_upload(xyz, tets)
    ndof, _ = lib.problem_setup(space)
    ncomp = 3 if space == 5 else 1
    ot = restated.orient(xyz, tets)
    XY = xyz[ot].reshape(-1, 12)
    ed = lib.element_dofs().cpu().numpy()
    nds = ndof // ncomp
    p4, _ = restated.quadrature(4)
    x = meshgen.normal(77 + space, ndof)
    gd = np.concatenate([x[c * nds + ed] for c in range(ncomp)], axis=1)  # [nt, ncomp*nloc]
    base = {1: 1, 2: 2, 5: 2}[space]
    code_space = space if space != 5 else 5
    for op in (anigpu.IDEN, anigpu.GRAD):
        got = lib.eval_solution(op, x, p4).cpu().numpy()
        ref = restated.fem3d_apply(10 * code_space + op, XY, p4, gd)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), op
    if base == 2:
        c = lib.dof_coords().cpu().numpy()
        f = lambda P: P[..., 0] ** 2 + P[..., 1] * P[..., 2] - 0.5 * P[..., 2]  # noqa: E731
        u = f(c)
        val = lib.eval_solution(anigpu.IDEN, u, p4).cpu().numpy()
        grad = lib.eval_solution(anigpu.GRAD, u, p4).cpu().numpy()
        XG = restated.quad_points(4, XY)
        gx = np.stack([2 * XG[..., 0], XG[..., 2], XG[..., 1] - 0.5], axis=-1)
        k = ncomp  # every component holds the same field when ncomp = 3
        assert np.abs(val[..., 0] - f(XG)).max() <= 1e-12
        assert np.abs(grad[..., :3] - gx).max() <= 1e-11
        if k == 3:
            assert np.abs(val[..., 2] - f(XG)).max() <= 1e-12


def test_fem3dface_matches_reference(lib, golden):
    """anigpu_fem3dface (FP64) against the reference's fem3Dface on every face, orders 1-9, constant,
    per-tet and per-point tensors: within 1e-12 per tet."""
    import anigpu
    XY = golden["tets_XY"]
    for name in golden["face_case_names"]:
        name = str(name)
        ca, cb = (int(v) for v in name.split("_")[:2])
        kname, order, face = name.split("_")[2], int(name.split("_")[3][1:]), int(name.split("_")[4][1:])
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        if kname.startswith("point"):
            q = lib.face_quadrature_points(order, face, XY).cpu().numpy()
            D = point_tensor(int(kname[5:]), q, dB, dA)
            A = lib.fem3dface(ca, cb, XY, face, D, anigpu.TENSOR_POINT, order)
        else:
            D = golden[f"face_{name}_D"] if f"face_{name}_D" in golden.files else None
            A = lib.fem3dface(ca, cb, XY, face, D, KIND_CODE[kname], order)
        err = rel_err_per_tet(A.cpu().numpy(), golden[f"face_{name}_A"])
        assert err <= 1e-12, (name, err)


def test_fem3dface_n_matches_reference(lib, golden):
    """anigpu_fem3dface_n (FP64) against the reference's fem3DfaceN: within 1e-12 per tet."""
    XY = golden["tets_XY"]
    for name in golden["facen_case_names"]:
        name = str(name)
        ca, cb = (int(v) for v in name.split("_")[:2])
        kname, order, face = name.split("_")[2], int(name.split("_")[3][1:]), int(name.split("_")[4][1:])
        D = golden[f"facen_{name}_D"] if f"facen_{name}_D" in golden.files else None
        A = lib.fem3dface(ca, cb, XY, face, D, KIND_CODE[kname], order, normal=True)
        err = rel_err_per_tet(A.cpu().numpy(), golden[f"facen_{name}_A"])
        assert err <= 1e-12, (name, err)


def test_runtime_space_layer_on_gpu(lib, golden, tmp_path):
    """fem3Dtet / fem3Dface through the C++ runtime-space layer equal the same calls through the
    C ABI, and an invalid face comes back as std::runtime_error."""
    import subprocess

    import anigpu
    from helpers import build_runtime_space_test
    exe = build_runtime_space_test(str(tmp_path))
    XY = np.ascontiguousarray(golden["tets_XY"], dtype=np.float64)
    nt = XY.shape[0]
    XY.tofile(tmp_path / "xy.bin")
    r = subprocess.run([exe, "gpu", str(tmp_path / "xy.bin"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    A = lib.fem3dtet(22, 22, XY, None, anigpu.TENSOR_NULL, 4).cpu().numpy().reshape(-1)
    F = lib.fem3dface(1, 21, XY, 1, None, anigpu.TENSOR_NULL, 4).cpu().numpy().reshape(-1)
    assert np.array_equal(out[:nt * 100], A) and np.array_equal(out[nt * 100:nt * 110], F)
    # the ApplyOpCustom operator (GRAD P2 values from fem3DapplyL) integrates to fem3Dtet's matrix
    C = out[nt * 110:]
    assert rel_err_per_tet(C.reshape(nt, 100), A.reshape(nt, 100)) <= 1e-13


@pytest.mark.parametrize("ca,cb,kind", [(22, 22, "tsym"), (12, 22, "tgeneral"), (21, 11, "point0"), (94, 94, "null")])
def test_custom_operators_match_builtin(lib, golden, ca, cb, kind):
    """anigpu_fem3dtet_custom (ApplyOpCustom) with the operators' values taken from fem3DapplyL on
    unit DOF vectors gives the built-in fem3Dtet matrices (FP64 within 1e-13 per tet, FP32 within
    2e-5): the user-operator path integrates exactly what it is given."""
    import anigpu
    XY = golden["tets_XY"]
    nt = XY.shape[0]
    order = 4
    pts = anigpu.quadrature(order)[0]

    def values(code):
        nf, dim = op_info(code)
        cols = []
        for i in range(nf):
            e = np.zeros((nt, nf))
            e[:, i] = 1.0
            cols.append(lib.fem3d_apply(code, XY, pts, e))
        import torch
        return torch.stack(cols, dim=2)  # [nt, q, nf, dim]

    UA = values(ca)
    VB = None if cb == ca else values(cb)
    nfA, dA = op_info(ca)
    nfB, dB = op_info(cb)
    if kind.startswith("point"):
        q = lib.quadrature_points(order, XY).cpu().numpy()
        D, code = point_tensor(int(kind[5:]), q, dB, dA), anigpu.TENSOR_POINT
    elif kind == "tsym":
        D, code = np.tile([2.0, 0.3, -0.1, 1.5, 0.2, 1.1], (nt, 1)), anigpu.TENSOR_TET_SYM
    elif kind == "tgeneral":
        D, code = np.random.default_rng(5).normal(size=(nt, dB * dA)), anigpu.TENSOR_TET_GENERAL
    else:
        D, code = None, anigpu.TENSOR_NULL
    ref = lib.fem3dtet(ca, cb, XY, D, code, order).cpu().numpy()
    got = lib.fem3dtet_custom(UA, XY, VB, D, code, order).cpu().numpy()
    assert rel_err_per_tet(got, ref) <= 1e-13
    got32 = lib.fem3dtet_custom(UA, XY, VB, D, code, order, anigpu.F32).double().cpu().numpy()
    assert rel_err_per_tet(got32, ref) <= 2e-5
