"""GPU parity of the global path: DOF numbering, CSR template (bit-exact), row-gather
assembly with Dirichlet elimination, drop-rule pattern, and the Krylov solves, against the
restated oracle on the same seeded inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(lib, restated, n, space, perturb, kind, order, dirichlet=True, seed=1, f=None, bc_value=None):
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=perturb, seed=seed)
    nt = tets.shape[0]
    D = None
    if kind == anigpu.TENSOR_TET_SYM:
        D = meshgen.aniso_tensors(nt, 1.5, seed + 10)
    elif kind == anigpu.TENSOR_TET_SCALAR:
        D = np.exp(meshgen.normal(seed + 20, nt))
    elif kind == anigpu.TENSOR_CONST_SCALAR:
        D = np.array([1.7])
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(space)
    coords = lib.dof_coords().cpu().numpy()
    mask = meshgen.boundary_mask(coords) if dirichlet else np.zeros(ndof, np.uint8)
    bc = None
    if bc_value is not None:
        bc = np.where(mask == 1, bc_value(coords), 0.0)
    lib.set_dirichlet(mask if dirichlet else None, bc)
    ref = restated.assemble_problem(xyz, tets, space, kind, D, 1.0, order,
                                    dirichlet=(mask, bc) if dirichlet else None, f=f)
    return dict(xyz=xyz, tets=tets, D=D, mask=mask, ref=ref, ndof=ndof, nnz=nnz, bc=bc)


@pytest.mark.parametrize("space,n,perturb", [(1, 4, 0.0), (1, 5, 0.2), (2, 3, 0.0), (2, 4, 0.2)])
def test_numbering_and_template_bit_exact(lib, restated, space, n, perturb):
    import anigpu
    P = _problem(lib, restated, n, space, perturb, anigpu.TENSOR_NULL, 2)
    ref = P["ref"]
    assert P["ndof"] == ref["ndof"]
    ed = lib.element_dofs().cpu().numpy()
    assert np.array_equal(ed, ref["edofs"])
    rp, col = lib.csr_template()
    assert np.array_equal(rp.cpu().numpy(), ref["rowptr"])
    assert np.array_equal(col.cpu().numpy(), ref["col"])


@pytest.mark.parametrize("space,kind,order", [(1, 0, 2), (1, 2, 2), (2, 3, 4), (2, 1, 4), (2, 3, 2), (2, 0, 5),
                                              (2, 3, 1), (1, 3, 0)])
def test_assembly_f64_matches_oracle(lib, restated, space, kind, order):
    import anigpu
    P = _problem(lib, restated, 4, space, 0.2, kind, order)
    vals, rhs, touched = lib.assemble(kind, P["D"], None, 1.0, order, anigpu.F64, touched=True)
    ref = P["ref"]
    v = vals.cpu().numpy()
    scale = np.abs(ref["vals"]).max()
    assert np.abs(v - ref["vals"]).max() <= 1e-12 * scale
    assert np.abs(rhs.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * max(np.abs(ref["rhs"]).max(), 1e-300)
    assert np.array_equal(touched.cpu().numpy(), ref["touched"])


def test_assembly_f32_error(lib, restated):
    import anigpu
    P = _problem(lib, restated, 5, 2, 0.2, anigpu.TENSOR_TET_SYM, 4)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32)
    ref = P["ref"]
    rp = ref["rowptr"]
    v = vals.double().cpu().numpy()
    # per-row relative error against the FP64 oracle
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    rown = np.sqrt(np.bincount(rows, ref["vals"] ** 2))
    err = np.sqrt(np.bincount(rows, (v - ref["vals"]) ** 2)) / np.maximum(rown, 1e-300)
    print("FP32 assembly: max/median per-row relative error", err.max(), np.median(err))
    assert err.max() <= 5e-5


def test_assembly_nonhomogeneous_dirichlet(lib, restated):
    import anigpu
    P = _problem(lib, restated, 4, 2, 0.15, anigpu.TENSOR_TET_SCALAR, 4,
                 bc_value=lambda c: 1.0 + c[:, 0] - 2 * c[:, 2])
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SCALAR, P["D"], None, 1.0, 4, anigpu.F64)
    ref = P["ref"]
    assert np.abs(vals.cpu().numpy() - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
    assert np.abs(rhs.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()


def test_per_tet_source(lib, restated):
    import anigpu
    from anigpu import meshgen
    f = meshgen.normal(99, 6 * 4 ** 3)
    P = _problem(lib, restated, 4, 1, 0.1, anigpu.TENSOR_NULL, 2, f=f)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_NULL, None, f, 0.0, 2, anigpu.F64)
    assert np.abs(rhs.cpu().numpy() - P["ref"]["rhs"]).max() <= 1e-12 * np.abs(P["ref"]["rhs"]).max()


@pytest.mark.parametrize("space", [1, 2])
def test_drop_rule_pattern(lib, restated, space):
    """The assembler without a template keeps only |a| > drop entries plus the diagonal
    (assembler.inl:114-135,416-418); Dirichlet rows/columns create exact zeros.  A perturbed
    mesh is used: on the unperturbed Kuhn mesh some entries are zero only mathematically,
    and the contracted formulation leaves them at rounding level (|a| ~ 1e-17 |A|)."""
    import anigpu
    P = _problem(lib, restated, 5, space, 0.2, anigpu.TENSOR_NULL, 2)
    vals, rhs, touched = lib.assemble(anigpu.TENSOR_NULL, None, None, 1.0, 2, anigpu.F64, touched=True)
    rp, col = lib.csr_template()
    nnz = lib.csr_compact(rp, col, vals, anigpu.F64, touched)
    ref = P["ref"]
    rp_o, col_o, v_o = restated.csr_compact(ref["rowptr"], ref["col"], ref["vals"], ref["touched"])
    assert nnz == col_o.size < P["nnz"]
    assert np.array_equal(rp.cpu().numpy(), rp_o)
    assert np.array_equal(col[:nnz].cpu().numpy(), col_o)
    assert np.abs(vals[:nnz].cpu().numpy() - v_o).max() <= 1e-12 * np.abs(v_o).max()


def test_assembly_is_deterministic(lib, restated):
    import anigpu
    P = _problem(lib, restated, 6, 2, 0.2, anigpu.TENSOR_TET_SYM, 4, dirichlet=True)
    a1, r1, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32)
    a2, r2, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32)
    assert bool((a1 == a2).all()) and bool((r1 == r2).all())


def test_nonfinite_tensor_reports_status(lib, restated):
    import anigpu
    P = _problem(lib, restated, 3, 2, 0.0, anigpu.TENSOR_TET_SCALAR, 4, dirichlet=False)
    D = P["D"].copy()
    D[5] = np.nan  # injected on the host
    with pytest.raises(anigpu.AnigpuError) as e:
        lib.assemble(anigpu.TENSOR_TET_SCALAR, D, None, 1.0, 4, anigpu.F64)
    assert e.value.code == anigpu.ERR_NONFINITE
    # the handle stays usable
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SCALAR, P["D"], None, 1.0, 4, anigpu.F64)
    assert np.isfinite(vals.cpu().numpy()).all()


def test_config1_end_to_end(lib, restated):
    """Config 1: P1 Poisson on 16^3 x 6 Kuhn tets, identity tensor, order 2, f = 1,
    homogeneous Dirichlet, Jacobi-PCG to 1e-10."""
    import anigpu
    P = _problem(lib, restated, 16, 1, 0.0, anigpu.TENSOR_NULL, 2)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_NULL, None, None, 1.0, 2, anigpu.F64)
    ref = P["ref"]
    assert np.abs(vals.cpu().numpy() - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
    x, st = lib.solve(vals, rhs, anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-10, maxit=20000)
    xh = x.cpu().numpy()
    tr = restated.true_residual(ref["rowptr"], ref["col"], ref["vals"], xh, ref["rhs"])
    assert tr <= 1e-10 and st.rel_residual <= 1e-10
    xo, it_o, rel_o = restated.jacobi_pcg(ref["rowptr"], ref["col"], ref["vals"], ref["rhs"], 1e-10, 20000)
    assert abs(st.iterations - it_o) <= 2
    assert np.abs(xh - xo).max() <= 1e-8 * np.abs(xo).max()


def test_ir_cg32_reaches_fp64_tolerance(lib, restated):
    import anigpu
    P = _problem(lib, restated, 8, 2, 0.2, anigpu.TENSOR_TET_SYM, 4)
    vals32, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32)
    x, st = lib.solve(vals32, rhs, anigpu.SOLVE_IR_CG32, anigpu.F32, rtol=1e-8, maxit=200000)
    assert st.rel_residual <= 1e-8 and st.outer_iterations >= 1
    ref = P["ref"]
    # FP64 true residual against the FP32-assembled matrix (the system that is solved)
    v32 = vals32.double().cpu().numpy()
    r32 = rhs.cpu().numpy()  # the FP32 path accumulates its right-hand side in FP32 too
    assert restated.true_residual(ref["rowptr"], ref["col"], v32, x.cpu().numpy(), r32) <= 1e-8
    # and against the FP64 oracle matrix: bounded by the FP32 assembly error
    tr64 = restated.true_residual(ref["rowptr"], ref["col"], ref["vals"], x.cpu().numpy(), ref["rhs"])
    print("IR-CG32 residual vs FP64 oracle matrix:", tr64)
    assert tr64 <= 1e-4


def test_spmv_matches_oracle(lib, restated):
    import anigpu
    P = _problem(lib, restated, 5, 2, 0.2, anigpu.TENSOR_TET_SYM, 4)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F64)
    xx = np.sin(np.arange(P["ndof"]) * 0.37)
    y = lib.spmv(vals, xx).cpu().numpy()
    ref = P["ref"]
    yo = restated.spmv(ref["rowptr"], ref["col"], ref["vals"], xx)
    assert np.abs(y - yo).max() <= 1e-12 * np.abs(yo).max()


def test_async_assembly_and_status(lib, restated):
    """anigpu_assemble_async enqueues without waiting; anigpu_status reports (and clears) a
    non-finite value met by any assembly since the last check."""
    import anigpu
    P = _problem(lib, restated, 4, 2, 0.2, anigpu.TENSOR_TET_SYM, 4)
    v_sync, r_sync, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32)
    v_async, r_async, _ = lib.assemble(anigpu.TENSOR_TET_SYM, P["D"], None, 1.0, 4, anigpu.F32, sync=False)
    lib.status()
    assert bool((v_sync == v_async).all()) and bool((r_sync == r_async).all())
    D = P["D"].copy()
    D[3, 0] = np.inf  # injected on the host
    lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, anigpu.F32, sync=False)  # returns at once
    with pytest.raises(anigpu.AnigpuError) as e:
        lib.status()
    assert e.value.code == anigpu.ERR_NONFINITE
    lib.status()  # cleared


def _lame9(lam, mu):
    """The Lame tensor as the 9x9 GENERAL tensor of Operator<GRAD, FemVec<3,P2>>: index j + 3 c for
    derivative j of component c (lin_elast.cpp:100-118); symmetric, so its column-major layout is
    the same as its row-major one."""
    D = np.zeros((lam.size, 9, 9))
    for c1 in range(3):
        for j1 in range(3):
            for c2 in range(3):
                for j2 in range(3):
                    D[:, j1 + 3 * c1, j2 + 3 * c2] = (lam * (j1 == c1) * (j2 == c2)
                                                      + mu * ((c1 == c2) * (j1 == j2) + (c1 == j2) * (j1 == c2)))
    return D.reshape(lam.size, 81)


@pytest.mark.parametrize("n,clamped,bcnz", [(3, False, False), (4, True, False), (4, True, True), (3, False, True)])
def test_vector_p2_lame_matches_oracle(lib, restated, n, clamped, bcnz):
    """Vector P2 linear elasticity (config 5 operator): FP64 assembly with per-tet Lame parameters
    equals the restated assembler with the 9x9 GENERAL tensor; FP32 within 5e-5 per row; with
    non-zero boundary displacements (different per component) the right-hand side too."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=0.2, seed=5)
    nt = tets.shape[0]
    E = np.exp(0.5 * meshgen.normal(61, nt))
    nu = 0.2 + 0.25 * meshgen.uniform(62, nt)
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(anigpu.VEC3_P2)
    coords = lib.dof_coords().cpu().numpy()
    mask = (np.abs(coords[:, 0]) < 1e-12).astype(np.uint8) if clamped else meshgen.boundary_mask(coords)
    bc = None
    if bcnz:
        comp = np.repeat(np.arange(3), ndof // 3)
        bc = (0.1 * coords[:, 1] - 0.05 * coords[:, 2] + 0.02 * (comp + 1)) * mask
    lib.set_dirichlet(mask, bc)
    LM = np.stack([lam, mu], axis=1)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.5, 4, anigpu.F64)
    ref = restated.assemble_problem(xyz, tets, 5, 4, _lame9(lam, mu), 0.5, 4, dirichlet=(mask, bc))
    rp, col = lib.csr_template()
    assert np.array_equal(rp.cpu().numpy(), ref["rowptr"]) and np.array_equal(col.cpu().numpy(), ref["col"])
    v = vals.cpu().numpy()
    assert np.abs(v - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
    assert np.abs(rhs.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * max(np.abs(ref["rhs"]).max(), 1e-300)
    v32, _, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.5, 4, anigpu.F32)
    rows = np.repeat(np.arange(ndof), np.diff(ref["rowptr"]))
    rown = np.sqrt(np.bincount(rows, ref["vals"] ** 2))
    err = np.sqrt(np.bincount(rows, (v32.double().cpu().numpy() - ref["vals"]) ** 2)) / np.maximum(rown, 1e-300)
    assert err.max() <= 5e-5


def test_vector_p2_solves_match_oracle(lib, restated):
    """Vector P2 elasticity solves (block SpMV of the 3-component template): FP64 Jacobi-PCG
    against the oracle's Jacobi-PCG on the same system (iterations within 2, solution), and
    IR-CG32 to an FP64 true residual of 1e-8 on its FP32 matrix."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(5, perturb=0.2, seed=5)
    nt = tets.shape[0]
    E = np.exp(0.5 * meshgen.normal(81, nt))
    nu = 0.2 + 0.25 * meshgen.uniform(82, nt)
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    lib.mesh_upload(xyz, tets)
    ndof, _ = lib.problem_setup(anigpu.VEC3_P2)
    coords = lib.dof_coords().cpu().numpy()
    mask = (np.abs(coords[:, 0]) < 1e-12).astype(np.uint8)
    lib.set_dirichlet(mask)
    LM = np.stack([lam, mu], axis=1)
    vals, _, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.0, 4, anigpu.F64)
    rp, col = lib.csr_template()
    rp, col, v = rp.cpu().numpy(), col.cpu().numpy(), vals.cpu().numpy()
    b = meshgen.normal(83, ndof) * (1 - mask)
    x, st = lib.solve(vals, b, anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-10, maxit=100000)
    xh = x.cpu().numpy()
    assert st.rel_residual <= 1e-10
    assert restated.true_residual(rp, col, v, xh, b) <= 1e-10
    xo, it_o, _ = restated.jacobi_pcg(rp, col, v, b, 1e-10, 100000)
    assert abs(st.iterations - it_o) <= max(2, 0.02 * it_o)  # summation order differs from the CSR walk
    assert np.abs(xh - xo).max() <= 1e-7 * np.abs(xo).max()
    # the product itself against the oracle SpMV
    y = lib.spmv(vals, xh, anigpu.F64).cpu().numpy()
    assert np.abs(y - restated.spmv(rp, col, v, xh)).max() <= 1e-12 * np.abs(y).max()
    v32, _, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.0, 4, anigpu.F32)
    x32, st32 = lib.solve(v32, b, anigpu.SOLVE_IR_CG32, anigpu.F32, rtol=1e-8, maxit=200000)
    assert st32.rel_residual <= 1e-8
    assert restated.true_residual(rp, col, v32.double().cpu().numpy(), x32.cpu().numpy(), b) <= 1e-8


@pytest.mark.parametrize("space", [1, 2, 5])
def test_enumerations_match_oracle(lib, restated, space):
    """Every GlobEnumeration type: the GPU's permutation, renumbered template and renumbered
    values / right-hand side equal the oracle's lexicographic ordering applied to the NATURAL
    system (bit for bit); a vector comes back to NATURAL."""
    import anigpu
    from anigpu import meshgen
    from oracle.oracle import enumeration_perm, permute_csr
    xyz, tets = meshgen.kuhn_cube(3, perturb=0.2, seed=4)
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(space)
    ncomp = 3 if space == 5 else 1
    lib.set_dirichlet(meshgen.boundary_mask(lib.dof_coords().cpu().numpy()))
    if space == 5:
        nt = tets.shape[0]
        LM = np.stack([np.full(nt, 1.5), np.full(nt, 1.0)], axis=1)
        vals, rhs, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.5, 4, anigpu.F64)
    else:
        vals, rhs, _ = lib.assemble(anigpu.TENSOR_NULL, None, None, 1.0, 4, anigpu.F64)
    rp, col = lib.csr_template()
    rp, col, v, b = rp.cpu().numpy(), col.cpu().numpy(), vals.cpu().numpy(), rhs.cpu().numpy()
    nv = xyz.shape[0]
    for etype in range(6):
        perm = enumeration_perm(nv, ndof // ncomp, ncomp, etype)
        rp_o, col_o, v_o = permute_csr(rp, col, v, perm)
        grp, gcol, gperm = lib.enumeration_setup(etype)
        assert np.array_equal(gperm.cpu().numpy(), perm), etype
        assert np.array_equal(grp.cpu().numpy(), rp_o) and np.array_equal(gcol.cpu().numpy(), col_o), etype
        gv, gb = lib.enumeration_apply(vals, anigpu.F64, rhs)
        assert np.array_equal(gv.cpu().numpy(), v_o), etype
        b_o = np.empty_like(b)
        b_o[perm] = b
        assert np.array_equal(gb.cpu().numpy(), b_o), etype
        assert np.array_equal(lib.enumeration_to_natural(gb).cpu().numpy(), b), etype


@pytest.mark.parametrize("space,bcnz", [(1, False), (2, False), (2, True)])
def test_assembly_from_element_matrices_fast_template(lib, restated, space, bcnz):
    """The local-assembler contract on the P1 / P2 template: element matrices computed by the caller
    (GRAD.GRAD with per-tet SYM tensors from fem3Dtet on the library's oriented tets, plus the
    P0 x P_k right-hand side) scatter to the same system as anigpu_assemble, Dirichlet rows and
    columns (zero or non-zero boundary values) included; a reaction term added to the element
    matrices shows up as the assembled mass matrix."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(4, perturb=0.2, seed=21)
    nt = tets.shape[0]
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    c = lib.dof_coords().cpu().numpy()
    mask = meshgen.boundary_mask(c)
    bc = (0.5 + c[:, 0] - c[:, 2]) * mask if bcnz else None
    lib.set_dirichlet(mask, bc)
    D6 = meshgen.aniso_tensors(nt, 1.0, 22)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D6, None, 1.5, 4, anigpu.F64)
    XY = lib.element_coords()
    g = 10 * space + 2
    A = lib.fem3dtet(g, g, XY, D6, anigpu.TENSOR_TET_SYM, 4)
    F = lib.fem3dtet(1, 10 * space + 1, XY, np.array([1.5]), anigpu.TENSOR_CONST_SCALAR, 4).reshape(nt, -1)
    v, r = lib.assemble_elements(A, F)
    ref_v, ref_r = vals.cpu().numpy(), rhs.cpu().numpy()
    assert np.abs(v.cpu().numpy() - ref_v).max() <= 1e-12 * np.abs(ref_v).max()
    assert np.abs(r.cpu().numpy() - ref_r).max() <= 1e-12 * np.abs(ref_r).max()
    # reaction term: K + M from the element matrices equals K plus the scattered mass matrices
    M = lib.fem3dtet(10 * space + 1, 10 * space + 1, XY, None, anigpu.TENSOR_NULL, 4)
    vkm, _ = lib.assemble_elements(A + M, F)
    vm, _ = lib.assemble_elements(M, None)
    rp = lib.csr_template()[0].cpu().numpy()
    on_dir = mask.astype(bool)[np.repeat(np.arange(rp.size - 1), np.diff(rp))]
    exp = v.cpu().numpy() + vm.cpu().numpy()
    exp[on_dir] = v.cpu().numpy()[on_dir]
    assert np.abs(vkm.cpu().numpy() - exp).max() <= 1e-13 * np.abs(exp).max()


@pytest.mark.parametrize("bcnz", [False, True])
def test_vector_p2_from_element_matrices(lib, bcnz):
    """The reference's own elasticity form, fem3Dtet<GRAD P2^3, GRAD P2^3> with the 9x9 GENERAL Lame
    tensor per tet (lin_elast.cpp:100-118), computed by the caller on the library's oriented tets
    and scattered into the vector template, equals the fast Lame assembly (FP64, 1e-12), right-hand
    side and per-component Dirichlet values included."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(3, perturb=0.2, seed=23)
    nt = tets.shape[0]
    E = np.exp(0.5 * meshgen.normal(63, nt))
    nu = 0.2 + 0.25 * meshgen.uniform(64, nt)
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(anigpu.VEC3_P2)
    coords = lib.dof_coords().cpu().numpy()
    mask = (np.abs(coords[:, 0]) < 1e-12).astype(np.uint8)
    bc = None
    if bcnz:
        comp = np.repeat(np.arange(3), ndof // 3)
        bc = (0.1 * coords[:, 1] - 0.05 * coords[:, 2] + 0.02 * (comp + 1)) * mask
    lib.set_dirichlet(mask, bc)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_LAME, np.stack([lam, mu], axis=1), None, 0.5, 4, anigpu.F64)
    XY = lib.element_coords()
    A = lib.fem3dtet(52, 52, XY, _lame9(lam, mu), anigpu.TENSOR_TET_GENERAL, 4)
    F = lib.fem3dtet(1, 51, XY, np.array([0.5]), anigpu.TENSOR_CONST_SCALAR, 4).reshape(nt, -1)
    v, r = lib.assemble_elements(A, F)
    ref_v, ref_r = vals.cpu().numpy(), rhs.cpu().numpy()
    assert np.abs(v.cpu().numpy() - ref_v).max() <= 1e-12 * np.abs(ref_v).max()
    assert np.abs(r.cpu().numpy() - ref_r).max() <= 1e-12 * np.abs(ref_r).max()
