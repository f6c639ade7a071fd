"""GPU parity of the ring-order gather of P2 edge rows (the tets around each edge walked face to
face, each value written once) against the restated assembler, against the record gather on the
same inputs, and its fallback on a mesh whose edges do not all have rings."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(lib, n, perturb, seed, dirichlet=True):
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=perturb, seed=seed)
    D = meshgen.aniso_tensors(tets.shape[0], 1.5, seed + 10)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.P2)
    mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy()) if dirichlet else None
    lib.set_dirichlet(mask)
    return xyz, tets, D, mask


@pytest.mark.parametrize("dirichlet,order", [(True, 4), (False, 2), (True, 6)])
def test_ring_gather_f64_matches_oracle(lib, restated, dirichlet, order):
    import anigpu
    xyz, tets, D, mask = _setup(lib, 5, 0.2, 3, dirichlet)
    assert lib.gather_layouts() == (True, True)
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, order, anigpu.F64)
    ref = restated.assemble_problem(xyz, tets, 2, anigpu.TENSOR_TET_SYM, D, 1.0, order,
                                    dirichlet=(mask, None) if dirichlet else None)
    scale = np.abs(ref["vals"]).max()
    assert np.abs(vals.cpu().numpy() - ref["vals"]).max() <= 1e-12 * scale
    assert np.abs(rhs.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()


@pytest.mark.parametrize("precision", ["F64", "F32"])
def test_ring_gather_matches_record_gather(lib, precision):
    """Same inputs through both gathers: the values agree to rounding (FP64 4e-15, FP32 1e-6 of
    the largest value), the right-hand sides likewise, and the ring gather is deterministic."""
    import anigpu
    prec = getattr(anigpu, precision)
    _, _, D, _ = _setup(lib, 6, 0.25, 5)
    lib.set_gather_layouts(True)
    v1, r1, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, prec)
    v1, r1 = v1.clone(), r1.clone()
    v1b, _, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, prec)
    assert bool((v1b == v1).all())
    lib.set_gather_layouts(False)
    try:
        v0, r0, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, prec)
    finally:
        lib.set_gather_layouts(True)
    tol = 4e-15 if precision == "F64" else 1e-6
    a, b = v1.double().cpu().numpy(), v0.double().cpu().numpy()
    assert np.abs(a - b).max() <= tol * np.abs(b).max()
    assert np.abs(r1.cpu().numpy() - r0.cpu().numpy()).max() <= tol * np.abs(r0.cpu().numpy()).max()
    # the zero pattern (Dirichlet columns, opposite-edge entries) is the same
    assert np.array_equal(a == 0, b == 0)


def test_ring_fallback_on_nonmanifold_edge(lib, restated):
    """Two tets that share only the edge (0, 1): that edge has no ring, the mesh keeps the record
    gather, and the assembly still matches the oracle."""
    import anigpu
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0.3, -1, 0.1], [0.2, 0.1, -1]], np.float64)
    tets = np.array([[0, 1, 2, 3], [0, 1, 4, 5]], np.int32)
    D = np.tile(np.array([2.0, 1.0, 1.5, 0.1, 0.0, 0.2]), (2, 1))
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.P2)
    lib.set_dirichlet(None)
    assert lib.gather_layouts()[0] is False
    vals, rhs, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, anigpu.F64)
    ref = restated.assemble_problem(xyz, tets, 2, anigpu.TENSOR_TET_SYM, D, 1.0, 4, dirichlet=None)
    assert np.abs(vals.cpu().numpy() - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()


@pytest.mark.parametrize("space,kind", [(1, 2), (1, 3), (2, 2)])
def test_interleaved_vertex_rows_match_oracle(lib, restated, space, kind):
    """Vertex rows from the lane-interleaved records (P1: every row) against the oracle, with
    Dirichlet rows and columns, FP64."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(5, perturb=0.2, seed=11)
    nt = tets.shape[0]
    D = meshgen.aniso_tensors(nt, 1.5, 21) if kind == anigpu.TENSOR_TET_SYM else np.exp(meshgen.normal(22, nt))
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy())
    lib.set_dirichlet(mask)
    assert lib.gather_layouts()[1]
    vals, rhs, _ = lib.assemble(kind, D, None, 1.0, 2, anigpu.F64)
    ref = restated.assemble_problem(xyz, tets, space, kind, D, 1.0, 2, dirichlet=(mask, None))
    assert np.abs(vals.cpu().numpy() - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
    assert np.abs(rhs.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()


@pytest.mark.parametrize("precision", ["F64", "F32"])
def test_vector_ring_gather_matches_record_gather(lib, restated, precision):
    """Vector P2 (Lame) edge rows in ring order against the record gather on the same inputs, with
    clamped and non-zero Dirichlet values, and the FP64 result against the oracle."""
    import anigpu
    from anigpu import meshgen
    prec = getattr(anigpu, precision)
    xyz, tets = meshgen.kuhn_cube(4, perturb=0.2, seed=13)
    nt = tets.shape[0]
    LM = np.stack([1.0 + meshgen.uniform(31, nt), 0.5 + meshgen.uniform(32, nt)], axis=1)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.VEC3_P2)
    coords = lib.dof_coords().cpu().numpy()
    mask = (np.abs(coords[:, 0]) < 1e-12).astype(np.uint8)
    bc = np.where(mask == 1, 0.1 * coords[:, 1], 0.0)
    lib.set_dirichlet(mask, bc)
    assert lib.gather_layouts() == (True, True)
    v1, r1, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.5, 4, prec)
    v1, r1 = v1.clone(), r1.clone()
    lib.set_gather_layouts(False)
    try:
        v0, r0, _ = lib.assemble(anigpu.TENSOR_LAME, LM, None, 0.5, 4, prec)
    finally:
        lib.set_gather_layouts(True)
    tol = 4e-15 if precision == "F64" else 1e-6
    a, b = v1.double().cpu().numpy(), v0.double().cpu().numpy()
    assert np.abs(a - b).max() <= tol * np.abs(b).max()
    assert np.abs(r1.cpu().numpy() - r0.cpu().numpy()).max() <= tol * np.abs(r0.cpu().numpy()).max()
    if precision == "F64":
        ref = restated.assemble_problem(xyz, tets, 5, 4, meshgen.lame9(LM[:, 0], LM[:, 1]), 0.5, 4,
                                        dirichlet=(mask, bc))
        assert np.abs(a - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
        assert np.abs(r1.cpu().numpy() - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()


def _star_mesh():
    """A vertex at the origin and the 80 tets that join it to a once-subdivided icosahedron: the
    centre's row has 80 incidences, every other vertex row 5 or 6, so the vertex rows' interleaved
    layout keeps per-warp offsets (a uniform stride would double it)."""
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    pts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    mid = {}

    def midpoint(a, b):
        key = (min(a, b), max(a, b))
        if key not in mid:
            m = pts[a] + pts[b]
            pts.append(m / np.linalg.norm(m))
            mid[key] = len(pts) - 1
        return mid[key]

    faces = []
    for a, b, c in f:
        ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
        faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    xyz = np.vstack([np.zeros((1, 3))] + [p[None] for p in pts])
    tets = np.array([(0, a + 1, b + 1, c + 1) for a, b, c in faces], np.int32)
    return xyz, tets


@pytest.mark.parametrize("precision", ["F64", "F32"])
def test_gathers_with_per_warp_offsets(lib, restated, precision):
    """The star mesh (one vertex row of 80 incidences among rows of 5-6): both gathers against the
    record gather, FP64 against the oracle, with the walks' first records read past short rows."""
    import anigpu
    prec = getattr(anigpu, precision)
    xyz, tets = _star_mesh()
    assert tets.shape[0] == 80 and xyz.shape[0] == 43
    D = np.tile(np.array([2.0, 1.0, 1.5, 0.1, 0.0, 0.2]), (tets.shape[0], 1))
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.P2)
    mask = (np.linalg.norm(lib.dof_coords().cpu().numpy(), axis=1) > 0.99).astype(np.uint8)
    lib.set_dirichlet(mask)
    assert lib.gather_layouts() == (True, True)
    v1, r1, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, prec)
    v1, r1 = v1.double().cpu().numpy(), r1.cpu().numpy()
    lib.set_gather_layouts(False)
    try:
        v0, r0, _ = lib.assemble(anigpu.TENSOR_TET_SYM, D, None, 1.0, 4, prec)
    finally:
        lib.set_gather_layouts(True)
    v0, r0 = v0.double().cpu().numpy(), r0.cpu().numpy()
    tol = 4e-15 if precision == "F64" else 1e-6
    assert np.abs(v1 - v0).max() <= tol * np.abs(v0).max()
    assert np.abs(r1 - r0).max() <= tol * np.abs(r0).max()
    if precision == "F64":
        ref = restated.assemble_problem(xyz, tets, 2, anigpu.TENSOR_TET_SYM, D, 1.0, 4, dirichlet=(mask, None))
        assert np.abs(v1 - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
        assert np.abs(r1 - ref["rhs"]).max() <= 1e-12 * np.abs(ref["rhs"]).max()
