"""GPU tests of the batched uneven instances (one graph launch assembles and solves every instance):
every instance's CSR block and solution against the oracle's restated assembler and Jacobi-PCG on
that instance alone, and P1 and P2 instance sets run together as one graph launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TET_SCALAR = 2


def _instances(ns, seed):
    from anigpu import meshgen
    meshes = [meshgen.kuhn_cube(n, perturb=0.15, seed=seed + i) for i, n in enumerate(ns)]
    coefs = [np.exp(meshgen.normal(seed + 100 + i, m[1].shape[0])) for i, m in enumerate(meshes)]
    return meshes, coefs


def _setup(lib, space, ns, seed, order):
    import anigpu
    from anigpu import meshgen
    meshes, coefs = _instances(ns, seed)
    xyz, tets, toff = meshgen.union(meshes)
    coef = np.concatenate(coefs)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy())
    lib.set_dirichlet(mask)
    vals0, _, _ = lib.assemble(anigpu.TENSOR_TET_SCALAR, coef, None, 1.0, order, anigpu.F64)
    vals0 = vals0.clone()
    lib.batch_set_instances(toff, vals0)
    b = meshgen.normal(7 + space, lib.ndof) * (1 - mask)
    return dict(meshes=meshes, coefs=coefs, xyz=xyz, coef=coef, mask=mask, b=b, vals0=vals0)


def _check_against_oracle(lib, restated, space, order, S, x, vals, st, rtol):
    """Each instance: its rows and columns of the batched CSR equal the oracle's template of the
    instance, its values the oracle's to 1e-12, its solution the oracle's Jacobi-PCG solution."""
    rp, col = lib.csr_template()
    rp, col = rp.cpu().numpy(), col.cpu().numpy()
    v, xb = vals.cpu().numpy(), x.cpu().numpy()
    nv_tot = S["xyz"].shape[0]
    voff = np.concatenate([[0], np.cumsum([m[0].shape[0] for m in S["meshes"]])])
    eoff = 0
    for i, (m, c) in enumerate(zip(S["meshes"], S["coefs"])):
        nvi = m[0].shape[0]
        ne = restated.edges(nvi, restated.orient(m[0], m[1]))[0] if space == 2 else 0
        idx = np.concatenate([voff[i] + np.arange(nvi), nv_tot + eoff + np.arange(ne)]).astype(np.int64)
        eoff += ne
        # the oracle's system of the instance alone, with the instance's Dirichlet DOFs of the batch
        ref = restated.assemble_problem(m[0], m[1], space, TET_SCALAR, c, 1.0, order,
                                        dirichlet=(S["mask"][idx], None))
        inv = -np.ones(rp.size - 1, dtype=np.int64)
        inv[idx] = np.arange(idx.size)
        lens = rp[idx + 1] - rp[idx]
        assert np.array_equal(lens, np.diff(ref["rowptr"])), i
        sel = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in idx])
        assert np.array_equal(inv[col[sel]], ref["col"].astype(np.int64)), i
        assert np.abs(v[sel] - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max(), i
        xo, it, rel = restated.jacobi_pcg(ref["rowptr"], ref["col"], ref["vals"], S["b"][idx], rtol, 100000)
        assert abs(it - st[i].iterations) <= 2, (i, it, st[i].iterations)
        assert np.abs(xb[idx] - xo).max() <= 1e-7 * max(np.abs(xo).max(), 1e-300), i
        tr = restated.true_residual(ref["rowptr"], ref["col"], ref["vals"], xb[idx], S["b"][idx])
        assert tr <= rtol * 1.0001, (i, tr)


@pytest.mark.parametrize("space,order", [(1, 2), (2, 4)])
def test_batched_instances_match_oracle(lib, restated, space, order):
    import anigpu
    S = _setup(lib, space, [3, 5, 4, 6, 2], 40 + space, order)
    x, vals, st = lib.batch_run(S["b"], anigpu.TENSOR_TET_SCALAR, S["coef"], None, 1.0, order, rtol=1e-10,
                                maxit=20000)
    info = lib.batch_info()
    assert info["lanes_per_row"] in (2, 4, 8, 16) and info["ntiles"] > 0
    warps, ms = lib.batch_assembly_tuning()
    assert warps in (1, 2) and all(t > 0 for t in ms)
    assert bool((vals == S["vals0"]).all())  # the graph's assembly is the plain assembly
    assert all(s.rel_residual <= 1e-10 for s in st)
    _check_against_oracle(lib, restated, space, order, S, x, vals, st, 1e-10)


def test_p1_and_p2_instances_in_one_graph_launch(lib, restated):
    """The P1 instance set and the P2 instance set as two jobs of one graph launch
    (anigpu_batch_run_jobs): the same results as their separate launches, bitwise, and the oracle's."""
    import anigpu
    lib2 = anigpu.Anigpu(0)
    try:
        S1 = _setup(lib, anigpu.P1, [4, 2, 5], 70, 2)
        S2 = _setup(lib2, anigpu.P2, [3, 4, 2], 80, 4)
        jobs = [dict(lib=lib, b=S1["b"], kind=anigpu.TENSOR_TET_SCALAR, D=S1["coef"], order=2),
                dict(lib=lib2, b=S2["b"], kind=anigpu.TENSOR_TET_SCALAR, D=S2["coef"], order=4)]
        (x1, v1, st1), (x2, v2, st2) = anigpu.batch_run_jobs(jobs, rtol=1e-10, maxit=20000)
        assert lib.batch_info()["device_loop"] == lib2.batch_info()["device_loop"]
        y1, w1, s1 = lib.batch_run(S1["b"], anigpu.TENSOR_TET_SCALAR, S1["coef"], None, 1.0, 2, rtol=1e-10,
                                   maxit=20000)
        y2, w2, s2 = lib2.batch_run(S2["b"], anigpu.TENSOR_TET_SCALAR, S2["coef"], None, 1.0, 4, rtol=1e-10,
                                    maxit=20000)
        assert bool((x1 == y1).all()) and bool((x2 == y2).all())
        assert [a.iterations for a in st1] == [a.iterations for a in s1]
        _check_against_oracle(lib, restated, anigpu.P1, 2, S1, x1, v1, st1, 1e-10)
        _check_against_oracle(lib2, restated, anigpu.P2, 4, S2, x2, v2, st2, 1e-10)
    finally:
        lib2.close()
