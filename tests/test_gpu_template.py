"""GPU parity of the drop-in template interface (include/anigpu_fem.hpp): tests/cpp/fem_template.cpp
is spelled as code against AniFem++'s own headers -- fem3Dtet<Operator<...>, Operator<...>,
DfuncTraits<...>> with host tensor functors (per point, constant, PerTetra over a fused batch,
fusive), PlainMemory orders 12 and 20, fem3Dface / fem3DfaceN, the reference's errors, and the
ex1 tutorial's local assembler run through GenerateElemMatRhs + Assembler -- and every result
is compared with the oracle (FP64, 1e-12)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from helpers import point_tensor, rel_err_per_tet

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
POINT, TET_SCALAR, TET_GENERAL, CONST_SCALAR, NULL = 5, 2, 4, 1, 0


def build_fem_template(outdir):
    import anigpu
    libdir = os.path.dirname(anigpu.LIB_PATH)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(outdir, "fem_template")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(REPO, "tests", "cpp", "fem_template.cpp"), "-o", exe, "-L", libdir, "-lanigpu",
           f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def read_blocks(path):
    out = {}
    with open(path, "rb") as fh:
        data = fh.read()
    pos = 0
    while pos < len(data):
        (ln,) = struct.unpack_from("<i", data, pos)
        pos += 4
        name = data[pos:pos + ln].decode()
        pos += ln
        (n,) = struct.unpack_from("<q", data, pos)
        pos += 8
        out[name] = np.frombuffer(data, dtype=np.float64, count=n, offset=pos).copy()
        pos += 8 * n
    return out


@pytest.fixture(scope="module")
def run(tmp_path_factory, lib):
    from anigpu import meshgen
    d = tmp_path_factory.mktemp("fem_template")
    exe = build_fem_template(str(d))
    xyz, tets = meshgen.kuhn_cube(5, perturb=0.2, seed=13)
    XY = meshgen.random_tets(16, seed=17)
    inp, outp = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(inp, "wb") as fh:
        fh.write(struct.pack("<qqq", xyz.shape[0], tets.shape[0], XY.shape[0]))
        fh.write(np.ascontiguousarray(xyz, dtype=np.float64).tobytes())
        fh.write(np.ascontiguousarray(tets, dtype=np.int32).tobytes())
        fh.write(np.ascontiguousarray(XY, dtype=np.float64).tobytes())
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return read_blocks(outp), xyz, tets, XY


def _cmp(got, ref, tol=1e-12):
    got = got.reshape(ref.shape[0], -1)
    err = rel_err_per_tet(got, ref.reshape(ref.shape[0], -1))
    assert err <= tol, err
    return err


def test_element_integrals_match_oracle(run, restated):
    out, _, _, XY = run
    q4 = restated.quad_points(4, XY)
    _cmp(out["p2_aniso_point_o4"], restated.fem3dtet(22, 22, POINT, 4, XY, point_tensor(2, q4, 3, 3)))
    _cmp(out["p1_null_o2"], restated.fem3dtet(12, 12, NULL, 2, XY))
    _cmp(out["rhs_p2_const_o3"], restated.fem3dtet(1, 21, CONST_SCALAR, 3, XY, np.array([2.5])))
    lam, mu = 1.0, 3.0
    C = np.zeros((9, 9))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    C[i + 3 * j, k + 3 * l] = lam * (i == j) * (k == l) + mu * ((i == k) * (j == l) + (i == l) * (j == k))
    Cg = np.tile(C.T.reshape(1, 81), (XY.shape[0], 1))  # column-major 9 x 9 per tet
    _cmp(out["vecp2_lame_o4"], restated.fem3dtet(52, 52, TET_GENERAL, 4, XY, Cg))
    n4 = XY.shape[0] // 4 * 4
    s = 1.5 + np.arange(n4) % 4
    _cmp(out["p2_pertet_fused4_o5"], restated.fem3dtet(22, 22, TET_SCALAR, 5, XY[:n4], s))
    _cmp(out["p2_fusive_o4"], restated.fem3dtet(22, 22, POINT, 4, XY, point_tensor(2, q4, 3, 3)))
    for order in (12, 20):
        qo = restated.quad_points(order, XY)
        _cmp(out[f"p2_aniso_point_o{order}"], restated.fem3dtet(22, 22, POINT, order, XY, point_tensor(2, qo, 3, 3)))
    fq = restated.face_quad_points(5, 2, XY)
    Df = (1 + fq[..., 0] * fq[..., 1])[..., None]
    _cmp(out["face2_p2_load_o5"], restated.fem3dface(1, 21, POINT, 5, 2, XY, Df))
    fq1 = restated.face_quad_points(5, 1, XY)
    Dn = 0.5 * (np.arange(9) + 1)[None, None, :] + np.arange(9)[None, None, :] * fq1[..., 2:3]
    _cmp(out["facen1_vecp2_trac_o5"], restated.fem3dface(1, 51, POINT, 5, 1, XY, Dn, normal=True))
    assert out["errors_caught"][0] == 3


def test_ex1_local_assembler_matches_restated_assembler(run, restated):
    """The ex1 tutorial's local assembler (P1, D = 1 + x^2 per point, f = 1, applyDir on boundary
    nodes) through GenerateElemMatRhs + Assembler equals the restated AssemblerT::Assemble."""
    out, xyz, tets, _ = run
    assert out["ex1_status"][0] == 0
    t = restated.orient(xyz, tets)
    XYo = np.ascontiguousarray(xyz[t].reshape(-1, 12))
    q2 = restated.quad_points(2, XYo)
    D = (1 + q2[..., 0] ** 2)[..., None] * np.eye(3).reshape(1, 1, 9)  # s I per point (GRAD . GRAD)
    bnd = (np.any(np.abs(xyz) < 1e-14, axis=1) | np.any(np.abs(xyz - 1) < 1e-14, axis=1)).astype(np.uint8)
    ref = restated.assemble_problem(xyz, tets, 1, POINT, D, 1.0, 2, dirichlet=(bnd, None))
    assert np.array_equal(out["ex1_rowptr"].astype(np.int64), ref["rowptr"])
    assert np.array_equal(out["ex1_col"].astype(np.int64), ref["col"].astype(np.int64))
    v, rv = out["ex1_vals"], ref["vals"]
    assert np.abs(v - rv).max() <= 1e-12 * np.abs(rv).max()
    b, rb = out["ex1_rhs"], ref["rhs"]
    assert np.abs(b - rb).max() <= 1e-12 * np.abs(rb).max()
