#!/usr/bin/env python3
"""Generate the golden fixtures of the parity tests from the reference itself.

Run where the reference sources exist (they are not present on GPU machines):
    make -C oracle ref && python tests/golden/gen_golden.py [REF_ROOT]

Writes tests/golden/golden.npz with
  * int_tet_test_*   the golden matrices of the reference's own unit tests, read as text
                     from tests/fem/operations/int_tet_test.cpp (Operations_IntTet_OnePointTensor
                     :229-243 and :333-346, RhsEval :455) together with their scale factors;
  * quad_<order>     the reference's tetrahedron rules (quadrature_formulas.cpp:526);
  * case_<name>_*    inputs and outputs of the reference's fem3Dtet (compiled from its
                     sources by oracle/Makefile) on seeded random tets, for every operator
                     pair and tensor kind the GPU path provides;
  * apply_<code>_*   the reference's fem3DapplyL (order-4 quadrature points) and fem3DapplyX
                     (seeded physical points) on the same tets for every operator code;
  * tri_<order>_*    the reference's triangle rules (quadrature_formulas.cpp:109);
  * sliver_<name>_*  the reference's fem3Dtet on badly shaped tets (slivers, caps, needles);
  * face_<name>_*    the reference's fem3Dface (int_face.inl:12-44) on the same tets, every face;
  * facen_<name>_*   the reference's fem3DfaceN (int_face.inl:48-78), tensors of 3*dimB rows.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "inmost-fem_gb300"))

from oracle.oracle import Reference  # noqa: E402
from anigpu import meshgen  # noqa: E402

# operator codes: 10*space + op (space 0 P0, 1 P1, 2 P2, 3 P3, 4 Vec3P1, 5 Vec3P2; op 1 IDEN, 2 GRAD)
NF = {0: 1, 1: 4, 2: 10, 3: 20, 4: 12, 5: 30, 6: 4, 7: 6, 8: 1}
DIM = {1: 1, 2: 3}


def op_nf_dim(code):
    space, op = divmod(code, 10)
    if space in (9, 10):  # ND0, RT0
        return (6 if space == 9 else 4), {1: 3, 2: 9, 3: 1, 4: 3}[op]
    nc = 3 if space in (4, 5) else 1
    return NF[space], DIM[op] * nc


def parse_int_tet_test(path):
    src = open(path).read()
    # 12 x 20 block of Operations_IntTet_OnePointTensor
    m = re.search(r"At_exp_m\{std::array<double, 20>\s*(.*?)\};", src, re.S)
    rows = re.findall(r"\{([^{}]*)\}", m.group(1))
    A1 = np.array([[float(v) for v in r.replace("\n", " ").split(",") if v.strip()] for r in rows])
    m = re.search(r"double A_exp_m1p\[\] = \{(.*?)\};", src, re.S)
    A2 = np.array([float(v) for v in m.group(1).split(",") if v.strip()]).reshape(12, 12)
    m = re.search(r"Bp\[30\] = \{(.*?)\}", src, re.S)
    Bp = np.array([float(v) for v in m.group(1).split(",") if v.strip()])
    return A1, A2, Bp


def point_tensor(fn, X, nr, nc):
    """The analytic per-point fields of oracle/ref_driver.cpp (eval_fn), column-major nr x nc."""
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    if fn == 0:
        out = np.zeros(X.shape[:-1] + (nr * nc,))
        cnt = 0
        for i in range(nr):
            for j in range(nc):
                out[..., i + nr * j] = (i * x + j * y + (i % 2) * z) * cnt
                cnt += 1
        return out
    if fn == 2:
        m = [1 + x * x, x * y / 2, 0 * x, x * y / 2, 1 + y * y, z / 3, 0 * x, z / 3, 2 + z * z]
        return np.stack(m, axis=-1)
    raise ValueError(fn)


# operator pairs whose fixtures also cover orders 8, 13 and 20 (the PlainMemory overload of
# fem3Dtet, int_tet.inl:30-57, takes orders up to 20)
HIGH_ORDER_PAIRS = ((12, 12), (22, 22), (52, 52), (32, 32), (1, 21), (91, 91), (102, 102))


def sliver_tets(seed=91):
    """Badly shaped tets, each rotated, scaled and moved by seeded random values: slivers (four
    nearly coplanar vertices), caps (a vertex close to the opposite face), needles, wedges and
    spindles, with shape parameters e from 0.3 down to 1e-3."""
    shapes = []
    for e in (0.3, 0.1, 0.05, 0.02, 0.01, 1e-3):
        shapes.append([(0, 0, 0), (1, 1, 0), (1, 0, e), (0, 1, e)])          # sliver
        shapes.append([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0.3, 0.3, e)])      # cap
        shapes.append([(0, 0, 0), (1, 0, 0), (0.5, e, 0), (0.5, 0, e)])      # spindle
        shapes.append([(0, 0, 0), (1, 0, 0), (1, e, 0), (0.3, 0.2, e)])      # wedge
    shapes.append([(0, 0, 0), (1e-2, 0, 0), (0, 1e-2, 0), (0, 0, 1)])          # needle
    n = len(shapes)
    X = np.array(shapes, dtype=np.float64)                                  # n x 4 x 3
    qv = meshgen.normal(seed, 4 * n).reshape(n, 4)
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    w, x, y, z = qv.T
    R = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                  2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                  2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1).reshape(n, 3, 3)
    scale = 0.5 + meshgen.uniform(seed + 1, n)
    shift = (meshgen.uniform(seed + 2, 3 * n).reshape(n, 1, 3) - 0.5) * 200.0
    X = np.einsum("tij,tvj->tvi", R, X) * scale[:, None, None] + shift
    return np.ascontiguousarray(X.reshape(n, 12))


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ANIFEM_REF_ROOT", "")
    if not ref_root:
        raise SystemExit("usage: gen_golden.py REF_ROOT (or set ANIFEM_REF_ROOT)")
    if not Reference.available():
        raise SystemExit("build the reference oracle first: make -C oracle ref")
    R = Reference()
    out = {}
    A1, A2, Bp = parse_int_tet_test(os.path.join(ref_root, "tests/fem/operations/int_tet_test.cpp"))
    out["int_tet_test_onepoint_12x20"] = A1
    out["int_tet_test_onepoint_coef"] = np.array(9 * 80.0)
    out["int_tet_test_vecp1_12x12"] = A2
    out["int_tet_test_vecp1_coef"] = np.array(9 * 160.0)
    out["int_tet_test_rhs_Bp"] = Bp
    # the golden tests' tets (XY1p+3 etc. in int_tet_test.cpp:191-201 and :398-403)
    out["int_tet_test_tet_onepoint"] = np.array([0, 0, 0, 2, 1, 1, 1, 2, 1, 2, 1, 2], dtype=np.float64)
    out["int_tet_test_tet_rhs"] = np.array([0, 0, 0, 2, 1, 1, 1, 2, 1, 2, 1, 2], dtype=np.float64)
    for o in range(21):
        p, w = R.quadrature(o)
        out[f"quad_{o}_p"] = p
        out[f"quad_{o}_w"] = w

    nt = 6
    XY = meshgen.random_tets(nt, seed=11)
    out["tets_XY"] = XY
    cases = []
    scalar_tet = np.exp(meshgen.normal(21, nt))
    sym6 = meshgen.aniso_tensors(nt, sigma=1.0, seed=22)
    for (ca, cb) in [(12, 12), (22, 22), (32, 32), (42, 42), (52, 52), (32, 42), (11, 11), (21, 21), (31, 31),
                     (1, 11), (1, 21), (1, 51), (12, 22), (22, 12),
                     (61, 61), (62, 62), (1, 61), (71, 71), (72, 72), (81, 81), (82, 82), (11, 81), (81, 11),
                     (91, 91), (94, 94), (92, 92), (101, 101), (103, 103), (102, 102), (103, 1), (91, 101)]:
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        kinds = []
        if dA == dB or dA == 1:
            kinds += [("null", 0, None), ("cscalar", 1, np.array([2.5])), ("tscalar", 2, scalar_tet)]
        if dA == 3 and dB == 3:
            kinds += [("tsym", 3, sym6)]
        gen = (meshgen.uniform(31 + ca + cb, nt * dA * dB) - 0.5).reshape(nt, dA * dB)
        kinds += [("tgeneral", 4, gen)]
        orders = (2, 3, 4, 5, 6) + ((8, 13, 20) if (ca, cb) in HIGH_ORDER_PAIRS else ())
        for order in orders:
            for kname, kind, D in kinds:
                name = f"{ca}_{cb}_{kname}_o{order}"
                A = R.fem3dtet(ca, cb, kind, order, XY, D, nfA=nfA, nfB=nfB)
                out[f"case_{name}_A"] = A
                if D is not None:
                    out[f"case_{name}_D"] = np.asarray(D, dtype=np.float64)
                cases.append(name)
            # per-point analytic field (fn 0 general; fn 2 symmetric 3x3)
            fns = [0] + ([2] if (dA == 3 and dB == 3) else [])
            for fn in fns:
                name = f"{ca}_{cb}_point{fn}_o{order}"
                A = R.fem3dtet(ca, cb, 5, order, XY, None, fn=fn, nfA=nfA, nfB=nfB)
                out[f"case_{name}_A"] = A
                cases.append(name)
    out["case_names"] = np.array(cases)
    # badly shaped tets (slivers, caps, needles, wedges; |det| / (|e1||e2||e3|) from 0.3 down to
    # 1e-3), where the FP32 kernels redo the geometry in FP64
    SX = sliver_tets()
    out["sliver_XY"] = SX
    ns = SX.shape[0]
    sym6s = meshgen.aniso_tensors(ns, sigma=1.0, seed=23)
    sliver_cases = []
    for (ca, cb) in [(12, 12), (22, 22), (52, 52), (32, 32), (1, 21)]:
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        kinds = [("tgeneral", 4, (meshgen.uniform(81 + ca + cb, ns * dA * dB) - 0.5).reshape(ns, dA * dB))]
        if dA == 3 and dB == 3:
            kinds += [("tsym", 3, sym6s)]
        if dA == dB or dA == 1:
            kinds += [("null", 0, None)]
        for kname, kind, D in kinds:
            name = f"{ca}_{cb}_{kname}_o4"
            out[f"sliver_{name}_A"] = R.fem3dtet(ca, cb, kind, 4, SX, D, nfA=nfA, nfB=nfB)
            if D is not None:
                out[f"sliver_{name}_D"] = np.asarray(D, dtype=np.float64)
            sliver_cases.append(name)
    out["sliver_case_names"] = np.array(sliver_cases)
    # fem3DapplyL at the order-4 quadrature points and fem3DapplyX at seeded physical points (some
    # outside the tet), for every operator code, on the same tets
    p4, _ = R.quadrature(4)
    out["apply_XYL"] = p4
    out["apply_X"] = meshgen.uniform(41, nt * 7 * 3).reshape(nt, 7, 3) * 3.0 - 1.0
    apply_codes = [1, 11, 12, 21, 22, 31, 32, 41, 42, 51, 52, 61, 62, 71, 72, 81, 82,
                   91, 92, 93, 94, 101, 102, 103, 104]
    for code in apply_codes:
        nf, dim = op_nf_dim(code)
        dofs = meshgen.normal(50 + code, nt * nf).reshape(nt, nf)
        out[f"apply_{code}_dofs"] = dofs
        out[f"apply_{code}_L"] = R.fem3d_apply(code, XY, p4, dofs, nf, dim)
        out[f"apply_{code}_X"] = R.fem3d_apply(code, XY, out["apply_X"], dofs, nf, dim, phys=True)
    out["apply_codes"] = np.array(apply_codes)
    # the reference's triangle rules and fem3Dface (every face, orders 0..9) on the same tets
    for o in range(21):
        p3, w3 = R.tri_quadrature(o)
        out[f"tri_{o}_p"] = p3
        out[f"tri_{o}_w"] = w3
    face_cases = []
    for (ca, cb) in [(1, 21), (21, 21), (1, 51), (11, 11), (1, 11), (22, 22), (12, 12)]:
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        gen = (meshgen.uniform(61 + ca + cb, nt * dA * dB) - 0.5).reshape(nt, dA * dB)
        kinds = [("tgeneral", 4, gen)]
        if dA == dB or dA == 1:
            kinds += [("null", 0, None), ("tscalar", 2, scalar_tet)]
        for order in (1, 2, 4, 7, 9) + ((13, 20) if (ca, cb) in ((1, 21), (22, 22)) else ()):
            for face in range(4):
                for kname, kind, D in kinds:
                    name = f"{ca}_{cb}_{kname}_o{order}_f{face}"
                    out[f"face_{name}_A"] = R.fem3dface(ca, cb, kind, order, face, XY, D, nfA=nfA, nfB=nfB)
                    if D is not None:
                        out[f"face_{name}_D"] = np.asarray(D, dtype=np.float64)
                    face_cases.append(name)
                name = f"{ca}_{cb}_point0_o{order}_f{face}"
                out[f"face_{name}_A"] = R.fem3dface(ca, cb, 5, order, face, XY, None, fn=0, nfA=nfA, nfB=nfB)
                face_cases.append(name)
    out["face_case_names"] = np.array(face_cases)
    # fem3DfaceN: tensors of 3*dimB rows contracted with the outward normal
    facen_cases = []
    for (ca, cb) in [(1, 51), (1, 21), (22, 21), (12, 11)]:
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        dBt = 3 * dB
        kinds = [("tgeneral", 4, (meshgen.uniform(71 + ca + cb, nt * dA * dBt) - 0.5).reshape(nt, dA * dBt))]
        if dA == dBt or dA == 1:
            kinds += [("null", 0, None), ("tscalar", 2, scalar_tet)]
        if dA == 3 and dBt == 3:
            kinds += [("tsym", 3, sym6)]
        for order in (2, 5, 8):
            for face in range(4):
                for kname, kind, D in kinds:
                    name = f"{ca}_{cb}_{kname}_o{order}_f{face}"
                    out[f"facen_{name}_A"] = R.fem3dface(ca, cb, kind, order, face, XY, D, nfA=nfA, nfB=nfB,
                                                         normal=True)
                    if D is not None:
                        out[f"facen_{name}_D"] = np.asarray(D, dtype=np.float64)
                    facen_cases.append(name)
    out["facen_case_names"] = np.array(facen_cases)
    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print(path, len(cases), "cases", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
