"""Shared helpers of the parity tests."""
import os

import numpy as np

EPS = np.finfo(np.float64).eps


def ref_tol(A):
    """The reference's tolerance convention ||A - A_exp||_F <= 10 (1 + ||A||_F) eps
    (tests/fem/operations/int_tet_test.cpp:257)."""
    return 10 * (1 + np.linalg.norm(A)) * EPS


def rel_err_per_tet(A, B):
    """max over tets of ||A_t - B_t||_F / ||B_t||_F."""
    A = np.asarray(A).reshape(A.shape[0], -1)
    B = np.asarray(B).reshape(B.shape[0], -1)
    nb = np.linalg.norm(B, axis=1)
    nb[nb == 0] = 1
    return float(np.max(np.linalg.norm(A - B, axis=1) / nb))


NF = {0: 1, 1: 4, 2: 10, 3: 20, 4: 12, 5: 30, 6: 4, 7: 6, 8: 1}
DIM = {1: 1, 2: 3}


def op_nf_dim(code):
    space, op = divmod(code, 10)
    if space in (9, 10):  # ND0, RT0: IDEN 3, GRAD 9, DIV 1, CURL 3
        return (6 if space == 9 else 4), {1: 3, 2: 9, 3: 1, 4: 3}[op]
    nc = 3 if space in (4, 5) else 1
    return NF[space], DIM[op] * nc


def point_tensor(fn, X, nr, nc):
    """Analytic per-point fields (same formulas as oracle/ref_driver.cpp eval_fn), column-major."""
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
    if fn == 3:
        return (x * x)[..., None]
    raise ValueError(fn)


def parse_case(name):
    a, b, kind, order = name.split("_")
    return int(a), int(b), kind, int(order[1:])


KIND_CODE = {"null": 0, "cscalar": 1, "tscalar": 2, "tsym": 3, "tgeneral": 4}


def build_runtime_space_test(outdir):
    """Compile tests/cpp/runtime_space.cpp against include/anigpu.hpp and the built library."""
    import subprocess
    import anigpu
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(anigpu.LIB_PATH)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(outdir, "runtime_space")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(repo, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(repo, "tests", "cpp", "runtime_space.cpp"), "-o", exe, "-L", libdir, "-lanigpu",
           f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe
