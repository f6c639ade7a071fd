"""CPU tests of the host side: the C ABI library loads and exports every declared symbol,
the synthetic inputs are deterministic, and the Python mirror declares every entry point."""
import os
import re

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "anigpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(anigpu_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import ctypes

    import anigpu
    anigpu.build()  # incremental: rebuilds when a source is newer than the library
    lib = ctypes.CDLL(anigpu.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    import anigpu
    assert set(declared_symbols()) == set(anigpu.SIGNATURES)


def test_library_load_without_gpu_fails_loudly():
    import anigpu
    import torch
    if torch.cuda.is_available():
        return
    try:
        anigpu.Anigpu(0)
    except RuntimeError as e:
        assert "CUDA" in str(e)
    else:
        raise AssertionError("handle created without a GPU")


def test_quadrature_from_library_matches_oracle(restated):
    import anigpu
    anigpu.load_library()
    for o in range(21):
        p, w = anigpu.quadrature(o)
        po, wo = restated.quadrature(o)
        assert np.array_equal(p, po) and np.array_equal(w, wo)


def test_drop_in_template_header_compiles():
    """include/anigpu_fem.hpp with code spelled against AniFem++'s headers (tests/cpp/fem_template.cpp:
    fem3Dtet<Operator<...>, Operator<...>, DfuncTraits<...>>, functors, GenerateElemMatRhs, Assembler)
    compiles as C++14 and C++17 (no GPU needed; tests/test_gpu_template.py runs it)."""
    import subprocess
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for std in ("c++14", "c++17"):
        r = subprocess.run(["g++", f"-std={std}", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                            os.path.join(REPO, "include"), "-I", os.path.join(cuda, "include"),
                            os.path.join(REPO, "tests", "cpp", "fem_template.cpp")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_splitmix_streams_are_fixed():
    from anigpu import meshgen
    z = meshgen.splitmix64(0, 3)
    # splitmix64 of state 0: published first outputs
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    u = meshgen.uniform(7, 1000)
    assert 0 <= u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.05


def test_kuhn_mesh_and_tensors():
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(4, perturb=0.2, seed=5)
    assert xyz.shape == (125, 3) and tets.shape == (384, 4)
    h = 1.0 / 4
    xyz0, _ = meshgen.kuhn_cube(4)
    assert np.abs(xyz - xyz0).max() <= 0.2 * h + 1e-15
    assert np.all(meshgen.boundary_mask(xyz)[meshgen.boundary_mask(xyz0) == 1] == 1)
    vol = np.linalg.det(np.stack([xyz[tets[:, k]] - xyz[tets[:, 3]] for k in range(3)], axis=1))
    assert np.all(np.abs(vol) > 1e-6)
    D = meshgen.sym6_to_full(meshgen.aniso_tensors(1000, 1.5, 9))
    ev = np.linalg.eigvalsh(D)
    assert np.all(ev > 0)
    assert np.allclose(D, np.transpose(D, (0, 2, 1)))


def test_config2_sizes():
    from anigpu import meshgen
    n = 64
    assert 6 * n ** 3 == 1572864 and (n + 1) ** 3 == 274625
    # P2 DOFs = vertices + edges of the Kuhn mesh
    ne = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert (n + 1) ** 3 + ne == 2146689


def test_runtime_space_header_host(tmp_path):
    """The C++ runtime-space layer (include/anigpu.hpp, mirroring Ani::FemSpace / ApplyOp):
    operator metadata and argument errors, compiled with g++ against the library (no GPU)."""
    import subprocess

    from helpers import build_runtime_space_test
    exe = build_runtime_space_test(str(tmp_path))
    r = subprocess.run([exe, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "host ok" in r.stdout
