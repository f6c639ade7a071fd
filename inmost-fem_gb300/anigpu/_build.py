"""In-tree build of libanigpu.so (nvcc, sm_103a only) and of the oracle used by tests."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                 # inmost-fem_gb300/
CSRC = os.path.join(ROOT, "csrc")
REPO = os.path.dirname(ROOT)
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libanigpu.so")

SOURCES = ["api.cu", "k_element.cu", "k_setup.cu", "k_assemble.cu", "k_solve.cu", "k_learned.cu", "k_fcg.cu", "k_batch.cu", "k_enum.cu", "k_general.cu", "basis.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", GENCODE, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose=False, force=False):
    """Compile every translation unit in parallel and link libanigpu.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "anigpu.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [sp] + headers):
            cmd = [nvcc] + NVCC_FLAGS + ["-I", CSRC, "-I", os.path.join(REPO, "include"), "-c", sp, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nvcc] + NVCC_FLAGS + ["-x", "cu", "-I", CSRC, "-I", os.path.join(REPO, "include"), "-c", sp, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(failed))
    if force or jobs or not os.path.exists(LIB_PATH):
        cmd = [nvcc, GENCODE, "-shared", "-o", LIB_PATH] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def build_oracle(with_reference=True, verbose=False):
    """Build the oracle (test infrastructure): the C restatement always, and the
    reference's own fem3Dtet when ANIFEM_REF_ROOT names a checkout of the reference sources."""
    oracle = os.path.join(REPO, "oracle")
    r = subprocess.run(["make", "-C", oracle, "restate"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    ref_root = os.environ.get("ANIFEM_REF_ROOT", "")
    if with_reference and ref_root and os.path.isdir(os.path.join(ref_root, "anifem++")):
        r = subprocess.run(["make", "-C", oracle, "ref", f"REF_ROOT={ref_root}"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference oracle build failed:\n" + r.stdout + r.stderr)


if __name__ == "__main__":
    build_library(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_oracle()
    print(LIB_PATH)
