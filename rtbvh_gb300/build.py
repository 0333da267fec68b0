"""Compiles the CUDA/C++ sources of the package into an in-tree shared
library, ``rtbvh_gb300/_lib/librtbvh_gb300.so`` (plus ``librtbvh_rs.so``, the
file name the reference's C users link against).

Every translation unit is built for sm_103a only, with FMA contraction off
(``--fmad=false`` for device code, ``-ffp-contract=off`` for host code) and
IEEE division, so that float results round exactly like the reference's
scalar code. Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "librtbvh_gb300.so")
ALIAS = os.path.join(OUT_DIR, "librtbvh_rs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-warn-spills"]
# The differentiable backward pass is float math without a bit-exactness
# requirement against the reference; it may contract to FMA.
PER_FILE = {"diff.cu": ["--fmad=true"]}


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources():
    return sorted(f for f in os.listdir(SRC_DIR) if f.endswith(".cu"))


def _headers_mtime():
    paths = [os.path.join(SRC_DIR, f) for f in os.listdir(SRC_DIR) if f.endswith((".h", ".cuh"))]
    paths.append(os.path.join(HERE, "..", "include", "rtbvh.h"))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, force):
    obj = os.path.join(OBJ_DIR, src[:-3] + ".o")
    sp = os.path.join(SRC_DIR, src)
    if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(sp)
            and os.path.getmtime(obj) >= _headers_mtime()):
        return obj, None
    flags = list(NVCC_FLAGS)
    for extra in PER_FILE.get(src, []):
        if extra.startswith("--fmad"):
            flags = [f for f in flags if not f.startswith("--fmad")]
        flags.append(extra)
    cmd = [nvcc(), *ARCH, *flags, "-c", sp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    errors = [err for _, err in results if err]
    if errors:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        if verbose:
            print("built", LIB)
    if os.path.lexists(ALIAS):
        os.remove(ALIAS)
    shutil.copyfile(LIB, ALIAS)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
