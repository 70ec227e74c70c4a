"""Build the CUDA library in-tree: grtm_cuda_gb300/_lib/libgrtm_gb300.so.

nvcc compiles each translation unit for sm_103a only (in parallel) and links
a shared library with a plain C ABI (include/grtm_gb300.h).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libgrtm_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 division and square root to ~2 ulp, subnormals flushed: the GRT kernel's
# 2x2 inverses and complex square roots dominate its instruction count, and
# its parity with the FP64 oracle is unchanged (FP64 code is not affected)
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
SOURCES = ["grt_api.cu", "grt_grt_f32.cu", "grt_grt_f64.cu", "grt_tc_tf32.cu", "grt_tc_bf16.cu", "grt_job.cpp",
           "grt_noalloc.cu", "grt_mlp.cu"]
# extra nvcc flags (e.g. -DGRT_POINT_MINB=4) and an alternative output path,
# for timing build variants side by side
EXTRA = os.environ.get("GRT_NVCC_EXTRA", "").split()
if os.environ.get("GRT_BUILD_TAG"):
    BUILD = BUILD + "_" + os.environ["GRT_BUILD_TAG"]
    LIB = os.path.join(LIBDIR, "libgrtm_gb300_" + os.environ["GRT_BUILD_TAG"] + ".so")


def _obj(src):
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def _stale(src):
    obj = _obj(src)
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "grtm_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False):
    cmd = [NVCC] + ARCH + FLAGS + EXTRA + (["-Xptxas", "-v"] if verbose else []) + [
        "-c", os.path.join(CSRC, src), "-o", _obj(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    todo = [s for s in SOURCES if force or _stale(s)]
    if todo:
        with ThreadPoolExecutor(max_workers=len(todo)) as ex:
            logs = list(ex.map(lambda s: _compile(s, verbose), todo))
        if verbose:
            for lg in logs:
                sys.stderr.write(lg)
    if todo or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + [_obj(s) for s in SOURCES] + ["-lcudart", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
