"""Builds the CUDA library ``libpg3gpu.so`` (sm_103a) in-tree.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into one shared object with the CUDA runtime linked statically, so the
library only needs the driver at run time. Output: pg3render_gb300/_build/.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpg3gpu.so")
ROOT = os.path.dirname(HERE)

SOURCES = ["pg3_api.cu", "pg3_host.cpp", "pg3_steerable.cpp", "pg3_megakernel.cu", "pg3_wavefront.cu", "pg3_lbvh.cu", "pg3_probe.cu",
           "pg3_batch.cu", "pg3_diff.cu", "pg3_steer_build.cu", "pg3_image.cpp", "pg3_emssd.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The rendering pipelines (wavefront, batch, megakernel) compile with fast division, square root
# and transcendentals and flushed subnormals (-use_fast_math: +10.7% on the environment-map
# benchmark), all three alike, so that they still give the same paths. Their results stay within
# the parity tests' tolerances; the pdf of every sampler is still evaluated with the same code
# that samples it. The rest (LBVH build, table builds, sampler probes) keeps IEEE arithmetic: the
# LBVH is bit-exact against its CPU build.
FAST_MATH_SOURCES = {"pg3_wavefront.cu", "pg3_batch.cu", "pg3_megakernel.cu"}
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "pg3gpu.h")]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra_flags=(), out_dir=None):
    """Compiles into out_dir (default pg3render_gb300/_build) and returns the library path."""
    bdir = out_dir or BUILD
    lib = os.path.join(bdir, "libpg3gpu.so")
    os.makedirs(bdir, exist_ok=True)
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _deps():
        return lib
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(bdir, src + ".o")
        fast = ["-use_fast_math"] if src in FAST_MATH_SOURCES else []
        cmd = [nvcc] + ARCH + NVCC_FLAGS + fast + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            # host code without floating-point contraction: the same results on x86 and Arm hosts
            # (build options given as -D reach the host sources too: some tables are shared)
            cmd = [nvcc] + NVCC_FLAGS + [f for f in extra_flags if f.startswith("-D")] + \
                ["-Xcompiler", "-ffp-contract=off", "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-8000:]))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-8000:])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
