#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref``: the reference renderer's own CPU code,
compiled with g++ so that it can serve as the statistical oracle and as the
timed CPU baseline.

Test infrastructure only. Nothing in the product path imports, links or runs
anything this script makes.

The reference (PG3Render) is MSVC C++ and does not compile with GCC as it lies.
This recipe therefore

1. copies ``src/*.hxx`` and ``src/*.cxx`` from the reference checkout into
   ``oracle/_ref/src`` (git-ignored build intermediate, never committed),
2. applies the mechanical MSVC -> GCC fixes listed in ``PATCHES`` below (each
   one only qualifies a name or adjusts a declaration; none changes the
   arithmetic), and
3. compiles ``oracle/ref_harness.cpp`` (this repository's own harness, which
   builds scenes through the reference's public ``Scene`` members and runs its
   ``PathTracer``) against the patched headers into ``oracle/_ref/``.

When the reference checkout is absent (e.g. on a machine that only received a
copy of this repository), step 1-2 are skipped and an existing
``oracle/_ref/src`` from an earlier run is compiled instead.

Usage: python oracle/build_ref.py [--ref-root DIR] [--jobs N]
"""
import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
STUBS = os.path.join(HERE, "stubs")


def default_ref_root():
    """The reference checkout: $PG3_REFERENCE_ROOT, else the `reference_path` of the repository's
    the benchmark spec (None when neither names one)."""
    env = os.environ.get("PG3_REFERENCE_ROOT")
    if env:
        return env
    try:
        import json
        with open(os.path.join(os.path.dirname(HERE), "BASELINE.json")) as f:
            return json.load(f).get("reference_path")
    except (OSError, ValueError):
        return None


def _sub_lines(text, first, last, pattern, repl):
    """Apply a regex substitution on 1-based lines [first, last] only."""
    lines = text.split("\n")
    for i in range(first - 1, min(last, len(lines))):
        lines[i] = re.sub(pattern, repl, lines[i])
    return "\n".join(lines)


def _qualify_member(text, name, skip_lines=()):
    """``name`` -> ``this->name`` where it is used as a bare identifier
    (dependent-base member lookup that MSVC accepts and GCC rejects)."""
    lines = text.split("\n")
    pat = re.compile(r"(?<![\w.>:])" + re.escape(name) + r"(?!\w)")
    for i, line in enumerate(lines):
        if (i + 1) in skip_lines:
            continue
        stripped = line.strip()
        # keep declarations of the member itself
        if re.match(r"^[A-Za-z_][\w:<>, ]*\s+" + name + r"\s*;", stripped):
            continue
        lines[i] = pat.sub("this->" + name, line)
    return "\n".join(lines)


def patch_spectrum(t):
    # SRGBSpectrumBase derives from the dependent base Vec3Base<T>: qualify x/y/z/Get.
    t = _sub_lines(t, 20, 85, r"(?<![\w.>])([xyz])(?![\w(])", r"this->\1")
    t = _sub_lines(t, 20, 85, r"(?<![\w.>])Get\(", r"this->Get(")
    return t


def patch_em_samplers(t):
    t = t.replace("EnvironmentMapSampler::", "EnvironmentMapSampler<TEmValues>::")
    return _qualify_member(t, "mEmImage")


def patch_steerable(t):
    t = patch_em_samplers(t)
    # constructor initialiser lists name the member of the class itself
    init_lines = {i + 1 for i, l in enumerate(t.split("\n")) if re.match(r"^\s*[:,]?\s*mBasisValues\s*\(", l)}
    t = _qualify_member(t, "mBasisValues", skip_lines=init_lines)
    return t


def patch_materials(t):
    return t.replace(
        "return aCtx.fresnelReflectance; // gets converted to spectrum...",
        "return SpectrumF().SetGreyAttenuation(aCtx.fresnelReflectance);")


def patch_utils(t):
    # explicit specialisations may not carry a storage class in ISO C++
    return re.sub(r"template <>\s*\n(\s*)static ", r"template <>\n\1", t)


def patch_va_args(t):
    return t.replace(", __VA_ARGS__", " __VA_OPT__(,) __VA_ARGS__")


def patch_hard_config(t):
    # make the environment-map sampler and the statistics print selectable with -D
    t = t.replace("#define PG3_USE_ENVMAP_SIMPLE_SPHERICAL_SAMPLER",
                  "#if !defined(PG3_USE_ENVMAP_STEERABLE_SAMPLER) && !defined(PG3_USE_ENVMAP_COSINE_SAMPLER)\n"
                  "#define PG3_USE_ENVMAP_SIMPLE_SPHERICAL_SAMPLER\n#endif")
    t = t.replace("#define PG3_COMPUTE_AND_PRINT_EM_STEERABLE_STATISTICS",
                  "#ifndef PG3_NO_EM_STEERABLE_STATISTICS\n#define PG3_COMPUTE_AND_PRINT_EM_STEERABLE_STATISTICS\n#endif")
    return t


PATCHES = {
    "spectrum.hxx": patch_spectrum,
    "em_cosine_sampler.hxx": patch_em_samplers,
    "em_simple_spherical_sampler.hxx": patch_em_samplers,
    "em_steerable_sampler.hxx": patch_steerable,
    "materials.hxx": patch_materials,
    "utils.hxx": patch_utils,
    "debugging.hxx": patch_va_args,
    "unit_testing.hxx": patch_va_args,
    "hard_config.hxx": patch_hard_config,
}

CXXFLAGS = ["-std=c++20", "-O2", "-fopenmp", "-fpermissive", "-w",
            "-D_MSC_VER=1900", "-D__declspec(x)=", "-include", "msvc_compat.h"]

# name -> extra defines; one harness binary per environment-map sampler choice
VARIANTS = {
    "pg3ref_cdf": [],
    "pg3ref_cos": ["-DPG3_USE_ENVMAP_COSINE_SAMPLER"],
    "pg3ref_steer": ["-DPG3_USE_ENVMAP_STEERABLE_SAMPLER", "-DPG3_NO_EM_STEERABLE_STATISTICS"],
}


def copy_and_patch(ref_root):
    src_dir = os.path.join(ref_root, "src")
    if os.path.isdir(SRC):
        shutil.rmtree(SRC)
    os.makedirs(SRC)
    for name in sorted(os.listdir(src_dir)):
        if not (name.endswith(".hxx") or name.endswith(".cxx")):
            continue
        with open(os.path.join(src_dir, name), "r", encoding="latin-1") as f:
            text = f.read()
        if name in PATCHES:
            text = PATCHES[name](text)
        with open(os.path.join(SRC, name), "w", encoding="latin-1") as f:
            f.write(text)


def compile_variants(jobs=3, variants=None):
    harness = os.path.join(HERE, "ref_harness.cpp")
    procs = []
    for name, defs in VARIANTS.items():
        if variants and name not in variants:
            continue
        out = os.path.join(OUT, name)
        cmd = (["g++"] + CXXFLAGS + defs + ["-I" + SRC, "-I" + STUBS, harness,
               os.path.join(SRC, "debugging.cxx"), "-o", out])
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        if len(procs) >= jobs:
            _wait(procs.pop(0))
    for p in procs:
        _wait(p)


def _wait(entry):
    name, p = entry
    out, _ = p.communicate()
    if p.returncode != 0:
        sys.stderr.write(out.decode(errors="replace")[-6000:])
        raise RuntimeError("oracle/_ref: compiling %s failed" % name)


GPU_SHIM = os.path.join(OUT, "pg3render_gpu")


def build_gpu_shim(force=False):
    """The reference's command line and render loop with the GPU renderer
    (pg3render_gb300/shim/pg3render_gpu.cpp + gpu_path_tracer.hxx), compiled against the patched
    reference headers and linked to the CUDA library -> oracle/_ref/pg3render_gpu. Needs the
    library built (pg3render_gb300/build.py) and the patched sources in oracle/_ref/src."""
    root = os.path.dirname(HERE)
    shim = os.path.join(root, "pg3render_gb300", "shim")
    libdir = os.path.join(root, "pg3render_gb300", "_build")
    lib = os.path.join(libdir, "libpg3gpu.so")
    srcs = [os.path.join(shim, "pg3render_gpu.cpp"), os.path.join(shim, "gpu_path_tracer.hxx"),
            os.path.join(root, "include", "pg3gpu.h"), lib]
    if not (os.path.isdir(SRC) and os.path.exists(lib)):
        return None
    if not force and os.path.exists(GPU_SHIM) and os.path.getmtime(GPU_SHIM) >= max(os.path.getmtime(f) for f in srcs):
        return GPU_SHIM
    cmd = (["g++"] + CXXFLAGS + ["-I" + SRC, "-I" + STUBS, "-I" + shim, "-I" + os.path.join(root, "include"),
           os.path.join(shim, "pg3render_gpu.cpp"), os.path.join(SRC, "debugging.cxx"),
           "-L" + libdir, "-lpg3gpu", "-Wl,-rpath," + libdir, "-o", GPU_SHIM])
    _wait(("pg3render_gpu", subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    return GPU_SHIM


def build(ref_root=None, jobs=3, variants=None):
    ref_root = ref_root or default_ref_root()
    os.makedirs(OUT, exist_ok=True)
    if ref_root and os.path.isdir(os.path.join(ref_root, "src")):
        copy_and_patch(ref_root)
    elif not os.path.isdir(SRC):
        return False
    compile_variants(jobs, variants)
    return True


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None)
    ap.add_argument("--jobs", type=int, default=3)
    ap.add_argument("--variant", action="append")
    a = ap.parse_args()
    ok = build(a.ref_root, a.jobs, a.variant)
    print("oracle/_ref built" if ok else "oracle/_ref: no reference sources, skipped")
