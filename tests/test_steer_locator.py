"""The steerable sampler's point-location tables, checked on the CPU.

tests/steer_locator_check.cpp is compiled with the host build of the tables
(pg3render_gb300/csrc/pg3_steerable.cpp) and repeats the device's location steps in float
(csrc/pg3_steer.cuh): it checks that the start cells give the same leaf as the path without them
(random directions and directions within ulps of the cells' borders), and that the candidate
lists give the leaf a brute-force test over all leaves gives. The GPU tests check the same tables
through the sampler's pdf consistency, chi-square and golden-image tests.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from pg3render_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pg3render_gb300", "csrc")


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("locator") / "steer_locator_check")
    # the library's host flags: no floating-point contraction
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", inc,
                    os.path.join(ROOT, "tests", "steer_locator_check.cpp"), os.path.join(CSRC, "pg3_steerable.cpp"),
                    "-o", exe, "-lpthread"], check=True, capture_output=True)
    return exe


def _run(args):
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_uniform_locator_tables(checker):
    out = _run([checker, "uniform", "6", "100000"])
    assert out.count("0 start-cell disagreements") == 7 and out.count("checks: 0 disagreements") == 7, out


def test_adaptive_locator_tables(checker, tmp_path):
    # the benchmark sky (1-3 degree suns) with the reference's default build: levels 4-9, error 5
    sky = S.cornell_env(8, 8, 1024, 512, em_seed=7).env_map
    path = str(tmp_path / "sky.bin")
    np.ascontiguousarray(sky, dtype=np.float32).tofile(path)
    out = _run([checker, "adaptive", path, "1024", "512", "4", "9", "5", "400000"])
    leaves = int(out.split("leaves ")[1].split(",")[0])   # 11216 here (the map's last bits vary by platform)
    assert leaves > 5000 and "0 start-cell disagreements" in out and "checks: 0 disagreements" in out, out
