#!/usr/bin/env python3
"""Builds the oracle (test infrastructure only): the C++ restatement
``pt_oracle.cpp`` -> ``oracle/_build/libpg3oracle.so`` and, when the reference
sources are reachable, the reference harness binaries in ``oracle/_ref``
(see build_ref.py)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpg3oracle.so")


def build_oracle(force=False):
    srcs = [os.path.join(HERE, f) for f in ("pt_oracle.cpp", "lbvh_oracle.cpp")]
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC"] + srcs + ["-o", LIB]
    subprocess.check_call(cmd)
    return LIB


def build_all(with_ref=True):
    build_oracle()
    if with_ref:
        sys.path.insert(0, HERE)
        import build_ref
        build_ref.build()
        build_ref.build_gpu_shim()


if __name__ == "__main__":
    build_all(with_ref="--no-ref" not in sys.argv)
    print("oracle built")
