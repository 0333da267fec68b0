"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement of the reference's CPU algorithms into
``oracle/_build/liboracle.so``. FMA contraction is disabled so that the
float arithmetic rounds exactly as the reference's scalar Rust code does,
on x86-64 and on aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "rtbvh_oracle.cpp")

CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", *CXXFLAGS, "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
