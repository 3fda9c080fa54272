"""Build recipe for the CPU oracle (test infrastructure, never part of the product path).

The reference crate is Rust and no Rust toolchain is available, so there is no
compiled reference under ``oracle/_ref``; the oracle is the C++ restatement in
``lq_oracle.cpp``, built here into ``oracle/_build/liblq_oracle.so``.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liblq_oracle.so")
SRC = os.path.join(HERE, "lq_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "lq_oracle.h"))
    ):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [
        "g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math",
        SRC, "-o", tmp,
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
