"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles oracle/esc_oracle.cpp into oracle/_build/liboracle.so with g++ and OpenMP.  Portable
flags only (no -march): the same recipe runs on x86_64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "esc_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(SO)
            and os.path.getmtime(SO) >= max(os.path.getmtime(SRC), os.path.getmtime(__file__))):
        return SO
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fcx-limited-range", "-fopenmp", "-shared", "-fPIC", "-o", SO + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(SO + ".tmp", SO)
    return SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
