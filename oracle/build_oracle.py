"""Builds the CPU oracle library oracle/liboracle.so with gcc.

TEST INFRASTRUCTURE: the oracle gives the parity tests' reference values and
the timed CPU baseline; the product never loads it.  FMA contraction is disabled so the
same sources give the same bits on x86-64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["oracle_beam.c", "oracle_shell.c", "oracle_solver.c"]
LIB = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in os.listdir(HERE) if h.endswith(".h")]
    deps.append(os.path.join(HERE, "..", "include", "giraffe_model.h"))
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d)
                                                  for d in deps):
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
