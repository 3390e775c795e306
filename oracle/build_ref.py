"""Builds oracle/_ref/libgiraffe_ref.so from the reference's own sources.

TEST INFRASTRUCTURE.  The reference (C++14 written for MSVC + oneMKL) is
compiled in place from the reference tree's src/ — nothing is copied — with the
headers in oracle/ref_shim/ (rvalue-binding overloads, BLAS/LAPACK
declarations, a CSR stand-in for Eigen's sparse header) and linked with
oracle/ref_blas.c, oracle/ref_support.cpp and oracle/ref_driver.cpp.  Symbols
that the listed sources reference only from branches the implicit beam/shell
path never takes (contact search, splines, particles, ...) are bound to
generated stubs that abort if ever called.

The library is x86-64 only and is built only where the reference tree is
present; it never travels to or runs on the GPU host.  Usage:

    python oracle/build_ref.py [--reference <reference tree>] [--jobs N]

The tree defaults to the environment variable GIRAFFE_REFERENCE.
"""
import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
OBJ = os.path.join(OUT, "obj")

# Reference translation units of the implicit Beam_1/Pipe_1/Shell_1 path.
SOURCES = [
    "Matrix", "Beam_1", "Shell_1", "Node", "LagrangeSave", "Hooke", "SecTube", "SecRectangle",
    "ShellSectionHomogeneous", "CoordinateSystem", "Table", "Static", "Dynamic", "Solution",
    "ConvergenceCriteria", "NodalLoad", "NodalConstraint", "NodeSet", "ElementSet", "BoolTable", "Load",
    "Element", "NodalDisplacement", "ShellLoad", "SolverOptions", "SolidSection", "Pipe_1", "PipeSection",
    "PipeLoad", "Modal", "Monitor",
]
# Per-source preprocessor definitions: Monitor.cpp's own file writer is
# renamed out of the way so that ref_support.cpp's recording hook takes the
# name (the rest of Monitor.cpp, its deck reader, is used as it is).
SOURCE_DEFINES = {"Monitor": ["-DUpdateMonitor=UpdateMonitor_file_writer"]}

CXXFLAGS = ["-std=c++14", "-O2", "-fPIC", "-fpermissive", "-w", "-fno-fast-math",
            "-ffp-contract=off"]


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise SystemExit(1)
    return r.stdout


def compile_one(src, obj, ref_src):
    if src.endswith(".c"):
        cmd = ["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj]
    else:
        extra = SOURCE_DEFINES.get(os.path.splitext(os.path.basename(src))[0], [])
        cmd = ["g++"] + CXXFLAGS + extra + ["-include", os.path.join(HERE, "ref_shim", "rvalue_shim.h"),
                                     "-I", os.path.join(HERE, "ref_shim"), "-I", ref_src,
                                     "-c", src, "-o", obj]
    run(cmd)
    return obj


LIB_PREFIXES = ("_ZNSt", "_ZNKSt", "_ZSt", "_Znw", "_Zna", "_Zdl", "_Zda", "_ZTVN10__cxxabiv1",
                "_ZNSo", "_ZNSi", "_ZNKSo", "_ZTISt", "_ZTIN10__cxxabiv1", "_ZGV", "__")


def stub_source(undefined):
    lines = ["// generated by oracle/build_ref.py: stubs for symbols off the implicit path",
             "#include <cstdio>", "#include <cstdlib>"]
    n = 0
    for sym in sorted(undefined):
        if sym.startswith("_ZTI"):
            # typeinfo of a class used only in typeid() comparisons: emit it
            # from a same-named polymorphic placeholder class.
            m = re.match(r"_ZTI(\d+)(\w+)$", sym)
            if not m or int(m.group(1)) != len(m.group(2)):
                raise SystemExit("cannot stub " + sym)
            name = m.group(2)
            lines.append(f"class {name} {{ public: virtual ~{name}(); }};")
            lines.append(f"{name}::~{name}() {{}}")
            continue
        n += 1
        lines.append(f'extern "C" void gf_ref_stub_{n}(void) __asm__("{sym}");')
        lines.append(f'extern "C" void gf_ref_stub_{n}(void) {{ fprintf(stderr, "reference '
                     f'build: stub {sym} called\\n"); abort(); }}')
    return "\n".join(lines) + "\n"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("GIRAFFE_REFERENCE", "/root/reference"))
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    ref_src = os.path.join(a.reference, "src")
    if not os.path.isdir(ref_src):
        print("reference sources not present; oracle/_ref not built")
        return 0
    os.makedirs(OBJ, exist_ok=True)
    jobs = [(os.path.join(ref_src, s + ".cpp"), os.path.join(OBJ, s + ".o")) for s in SOURCES]
    for s in ("ref_support.cpp", "ref_driver.cpp", "ref_blas.c"):
        jobs.append((os.path.join(HERE, s), os.path.join(OBJ, os.path.splitext(s)[0] + ".o")))
    with ThreadPoolExecutor(a.jobs) as ex:
        objs = list(ex.map(lambda j: compile_one(j[0], j[1], ref_src), jobs))
    defined, undefined = set(), set()
    for o in objs:
        for line in run(["nm", o]).splitlines():
            parts = line.split()
            if len(parts) == 2 and parts[0] in ("U", "w"):
                undefined.add(parts[1])
            elif len(parts) == 3 and parts[1] not in ("U", "w"):
                defined.add(parts[2])
    missing = {s for s in undefined - defined
               if s.startswith("_Z") and not s.startswith(LIB_PREFIXES)}
    stub = os.path.join(OBJ, "ref_stubs.cpp")
    with open(stub, "w") as f:
        f.write(stub_source(missing))
    objs.append(compile_one(stub, os.path.join(OBJ, "ref_stubs.o"), ref_src))
    lib = os.path.join(OUT, "libgiraffe_ref.so")
    run(["g++", "-shared", "-o", lib] + objs + ["-Wl,--no-undefined", "-lm"])
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
