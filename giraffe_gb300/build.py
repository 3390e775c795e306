"""Builds the CUDA library giraffe_gb300/libgiraffe_gpu.so in place (sm_103a).

The library is self-contained (static CUDA runtime) and exposes the C ABI of
include/giraffe_gpu.h.  Translation units compile in parallel; the build is a
few nvcc invocations, no CMake.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libgiraffe_gpu.so")
OBJ = os.path.join(HERE, "_build")
SOURCES = ["gf_kernels.cu", "gf_chain.cu", "gf_shell.cu", "gf_wideband.cu", "gf_host.cu", "gf_server.cu", "gf_sparse.cu", "gf_iter.cu", "gf_modal.cu", "gf_tune.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _deps():
    out = []
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cuh", ".h"))]
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in _deps()):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")

    def cc(src):
        obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        return obj, r.stderr

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        res = list(ex.map(cc, SOURCES))
    if verbose:
        for _, err in res:
            sys.stderr.write(err)
    tmp = LIB + ".tmp"
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in res], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
