"""CPU checks: the C-ABI library loads and exports every declared symbol,
the model/deck plumbing, section formulas and the seeded generators."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from giraffe_gb300 import configs
from giraffe_gb300.model import section_rectangle, section_tube

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_functions():
    names = set()
    for h in ("giraffe_gpu.h",):
        txt = open(os.path.join(ROOT, "include", h)).read()
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(gf_\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from giraffe_gb300 import build, gpu

    build.build()
    L = C.CDLL(gpu.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(L, n), n
    assert names == set(gpu.EXPORTS)


def test_section_formulas():
    A, I11, I22, I12, It, I33 = section_rectangle(0.1, 0.1)
    assert abs(A - 0.01) < 1e-15 and abs(I11 - 0.1 ** 4 / 12) < 1e-18
    # square: Saint-Venant torsion constant 0.1406 b^4
    assert abs(It / 0.1 ** 4 - 0.1406) < 2e-4
    A, I11, I22, I12, It, I33 = section_tube(0.4, 0.34)
    assert abs(It - 2 * I11) < 1e-15 and abs(I33 - It) < 1e-18


def test_generators_are_seeded():
    a = configs.batched_static(16, seed=3)
    b = configs.batched_static(16, seed=3)
    c = configs.batched_static(16, seed=4)
    assert [len(s.beams) for s in a] == [len(s.beams) for s in b]
    assert [len(s.beams) for s in a] != [len(s.beams) for s in c]
    ne = np.array([len(s.beams) for s in configs.batched_static(512, seed=0)])
    assert ne.min() >= 50 and ne.max() <= 2000


def test_rollup_20_element_shape():
    s = configs.cantilever_rollup()
    assert s.n_nodes == 41 and len(s.beams) == 20
    assert s.n_nodes * 6 == 246 and s.n_free == 240


def test_deck_roundtrip_keywords():
    txt = configs.tutorial01().to_inp()
    for kw in ("SolutionSteps", "Nodes\t11", "Elements\t5", "Beam_1", "Hooke", "Rectangle", "CoordinateSystems",
               "NodeSets", "NodalLoad", "NodalConstraint", "ConvergenceCriteria"):
        assert kw in txt
    assert "np.float64" not in txt


def test_reference_loop_driver_compiles_against_the_header(tmp_path):
    """The C++ Static::Solve loop that drives the Newton-iteration boundary
    (tests/iteration_abi/static_loop.cpp) compiles against include/ alone:
    the boundary is plain C, usable from the reference's C++."""
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = os.path.join(ROOT, "tests", "iteration_abi", "static_loop.cpp")
    subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src],
                   check=True)
