"""The library's quadrature rules against the oracle's, on the CPU: the
Gauss-Legendre rules on [0, 1] and the vertex-singular rules of the unit
square (the rule of QGaussOneOverR<2>(n, vertex, true),
source/bem_problem.cc:116-120) that the library loads into constant memory
are built by the host code in wavebem_gb300/csrc/quadrature_rules.h; the
oracle restates them independently (oracle/wbem_oracle.cpp). Points and
weights are bitwise equal (the library's rules print with 17 significant
digits, which round-trip doubles exactly)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def library_rules(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    exe = tmp_path_factory.mktemp("quad") / "quadrature_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "wavebem_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "quadrature_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    rules, i = {}, 0
    while i < len(out) and out[i]:
        head = out[i].split()
        n = int(head[1])
        rows = 2 * n * n if head[0] == "S" else n
        key = ("S", n, int(head[2])) if head[0] == "S" else ("G", n)
        rules[key] = np.array([[float(t) for t in out[i + 1 + r].split()] for r in range(rows)])
        i += 1 + rows
    return rules


def test_gauss_rules_match_oracle(library_rules):
    for n in range(1, 9):
        x, w = O.gauss01(n)
        lib = library_rules[("G", n)]
        assert np.array_equal(lib[:, 0], x) and np.array_equal(lib[:, 1], w), n


def test_vertex_singular_rules_match_oracle(library_rules):
    for n in range(1, 9):
        for v in range(4):
            px, py, w = O.singular_rule(n, v)
            lib = library_rules[("S", n, v)]
            assert (np.array_equal(lib[:, 0], px) and np.array_equal(lib[:, 1], py)
                    and np.array_equal(lib[:, 2], w)), (n, v)
