"""Host helpers of the FMA octree (wavebem_gb300/csrc/fma_tree.h), checked on
the CPU: Morton codes and their parent / octant relations, the stable radix
sort, the code-to-box index and the floating-point identity that lets one
sort of the deepest level's codes give every level's boxes."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fma_tree_helpers(tmp_path):
    exe = tmp_path / "fma_tree_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "wavebem_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fma_tree_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
