"""No CPU fallback. Without the built library the Python mirror refuses to
load, and on a machine without a usable CUDA device the library refuses to
create a handle (WBEM_ERR_CUDA). Neither computes anything on the host."""
import os

import pytest

import wavebem_gb300.bem_problem as B
from wavebem_gb300 import meshes as M


def test_missing_library_is_an_error(monkeypatch, tmp_path):
    monkeypatch.setattr(B, "_lib", None)  # no cached handle to the real library
    with pytest.raises(ImportError):
        B.load_library(str(tmp_path / "libwbem.so"))


def test_no_handle_without_a_cuda_device():
    from wavebem_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    m = M.wigley_mesh(600)
    try:
        g = B.BEMProblem(m.X, m.cells, m.dirichlet)
    except B.WBEMError as e:
        assert B.STATUS[e.code] == "ERR_CUDA"
        return
    g.close()
    pytest.skip("a CUDA device is present: the library runs on it")
