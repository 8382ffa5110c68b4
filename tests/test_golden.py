"""Regression fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import rel2, relmax

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["wigley300", "sphere6"]


def load(name):
    return dict(np.load(os.path.join(HERE, f"{name}.npz")))


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    g = load(name)
    P = O.Problem(g["X"], g["cells"], g["dn_ptr"], g["dn_idx"], g["dirichlet"])
    P.assemble()
    assert relmax(P.alpha, g["alpha"]) < 1e-13
    assert rel2(P.Nm @ g["v"], g["Nv"]) < 1e-13
    assert rel2(P.Dm @ g["v"], g["Dv"]) < 1e-13
    phi, dphi, _ = P.solve_system(g["b"])
    assert rel2(phi, g["phi"]) < 1e-12 and rel2(dphi, g["dphi"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(name):
    from wavebem_gb300.bem_problem import BEMProblem
    g = load(name)
    bem = BEMProblem(g["X"], g["cells"], g["dirichlet"], g["dn_ptr"], g["dn_idx"])
    bem.assemble_system()
    Nm, Dm = bem.matrices()
    assert relmax(bem.compute_alpha(), g["alpha"]) <= 1e-10
    assert np.abs(Nm[g["ii"], g["jj"]] - g["Nij"]).max() <= 1e-10 * np.abs(Nm).max()
    assert np.abs(Dm[g["ii"], g["jj"]] - g["Dij"]).max() <= 1e-10 * np.abs(Dm).max()
    assert rel2(Nm @ g["v"], g["Nv"]) <= 1e-10 and rel2(Dm @ g["v"], g["Dv"]) <= 1e-10
    phi, dphi = g["b"].copy(), g["b"].copy()
    bem.solve_system(phi, dphi, g["b"])
    assert rel2(phi, g["phi"]) <= 1e-9 and rel2(dphi, g["dphi"]) <= 1e-9
