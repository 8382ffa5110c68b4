"""Time-loop stand-in (BDF + Jacobian-free Newton-GMRES over the BEM's
Dirichlet-to-Neumann map): a few steps run, Newton converges, and the mixed
and FP64 forms give the same trajectory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_timeloop_mixed_matches_fp64_few_steps():
    from wavebem_gb300.bem_problem import PREC_FP64, PREC_MIXED
    from wavebem_gb300.timeloop import FreeSurfaceStandIn
    r64 = FreeSurfaceStandIn(1200, precision=PREC_FP64).run(steps=4, dt=0.01)
    rmx = FreeSurfaceStandIn(1200, precision=PREC_MIXED).run(steps=4, dt=0.01)
    assert r64["assemblies"] >= 4 and r64["solves"] > r64["assemblies"]
    assert np.isfinite(r64["final_Fx"]) and r64["max_eta"] > 0
    # Newton converged on every step, in both forms
    assert r64["newton_residual_max"] <= 1e-8 and rmx["newton_residual_max"] <= 1e-8
    # same trajectory: each BEM solve agrees to ~1e-9, four steps amplify little
    ym, y64 = rmx["final_state"], r64["final_state"]
    assert np.linalg.norm(ym - y64) <= 1e-6 * np.linalg.norm(y64)
    assert abs(rmx["final_Fx"] - r64["final_Fx"]) <= 1e-5 * abs(r64["final_Fx"])
