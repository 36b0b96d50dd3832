"""The FP64 oracle against golden vectors produced by the reference's own CPU
solver (``PythonUtils/Optimizer.py`` via ``tests/golden/make_golden.py``)."""
import os
import types

import numpy as np
import pytest

from oracle import lie
from oracle import solver as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NAMES = ["ref_small", "ref_medium"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = types.SimpleNamespace(**{k: z[k] for k in ["intrinsics", "T_rl", "host", "anchor_uv", "obs_ptr",
                                                   "obs_frame", "obs_uv", "poses", "alpha"]})
    p.n_poses = int(z["n_poses"])
    return p, z


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_jacobians_and_residual_match_reference(name):
    """getJacobiansAndResidual (Optimizer.py:291-373): same rows, same values."""
    p, z = load(name)
    lin = S.linearize(p, S.REFERENCE_CPU_LOSS)
    R = len(lin.r)
    assert np.abs(lin.r - z["ref_r"][:R]).max() < 1e-10
    assert np.all(z["ref_r"][R:] == 0)                      # unused rows stay zero in the reference
    assert rel(lin.J_T, z["ref_J_T"][:R]) < 1e-12
    assert rel(lin.j_a, z["ref_j_alpha"][:R]) < 1e-12
    assert np.all(z["ref_j_alpha_col"][:R] == lin.row_lm)


@pytest.mark.parametrize("name", NAMES)
def test_hessians_match_reference(name):
    """getHessians (Optimizer.py:376-383): H_TT, g_TT, diag(H_aa), g_aa, BB."""
    p, z = load(name)
    lin = S.linearize(p, S.REFERENCE_CPU_LOSS)
    assert rel(lin.A, z["ref_H_TT"]) < 1e-12
    assert rel(lin.g_T, z["ref_g_TT"]) < 1e-12
    assert rel(lin.C, z["ref_H_aa_diag"]) < 1e-12
    assert rel(lin.g_a, z["ref_g_aa"]) < 1e-12
    assert rel(lin.B, z["ref_BB"]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_cpu_step_matches_reference(name):
    """Two consecutive Optimizer.step calls (Optimizer.py:135-289)."""
    p, z = load(name)
    st = S.ReferenceCPUStepper()
    for k in range(2):
        st.step(p)
        assert np.abs(p.poses - z["ref_step_poses"][k]).max() < 1e-10
        assert np.abs(p.alpha - z["ref_step_alpha"][k]).max() < 1e-10


@pytest.mark.parametrize("name", NAMES)
def test_lie_matches_reference(name):
    """LieUtils.Exp_SE3 / J_l_SO3 / J_l_inv_SO3 (LieUtils.py:73-109)."""
    _, z = load(name)
    for i, xi in enumerate(z["lie_xi"]):
        assert np.abs(lie.exp_se3(xi) - z["ref_exp_se3"][i]).max() < 1e-12
        # the reference evaluates the closed form even at |psi| ~ 1e-6 (cancellation ~1e-11)
        assert np.abs(lie.left_jacobian_so3(xi[:3]) - z["ref_jl"][i]).max() < 1e-9
        assert np.abs(lie.inv_left_jacobian_so3(xi[:3]) - z["ref_jl_inv"][i]).max() < 1e-9
