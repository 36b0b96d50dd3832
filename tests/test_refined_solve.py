"""The reduced-camera solve's precision scheme, checked on the CPU (numpy / LAPACK,
no GPU): an FP32 Cholesky factor and one refinement step whose residual is formed
with FP64-grade accuracy.

k_factor_solve<float> and the multi-CTA path (csrc/k_solve.cu, csrc/k_chol_large.cu)
factor S = A + lam diag(A) - S_L in FP32, solve, form r = g_S - S x in double-float
from A and S_L, and solve once more with the same factor (the reference runs a plain
FP32 libtorch Cholesky, src/Optimization/linear_solvers.cu:195-218).  Here LAPACK's
FP32 Cholesky stands in for the kernels' blocked one and FP64 for the double-float
residual; the damped reduced system is the oracle's own (Optimizer.py:235-265).
"""
import numpy as np
import pytest
import scipy.linalg as sla

import spgo_gb300.scenes as scenes
from oracle import solver as S

f32 = np.float32


def reduced_system(p, lam, eps=1e-4):
    lin = S.linearize(p, S.Loss())
    D = lin.C * (1.0 + lam) + eps
    BD = lin.B / D[None, :]
    Sm = lin.A + np.diag(lam * np.diag(lin.A)) - BD @ lin.B.T
    gS = lin.g_T - BD @ lin.g_a
    return Sm, gS


@pytest.mark.parametrize("n_poses,lam", [(8, 1e-4), (20, 1e-4), (20, 1e-2)])
def test_fp32_factor_with_one_refinement_step(n_poses, lam):
    p = scenes.circle_scene(40 + n_poses, n_poses, 40 * n_poses)
    Sm, gS = reduced_system(p, lam)
    x64 = np.linalg.solve(Sm, gS)
    fac = sla.cho_factor(Sm.astype(f32), lower=True)            # FP32 factor
    assert fac[0].dtype == f32
    x0 = sla.cho_solve(fac, gS.astype(f32)).astype(np.float64)
    r = gS - Sm @ x0                                             # residual at FP64 grade
    x1 = x0 + sla.cho_solve(fac, r.astype(f32)).astype(np.float64)
    e0 = np.linalg.norm(x0 - x64) / np.linalg.norm(x64)
    e1 = np.linalg.norm(x1 - x64) / np.linalg.norm(x64)
    kappa = np.linalg.cond(Sm)
    # one step takes the FP32 error e0 ~ kappa 2^-24 down by about that factor again
    assert e1 < max(10 * e0 * kappa * 2.0 ** -24, 1e-12)
    assert e1 < 1e-2 * e0 or e0 < 1e-9
    # the predicted decrease the gain ratio divides by comes out FP64-accurate
    pred64 = x64 @ gS
    assert abs(x1 @ gS - pred64) / abs(pred64) < 1e-8
