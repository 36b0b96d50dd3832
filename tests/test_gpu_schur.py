"""Damped reduced camera system S = A + lam diag(A) - B D^-1 B^T and g_S from the
CUDA path (SIMT and tensor-core Schur complements) against the FP64 oracle.

S cancels most of A (on the 45-pose problem below max|A| / max|S| is ~600), so
errors are stated relative to the largest entry of A (and of g_T for g_S), the
scale the FP32 terms are formed at: FP64 path 1e-10; mixed path with the SIMT
FP32 Schur 2e-6; mixed path with the tensor-core Schur (split TF32 operands,
hi.hi + hi.lo + lo.hi, ~21-bit products, TMEM read back every 4 chunks into
FP32 registers) 2e-6."""
import numpy as np
import pytest

import spgo_gb300.scenes as scenes
from spgo_gb300.solver import BatchSolver
from oracle import solver as S

pytestmark = pytest.mark.gpu


def f32_obs(p):
    q = p.copy()
    q.obs_uv = p.obs_uv.astype(np.float32).astype(np.float64)
    q.anchor_uv = p.anchor_uv.astype(np.float32).astype(np.float64)
    q.intrinsics = p.intrinsics.astype(np.float32).astype(np.float64)
    return q


def oracle_reduced(p, lam, eps=1e-4):
    lin = S.linearize(f32_obs(p), S.Loss())
    D = lin.C * (1.0 + lam) + eps
    BD = lin.B / D[None, :]
    Sm = lin.A + np.diag(lam * np.diag(lin.A)) - BD @ lin.B.T
    return Sm, lin.g_T - BD @ lin.g_a, lin


@pytest.mark.parametrize("prec,use_tc,tol", [("fp64", 0, 1e-10), ("mixed", 0, 2e-6), ("mixed", 1, 2e-6)])
def test_reduced_system_matches_oracle(built_lib, cuda_device, prec, use_tc, tol):
    # sizes that exercise one, two and three 128-row tensor-core tiles (P = 54, 156, 84, 270)
    # and off-diagonal tiles with partial column ranges
    probs = [scenes.circle_scene(s, n, l) for s, n, l in
             [(301, 9, 240), (302, 26, 700), (303, 14, 380), (304, 45, 1200)]]
    bs = BatchSolver(probs, precision=prec)
    bs.set_params(loss="l2", use_tc=use_tc)
    for lam in (1e-4, 0.5):
        for b, p in enumerate(probs):
            got = bs.export_reduced(b, lam)
            Sm, gS, lin = oracle_reduced(p, lam)
            assert np.abs(got["S"] - Sm).max() / np.abs(lin.A).max() < tol, (b, lam)
            assert np.abs(got["gS"] - gS).max() / np.abs(lin.g_T).max() < tol, (b, lam)


def test_tensor_core_solve_converges(built_lib, cuda_device):
    """LM with the tensor-core Schur reaches the oracle's converged cost."""
    probs = [scenes.circle_scene(s, n, l) for s, n, l in [(200, 8, 500), (205, 18, 455), (214, 31, 234)]]
    bs = BatchSolver([f32_obs(p) for p in probs], precision="mixed")
    bs.set_params(loss="l2", max_iters=30, tol=1e-6, use_tc=1)
    sts = bs.solve()
    for b, p in enumerate(probs):
        res = S.lm_solve(f32_obs(p), S.Loss(), max_iters=30, tol=1e-6)
        assert abs(sts[b]["cost"] - res.cost) / res.cost < 1e-6


def test_autotune_picks_valid_shapes_and_restores_state(built_lib, cuda_device):
    """The autotuner returns shapes from its candidate sets, leaves the poses and
    inverse depths untouched, and the tuned solve reaches the untuned cost."""
    # problems that converge to their optimum (on a problem crawling in a poor local
    # minimum, a different summation order legitimately changes the endpoint)
    probs = [scenes.circle_scene(s, n, l) for s, n, l in [(200, 8, 500), (205, 18, 455), (214, 31, 234)]]
    bs = BatchSolver(probs, precision="mixed")
    bs.set_params(loss="l2", max_iters=30, tol=1e-6)
    base = [s["cost"] for s in bs.solve()]
    bs.load_state()
    p0, a0 = bs.poses.clone(), bs.alpha.clone()
    tuned = bs.autotune()
    assert tuned["cost_block"] in (64, 128, 256) and tuned["lin_block"] in (128, 256) and tuned["use_tc"] in (0, 1)
    assert bool((bs.poses == p0).all()) and bool((bs.alpha == a0).all())
    after = [s["cost"] for s in bs.solve()]
    for c0, c1 in zip(base, after):
        assert abs(c1 - c0) / c0 < 1e-6


def test_plan_shapes_autotune_and_equal_results(built_lib, cuda_device):
    """The plan-time Schur work shapes (chunks per tensor-core work item) change how
    the products are split into CTAs, not the reduced system: every shape reaches the
    oracle's cost, and autotune_plan_shapes returns one of its candidates without
    touching the solver it was called on."""
    probs = [scenes.circle_scene(s, n, l) for s, n, l in [(200, 8, 500), (205, 18, 455), (214, 31, 234)]]
    ref = [S.lm_solve(f32_obs(p), S.Loss(), max_iters=30, tol=1e-6).cost for p in probs]
    for split in (8, 32, 64):
        bs = BatchSolver([f32_obs(p) for p in probs], precision="mixed", plan_options=dict(tc_split=split))
        assert bs.sizes.tc_split == split
        bs.set_params(loss="l2", max_iters=30, tol=1e-6, use_tc=1)
        for st, c in zip(bs.solve(), ref):
            assert abs(st["cost"] - c) / c < 1e-6, (split, st["cost"], c)
        bs.close()
    bs = BatchSolver([f32_obs(p) for p in probs], precision="mixed")
    bs.set_params(loss="l2", max_iters=30, tol=1e-6, use_tc=1)
    p0, a0 = bs.poses.clone(), bs.alpha.clone()
    out = bs.autotune_plan_shapes(iterations=1, repeats=1)
    assert out["best"]["tc_split"] in (16, 32, 64) and len(out["ms"]) == 3
    assert bool((bs.poses == p0).all()) and bool((bs.alpha == a0).all())
    bs.close()
