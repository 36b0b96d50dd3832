"""Self-checks of the FP64 oracle: Lie identities, finite-difference Jacobians,
LM convergence.  Patterned on the reference's tests (tests/testExpSO3.cpp,
tests/testJacobiansSO3.cpp, PythonUtils/DepthOptimization.py:97-150)."""
import numpy as np
import pytest

import spgo_gb300.scenes as scenes
from oracle import lie
from oracle import solver as S


def norm_mix(rng, n):
    """Rotation-vector norms around the edge cases the reference tests hit:
    0, [1e-10, 1e-8], pi, > pi, and generic (testExpSO3.cpp:43-54)."""
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    norms = np.concatenate([np.zeros(2), rng.uniform(1e-10, 1e-8, 6), np.full(4, np.pi),
                            rng.uniform(np.pi, 2 * np.pi, 8), rng.uniform(0, np.pi, n - 20)])
    return axes * norms[:, None]


def test_exp_log_round_trip():
    rng = np.random.default_rng(0)
    for psi in norm_mix(rng, 200):
        R = lie.exp_so3(psi)
        assert np.abs(R @ R.T - np.eye(3)).max() < 1e-12
        R2 = lie.exp_so3(lie.log_so3(R))
        assert np.abs(R2 - R).max() < 1e-8


def test_left_jacobian_fd():
    """Exp(psi + d) ~ Exp(J_l(psi) d) Exp(psi); inf-norm error < 5e-5 at eps 1e-4
    (testJacobiansSO3.cpp:3-44)."""
    rng = np.random.default_rng(1)
    eps = 1e-4
    for psi in rng.normal(0, 1.0, (100, 3)):
        Jl = lie.left_jacobian_so3(psi)
        R = lie.exp_so3(psi)
        num = np.zeros((3, 3))
        for k in range(3):
            d = np.zeros(3)
            d[k] = eps
            num[:, k] = lie.log_so3(lie.exp_so3(psi + d) @ R.T) / eps
        assert np.abs(num - Jl).max() < 5e-5
        assert np.abs(Jl @ lie.inv_left_jacobian_so3(psi) - np.eye(3)).max() < 5e-5


def test_se3_round_trip():
    rng = np.random.default_rng(2)
    for xi in rng.normal(0, 1.0, (100, 6)):
        T = lie.exp_se3(xi)
        assert np.abs(lie.exp_se3(lie.log_se3(T)) - T).max() < 1e-9


@pytest.mark.parametrize("loss", [S.Loss(), S.REFERENCE_GPU_LOSS, S.Loss(S.LOSS_HUBER, 2.0)])
def test_jacobians_fd(loss):
    """Pose and inverse-depth Jacobians against central differences of the
    unweighted residual (r = z - h, so dr = -J dx)."""
    p = scenes.circle_scene(11, 4, 30)
    lin = S.linearize(p, loss)
    w = np.repeat(np.sqrt(loss.weight2_and_rho(
        np.sum(lin.raw_r.reshape(-1, 2) ** 2, 1),
        np.repeat(p.obs_frame, 2), np.repeat(p.host[np.repeat(np.arange(p.n_landmarks), np.diff(p.obs_ptr))], 2))[0]), 2)
    h = 1e-6
    for k in range(p.n_poses):
        for c in range(6):
            d = np.zeros(6)
            d[c] = h
            q1, q2 = p.copy(), p.copy()
            q1.poses = p.poses.copy(); q2.poses = p.poses.copy()
            q1.poses[k] = p.poses[k] @ lie.exp_se3(d)
            q2.poses[k] = p.poses[k] @ lie.exp_se3(-d)
            r1 = S.linearize(q1, S.Loss()).raw_r
            r2 = S.linearize(q2, S.Loss()).raw_r
            num = -(r1 - r2) / (2 * h) * w
            ana = lin.J_T[:, 6 * k + c]
            assert np.abs(num - ana).max() < 1e-4 * max(1.0, np.abs(ana).max())
    l = 3
    q1, q2 = p.copy(), p.copy()
    q1.alpha = p.alpha.copy(); q2.alpha = p.alpha.copy()
    q1.alpha[l] += h
    q2.alpha[l] -= h
    num = -(S.linearize(q1, S.Loss()).raw_r - S.linearize(q2, S.Loss()).raw_r) / (2 * h) * w
    ana = np.where(lin.row_lm == l, lin.j_a, 0.0)
    assert np.abs(num - ana).max() < 1e-4 * max(1.0, np.abs(ana).max())


def test_lm_converges_config0():
    p = scenes.config0()
    res = S.lm_solve(p, S.Loss(), max_iters=10, tol=1e-6)
    assert res.converged
    costs = [t["cost"] for t in res.trace]
    assert all(b <= a for a, b in zip(costs, costs[1:]))
    assert res.cost < 1e-2 * res.cost0
    lin = S.linearize(p, S.Loss())
    assert np.abs(lin.g_T).max() < 1e-3 * np.abs(S.linearize(scenes.config0(), S.Loss()).g_T).max()


def test_lm_stop_rho_defers_a_poorly_modelled_stop():
    """With a loose tolerance (0.2) the plain rule stops this scene on an accepted step
    whose gain ratio is 0.06; with stop_rho = 0.25 that step no longer ends the solve:
    the solve ends on a step with rho >= 0.25, later and at a lower cost."""
    p = scenes.circle_scene(301, 8, 200)
    r0 = S.lm_solve(p.copy(), S.Loss(), max_iters=30, tol=0.2)
    r1 = S.lm_solve(p.copy(), S.Loss(), max_iters=30, tol=0.2, stop_rho=0.25)
    last0 = [t for t in r0.trace if t["rho"] > 0][-1]
    last1 = [t for t in r1.trace if t["rho"] > 0][-1]
    assert r0.converged and r1.converged
    assert last0["rho"] < 0.25 and (last0["cost"] - last0["cand"]) < 0.2 * last0["cost"]
    assert last1["rho"] >= 0.25 and (last1["cost"] - last1["cand"]) < 0.2 * last1["cost"]
    assert r1.iterations > r0.iterations and r1.cost < r0.cost
    # the two runs agree up to the deferred stop
    assert [t["cand"] for t in r1.trace[:r0.iterations]] == [t["cand"] for t in r0.trace]


def test_reference_gn_step_decreases_cost():
    p = scenes.circle_scene(5, 6, 80)
    c0 = S.cost(p, S.REFERENCE_GPU_LOSS)
    S.reference_gn_step(p, iterations=3, step_size=1.0)
    assert S.cost(p, S.REFERENCE_GPU_LOSS) < 0.1 * c0


def test_mlp_oracle_gradient_fd():
    """The controller network's FP64 reference gradient against central differences."""
    from oracle import mlp as M
    rng = np.random.default_rng(0)
    theta = M.init(seed=2).astype(np.float64)
    X = rng.normal(0.0, 1.0, (7, M.D_IN))
    T = np.stack([rng.normal(0.0, 1.0, 7), rng.integers(0, 2, 7)], 1).astype(np.float64)
    _, g = M.loss_and_grad(theta, X, T)
    idx = rng.choice(M.N_PARAMS, 40, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(theta)
        e[i] = h
        fd = (M.loss_and_grad(theta + e, X, T)[0] - M.loss_and_grad(theta - e, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(g[i]))
