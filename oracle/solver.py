"""FP64 CPU oracle of S-PGO's stereo inverse-depth LM step (test infrastructure).

ORACLE — test infrastructure only.  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg import this module, and only as a checker
or as the timed CPU baseline.  The product path never calls into it.

What it restates (citations are paths inside the S-PGO project):

* pose chain  G[0] = I, G[k+1] = G[k] inv(T_k); right camera G_r = G T_r_to_l
  (``src/Optimization/Solver_cuda.cu:440-493``, ``PythonUtils/Optimizer.py:118-131``);
* inverse-depth point  t_a = K_l^-1 p_a / alpha, p_a the left pixel in the
  anchor frame (``Solver_cuda.cu:146-157``, ``Optimizer.py:170-181``);
* residual r = z - pi(K t_n), per camera 2 rows (``Solver_cuda.cu:159-176``,
  ``:231-237``; ``Optimizer.py:340-352``);
* pose Jacobian for every incremental pose i in [a, n):
  s * dpi/dt_n * R_{i->n} [-[t_i]x, I]   (``src/Optimization/LMutils.cu:552-582``,
  ``Solver_cuda.cu:248-290``, ``Optimizer.py:669-748``, ``:809-818``).  Targets
  before the anchor (n < a) get the mirrored range [n, a) with s = -1; the
  reference GPU kernel only fills n >= a (``Solver_cuda.cu:248``);
* inverse-depth Jacobian dpi/dt_n R_{a->n} (-t_a / alpha)
  (``Solver_cuda.cu:197-211``, ``Optimizer.py:751-784``);
* robust IRLS weight: Cauchy sqrt(1/(1+|r|^2/c^2)) (``Solver_cuda.cu:214-222``,
  ``Optimizer.py:351-352``), the x4 near-frame factor of the GPU kernel
  (``Solver_cuda.cu:224-228``), Huber (new);
* normal equations A = J_T^T J_T, B = J_T^T J_a, C = diag(J_a^T J_a), g_T, g_a
  (``Optimizer.py:235-240``, ``:376-383``) and the Schur solve
  S = A - B C^-1 B^T, delta_a = C^-1 (g_a - B^T delta) (``Optimizer.py:242-265``,
  ``Solver_cuda.cu:690-753``);
* update T_k <- T_k Exp(delta_k), alpha <- clamp(alpha + delta_a)
  (``Solver_cuda.cu:497-553``, ``Optimizer.py:645-667``).

Two reference step variants are restated exactly (``reference_gn_step`` for the
GPU ``updateState`` loop, ``reference_cpu_step`` for ``Optimizer.step``), and a
Nielsen Levenberg-Marquardt driver (new: the reference has no damping schedule)
is layered on the same linearisation.

A problem is any object with the attributes
``n_poses, intrinsics[8], T_rl[4,4], host[L], anchor_uv[L,2], obs_ptr[L+1],
obs_frame[O], obs_uv[O,4] (uL, vL, uR, vR), poses[N,4,4], alpha[L]``.
Observation rows are ordered (landmark, observation, camera L/R, x/y).
"""
from __future__ import annotations

import dataclasses
import numpy as np

from . import lie

LOSS_L2, LOSS_CAUCHY, LOSS_HUBER = 0, 1, 2


@dataclasses.dataclass
class Loss:
    kind: int = LOSS_L2
    scale: float = 3.0          # Cauchy c (c^2 = 9 in the GPU kernel) or Huber delta
    near_boost: bool = False    # x4 weight when |target - anchor| < 2 (Solver_cuda.cu:226-228)

    def weight2_and_rho(self, s, n, a):
        """Return (w^2, rho(s)) per camera residual; s = |r|^2.

        The IRLS weight w multiplies both residual and Jacobian, so w^2 is the
        derivative rho'(s) of the robust cost times the near-frame factor.
        """
        s = np.asarray(s, dtype=np.float64)
        if self.kind == LOSS_L2:
            w2 = np.ones_like(s)
            rho = s.copy()
        elif self.kind == LOSS_CAUCHY:
            c2 = self.scale * self.scale
            w2 = 1.0 / (1.0 + s / c2)
            rho = c2 * np.log1p(s / c2)
        elif self.kind == LOSS_HUBER:
            d = self.scale
            rs = np.sqrt(s)
            inl = rs <= d
            w2 = np.where(inl, 1.0, d / np.maximum(rs, 1e-300))
            rho = np.where(inl, s, 2.0 * d * rs - d * d)
        else:
            raise ValueError(self.kind)
        if self.near_boost:
            beta = np.where(np.abs(np.asarray(n) - np.asarray(a)) < 2, 16.0, 1.0)
            w2 = w2 * beta
            rho = rho * beta
        return w2, rho


REFERENCE_GPU_LOSS = Loss(LOSS_CAUCHY, 3.0, True)      # Solver_cuda.cu:214-228, LMutils.h:48
REFERENCE_CPU_LOSS = Loss(LOSS_CAUCHY, 3.0, False)     # Optimizer.py:351-352


def K_matrices(intr):
    intr = np.asarray(intr, dtype=np.float64).reshape(8)
    Kl = np.array([[intr[0], 0, intr[2]], [0, intr[1], intr[3]], [0, 0, 1.0]])
    Kr = np.array([[intr[4], 0, intr[6]], [0, intr[5], intr[7]], [0, 0, 1.0]])
    return Kl, Kr


def global_poses(poses):
    """G[0] = I, G[k+1] = G[k] inv(T_k)  (Solver_cuda.cu:472-491)."""
    poses = np.asarray(poses, dtype=np.float64)
    G = np.zeros((poses.shape[0] + 1, 4, 4))
    G[0] = np.eye(4)
    for k in range(poses.shape[0]):
        G[k + 1] = G[k] @ np.linalg.inv(poses[k])
    return G


def _expand(prob):
    """Per-observation landmark / anchor / target arrays."""
    L = len(prob.host)
    counts = np.diff(np.asarray(prob.obs_ptr))
    lm = np.repeat(np.arange(L), counts)
    a = np.asarray(prob.host)[lm].astype(np.int64)
    n = np.asarray(prob.obs_frame).astype(np.int64)
    return lm, a, n


@dataclasses.dataclass
class Linearization:
    r: np.ndarray          # (4O,) weighted residual rows (landmark, obs, cam, xy)
    J_T: np.ndarray        # (4O, 6N) weighted pose Jacobian (dense) or None
    j_a: np.ndarray        # (4O,) weighted inverse-depth Jacobian (column = landmark)
    row_lm: np.ndarray     # (4O,) landmark of each row
    A: np.ndarray          # (6N, 6N)
    B: np.ndarray          # (6N, L)
    C: np.ndarray          # (L,)
    g_T: np.ndarray        # (6N,)
    g_a: np.ndarray        # (L,)
    cost: float            # 0.5 * sum beta * rho(|r|^2) over camera residuals
    raw_r: np.ndarray      # (4O,) unweighted residuals


def _camera_terms(prob, G, lm, a, n):
    """Unweighted residual, dpi/dt_n, t_n, R_{a->n}, t_a for each (obs, cam)."""
    Kl, Kr = K_matrices(prob.intrinsics)
    Kl_inv = np.linalg.inv(Kl)
    T_rl = np.asarray(prob.T_rl, dtype=np.float64)
    alpha = np.asarray(prob.alpha, dtype=np.float64)[lm]
    uv = np.asarray(prob.anchor_uv, dtype=np.float64)[lm]
    pa = np.stack([uv[:, 0], uv[:, 1], np.ones(len(lm))], -1)
    t_a = (pa @ Kl_inv.T) / alpha[:, None]
    out = []
    for cam, K in ((0, Kl), (1, Kr)):
        Gn = G[n] if cam == 0 else G[n] @ T_rl
        T_an = lie.inv_se3(Gn) @ G[a]
        R_an = T_an[:, :3, :3]
        t_n = np.einsum('oij,oj->oi', R_an, t_a) + T_an[:, :3, 3]
        x, y, z = t_n[:, 0], t_n[:, 1], t_n[:, 2]
        proj = np.stack([K[0, 0] * x / z + K[0, 2], K[1, 1] * y / z + K[1, 2]], -1)
        zobs = np.asarray(prob.obs_uv, dtype=np.float64)[:, 2 * cam:2 * cam + 2]
        res = zobs - proj
        Jp = np.zeros((len(lm), 2, 3))
        Jp[:, 0, 0] = K[0, 0] / z
        Jp[:, 0, 2] = -K[0, 0] * x / (z * z)
        Jp[:, 1, 1] = K[1, 1] / z
        Jp[:, 1, 2] = -K[1, 1] * y / (z * z)
        out.append((res, Jp, Gn, R_an))
    return t_a, alpha, out


def linearize(prob, loss: Loss, dense_JT=True, chunk_rows=1 << 16):
    """Weighted residuals, Jacobians, normal-equation blocks and cost at prob's state."""
    N = int(prob.n_poses)
    L = len(prob.host)
    P = 6 * N
    G = global_poses(prob.poses)
    lm, a, n = _expand(prob)
    O = len(lm)
    t_a, alpha, cams = _camera_terms(prob, G, lm, a, n)
    lo = np.minimum(a, n)
    hi = np.maximum(a, n)
    sgn = np.where(n > a, 1.0, -1.0)
    Ginv = lie.inv_se3(G)

    r = np.zeros((O, 2, 2))       # obs, cam, xy
    raw = np.zeros((O, 2, 2))
    ja = np.zeros((O, 2, 2))
    w_all = np.zeros((O, 2))
    cost = 0.0
    for cam, (res, Jp, Gn, R_an) in enumerate(cams):
        s = np.sum(res * res, -1)
        w2, rho = loss.weight2_and_rho(s, n, a)
        w = np.sqrt(w2)
        w_all[:, cam] = w
        cost += 0.5 * float(np.sum(rho))
        raw[:, cam] = res
        r[:, cam] = w[:, None] * res
        dta = -t_a / alpha[:, None]
        ja[:, cam] = w[:, None] * np.einsum('oij,ojk,ok->oi', Jp, R_an, dta)

    # pose Jacobian blocks: for each incremental pose i, the observations whose
    # range [lo, hi) contains i (LMutils.cu:552-582 / Optimizer.py:809-818)
    JT = np.zeros((O, 2, 2, P)) if dense_JT else None
    A = np.zeros((P, P))
    g_T = np.zeros(P)
    B = np.zeros((P, L))
    Gn_list = [cams[0][2], cams[1][2]]
    for i in range(N):
        m = (lo <= i) & (i < hi)
        if not np.any(m):
            continue
        idx = np.nonzero(m)[0]
        # point in frame i (homogeneous): inv(G_i) G_a t_a
        T_ai = Ginv[i] @ G[a[idx]]
        t_i = np.einsum('oij,oj->oi', T_ai[:, :3, :3], t_a[idx]) + T_ai[:, :3, 3]
        St = lie.skew_batch(t_i)
        for cam in range(2):
            Gn = Gn_list[cam][idx]
            R_in = np.einsum('oji,jk->oik', Gn[:, :3, :3], G[i, :3, :3])   # R_n^T R_i
            D = np.concatenate([-R_in @ St, R_in], -1)                     # (o,3,6)
            Jb = np.einsum('oij,ojk->oik', cams[cam][1][idx], D)          # (o,2,6)
            Jb *= (sgn[idx] * w_all[idx, cam])[:, None, None]
            if dense_JT:
                JT[idx, cam, :, 6 * i:6 * i + 6] = Jb
            else:
                raise NotImplementedError
    JT2 = JT.reshape(O * 4, P)
    rr = r.reshape(O * 4)
    jj = ja.reshape(O * 4)
    row_lm = np.repeat(lm, 4)
    for s0 in range(0, O * 4, chunk_rows):
        s1 = min(O * 4, s0 + chunk_rows)
        Jc = JT2[s0:s1]
        A += Jc.T @ Jc
        g_T += Jc.T @ rr[s0:s1]
    C = np.bincount(row_lm, weights=jj * jj, minlength=L)
    g_a = np.bincount(row_lm, weights=jj * rr, minlength=L)
    # B[:, l] = sum over rows of l of J_T[row] * j_a[row]
    Wrows = JT2 * jj[:, None]
    order_starts = np.asarray(prob.obs_ptr)[:-1] * 4
    nonempty = np.diff(np.asarray(prob.obs_ptr)) > 0
    if O > 0:
        sums = np.add.reduceat(Wrows, order_starts[nonempty], axis=0)
        B[:, np.nonzero(nonempty)[0]] = sums.T
    return Linearization(rr, JT2, jj, row_lm, A, B, C, g_T, g_a, cost, raw.reshape(O * 4))


def cost(prob, loss: Loss):
    """0.5 * sum beta * rho(|r|^2) over all camera residuals (FP64)."""
    G = global_poses(prob.poses)
    lm, a, n = _expand(prob)
    _, _, cams = _camera_terms(prob, G, lm, a, n)
    tot = 0.0
    for res, *_ in cams:
        _, rho = loss.weight2_and_rho(np.sum(res * res, -1), n, a)
        tot += 0.5 * float(np.sum(rho))
    return tot


@dataclasses.dataclass
class Step:
    delta: np.ndarray      # (6N,)
    delta_a: np.ndarray    # (L,)
    pred: float            # predicted cost reduction of the damped model
    ok: bool               # factorisation succeeded


def solve_damped(lin: Linearization, lam: float, eps: float = 1e-4):
    """Schur solve of (H + Lambda) [d; da] = [g_T; g_a].

    Lambda = lam * diag(A) on poses and lam * C + eps on inverse depths
    (Marquardt scaling; eps is the reference's ``_eps`` guard, LMutils.h:50).
    With lam = 0 this is exactly the reference GPU step (Solver_cuda.cu:690-753).
    """
    A, B, C = lin.A, lin.B, lin.C
    lp = lam * np.diag(A)
    D = C * (1.0 + lam) + eps
    la = D - C
    BD = B / D[None, :]
    S = A + np.diag(lp) - BD @ B.T
    gS = lin.g_T - BD @ lin.g_a
    try:
        Lc = np.linalg.cholesky(S)
        y = np.linalg.solve(Lc, gS)
        d = np.linalg.solve(Lc.T, y)
        ok = bool(np.all(np.isfinite(d)))
    except np.linalg.LinAlgError:
        d = np.zeros_like(gS)
        ok = False
    da = (lin.g_a - B.T @ d) / D
    pred = 0.5 * (d @ (lin.g_T + lp * d) + da @ (lin.g_a + la * da))
    return Step(d, da, float(pred), ok)


def apply_update(poses, alpha, delta, delta_a, pose_scale=1.0,
                 alpha_min=1.0 / 30.0, alpha_max=1.0 / 0.2):
    """T_k <- T_k Exp(s * delta_k); alpha <- clamp(alpha + delta_a) (Solver_cuda.cu:511-551)."""
    poses = np.asarray(poses, dtype=np.float64)
    new_p = np.empty_like(poses)
    for k in range(poses.shape[0]):
        new_p[k] = poses[k] @ lie.exp_se3(pose_scale * delta[6 * k:6 * k + 6])
    new_a = np.clip(np.asarray(alpha, dtype=np.float64) + delta_a, alpha_min, alpha_max)
    return new_p, new_a


def reference_gn_step(prob, iterations=1, step_size=1.0, loss: Loss = REFERENCE_GPU_LOSS):
    """The reference GPU ``updateState`` loop (Solver_cuda.cu:557-795), in FP64.

    Undamped Gauss-Newton with C + eps (eps = 1e-4), a pose-only step size,
    the unscaled clamped inverse-depth update and the Cauchy c^2 = 9 weight
    with the x4 near-frame factor.  Mutates and returns ``prob``.
    """
    for _ in range(iterations):
        lin = linearize(prob, loss)
        st = solve_damped(lin, 0.0, 1e-4)
        prob.poses, prob.alpha = apply_update(prob.poses, prob.alpha, st.delta, st.delta_a,
                                              pose_scale=step_size)
    return prob


@dataclasses.dataclass
class LMResult:
    cost0: float
    cost: float
    iterations: int
    accepted: int
    converged: bool
    trace: list


def lm_solve(prob, loss: Loss = Loss(), max_iters=20, tol=1e-6, lam0=1e-4, eps=1e-4,
             alpha_min=1.0 / 30.0, alpha_max=1.0 / 0.2, lam_max=1e16, stop_rho=0.0):
    """Nielsen-damped Levenberg-Marquardt (new; the reference has no schedule).

    Marquardt scaling (see ``solve_damped``); gain ratio rho = (F - F') / pred.
    rho > 0: accept, lam *= max(1/3, 1 - (2 rho - 1)^3), nu = 2;
    otherwise reject, lam *= nu, nu *= 2.  Stops when an accepted step lowers
    the cost by less than ``tol`` relative with rho >= ``stop_rho``, a predicted
    decrease below ``tol`` relative, or an accepted step before it that was also
    below ``tol`` (default stop_rho 0: any accepted step), or after ``max_iters``
    solves (accepted + rejected).
    Mutates ``prob`` and returns an ``LMResult``.
    """
    lam, nu = lam0, 2.0
    lin = linearize(prob, loss)
    F = lin.cost
    F0 = F
    it = acc = 0
    converged = False
    small_prev = False
    trace = []
    while it < max_iters:
        st = solve_damped(lin, lam, eps)
        it += 1
        newp, newa = apply_update(prob.poses, prob.alpha, st.delta, st.delta_a, 1.0,
                                  alpha_min, alpha_max)
        old = (prob.poses, prob.alpha)
        prob.poses, prob.alpha = newp, newa
        Fn = cost(prob, loss) if st.ok else np.inf
        rho = (F - Fn) / st.pred if (st.ok and st.pred > 0) else -1.0
        trace.append(dict(it=it, cost=F, cand=Fn, pred=st.pred, rho=rho, lam=lam))
        if np.isfinite(Fn) and rho > 0:
            acc += 1
            rel = (F - Fn) / max(F, 1e-300)
            pred_rel = st.pred / max(F, 1e-300)
            F = Fn
            lam *= max(1.0 / 3.0, 1.0 - (2.0 * rho - 1.0) ** 3)
            nu = 2.0
            if rel < tol and (rho >= stop_rho or pred_rel < tol or small_prev):
                converged = True
                break
            small_prev = rel < tol
            lin = linearize(prob, loss)
        else:
            prob.poses, prob.alpha = old
            lam *= nu
            nu *= 2.0
            if lam > lam_max:
                converged = True
                break
    return LMResult(F0, F, it, acc, converged, trace)


# ---------------------------------------------------------------------------
# Restatement of the reference CPU step ``Optimizer.step`` (Optimizer.py:135-289)
# on the reference's own scene layout: every landmark l is anchored at
# map_value_to_index(l, L, N) (Optimizer.py:12-18) and observed in every frame
# n >= anchor, left and right.
# ---------------------------------------------------------------------------

def map_value_to_index(v, x, n):
    """Optimizer.py:12-18."""
    vc = max(0, min(v, x))
    return min(int((vc / x) * n), n - 1)


class ReferenceCPUStepper:
    """State of ``Optimizer`` that survives between ``step`` calls (step size, prev norm)."""

    def __init__(self, width=640, height=512, min_alpha=1.0 / 20.0, max_alpha=1.0 / 0.01):
        self.width, self.height = width, height
        self.min_alpha, self.max_alpha = min_alpha, max_alpha
        self.step_size = 1.0
        self.prev_norm = 1e10

    def step(self, prob):
        """One ``Optimizer.step``: masked Cauchy(c=1) weights, zeroed left-anchor
        depth Jacobian, C + 2e-3, S + I, adaptive step size.  ``prob`` must hold
        the reference's full observation set ordered by (landmark, frame)."""
        N = int(prob.n_poses)
        L = len(prob.host)
        G = global_poses(prob.poses)
        lm, a, n = _expand(prob)
        t_a, alpha, cams = _camera_terms(prob, G, lm, a, n)
        O = len(lm)
        P = 6 * N
        # row order of Optimizer.step: landmark, camera, frame, xy  (Optimizer.py:183-184)
        J_T = np.zeros((O, 2, 2, P))
        ja = np.zeros((O, 2, 2))
        r = np.zeros((O, 2, 2))
        Ginv = lie.inv_se3(G)
        for cam, (res, Jp, Gn, R_an) in enumerate(cams):
            zobs = np.asarray(prob.obs_uv)[:, 2 * cam:2 * cam + 2]
            inside = ~((zobs[:, 0] < 0) | (zobs[:, 1] < 0) | (zobs[:, 0] > self.width)
                       | (zobs[:, 1] > self.height))
            wmask = inside.astype(np.float64)
            nrm2 = np.sum(res * res, -1)
            sw = np.sqrt(1.0 / (1.0 + nrm2)) * wmask
            r[:, cam] = sw[:, None] * res
            jj = np.einsum('oij,ojk,ok->oi', Jp, R_an, -t_a / alpha[:, None])
            if cam == 0:
                jj[n == a] = 0.0
            ja[:, cam] = sw[:, None] * jj
            for i in range(N):
                idx = np.nonzero((a <= i) & (i < n))[0]
                if len(idx) == 0:
                    continue
                T_ai = Ginv[i] @ G[a[idx]]
                t_i = np.einsum('oij,oj->oi', T_ai[:, :3, :3], t_a[idx]) + T_ai[:, :3, 3]
                R_in = np.einsum('oji,jk->oik', Gn[idx, :3, :3], G[i, :3, :3])
                D = np.concatenate([-R_in @ lie.skew_batch(t_i), R_in], -1)
                J_T[idx, cam, :, 6 * i:6 * i + 6] = sw[idx, None, None] * np.einsum(
                    'oij,ojk->oik', Jp[idx], D)
        JT = J_T.reshape(-1, P)
        rr = r.reshape(-1)
        jj = ja.reshape(-1)
        row_lm = np.repeat(lm, 4)
        A = JT.T @ JT
        g_T = JT.T @ rr
        C = np.bincount(row_lm, weights=jj * jj, minlength=L) + 2e-3
        g_a = np.bincount(row_lm, weights=jj * rr, minlength=L)
        B = np.zeros((P, L))
        np.add.at(B.T, row_lm, JT * jj[:, None])
        Cinv = 1.0 / C
        BC = B * Cinv[None, :]
        H = A - BC @ B.T + np.eye(P)
        g = g_T - BC @ g_a
        d = np.linalg.solve(H, g)
        da = Cinv * (g_a - B.T @ d)
        r_norm = float(np.linalg.norm(rr))
        if self.prev_norm > r_norm:
            self.step_size *= 1.01
        elif self.prev_norm < r_norm:
            self.step_size *= 0.9
        self.step_size = min(max(self.step_size, 0.02), 10.0)
        self.prev_norm = r_norm
        new_p = np.empty_like(np.asarray(prob.poses, dtype=np.float64))
        for k in range(N):
            new_p[k] = prob.poses[k] @ lie.exp_se3(self.step_size * d[6 * k:6 * k + 6])
        prob.poses = new_p
        prob.alpha = np.clip(np.asarray(prob.alpha) + self.step_size * da,
                             self.min_alpha, self.max_alpha)
        return dict(r=rr, A=A, g_T=g_T, B=B, C=C, g_a=g_a)
