"""The factorised pose Jacobian the CUDA kernels build on, checked on the CPU
against the oracle's dense Jacobian (FP64 numpy, no GPU).

The reference forms a dense pose Jacobian row for every observation and every
incremental pose its anchor-target range covers (src/Optimization/LMutils.cu:552-582,
PythonUtils/Optimizer.py:809-818) and multiplies it out with cuBLAS
(src/Optimization/Solver_cuda.cu:636-668).  The kernels instead use, for an
observation anchored in frame a and seen in frame n,

    J_{o,i} = s_o w_o K_o Ad_i(x),   i in [lo, hi) = [min(a, n), max(a, n)),
    K_o = [ (X - x) x u_k , u_k ]  (rows k = u, v;  u = dpi/dt R_n^T),
    Ad_i(x) = [[R_i, 0], [[c_i - x]x R_i, R_i]],

so the pose blocks are A(i, j) = Ad_i^T F(i, j) Ad_j with F(i, j) the sum of the
per-(lo, hi) records M = sum w^2 K^T K over lo <= i, hi > j, each moved to a common
origin by E_z = [[I, 0], [-[z]x, I]] (M -> E_z^T M E_z).  This file restates that
assembly as the kernels run it (csrc/k_linearize.cu: records about the left centre
of frame lo; csrc/k_system.cu: prefix over lo re-centred step by step onto row i's
centre, suffix over hi, then Ad_i^T F Ad_j about c_i; the mixed path's variant with
one origin per problem) and checks A, g and the pose-depth blocks B against the
oracle's dense products.
"""
import numpy as np
import pytest

import spgo_gb300.scenes as scenes
from oracle import solver as S


def skew(v):
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def E(z):
    """Moves a record from origin x to origin x - z: K^{x - z} = K^x E(z)."""
    e = np.eye(6)
    e[3:, :3] = -skew(z)
    return e


def Ad(R, c, x):
    """World twist about origin x of a perturbation of the frame (R, c)."""
    a = np.zeros((6, 6))
    a[:3, :3] = R
    a[3:, 3:] = R
    a[3:, :3] = skew(c - x) @ R
    return a


def pair_assembly(prob, loss, one_origin=False):
    """A, g_T, B of the problem assembled the way the kernels do (FP64).  one_origin:
    the mixed path's order (csrc/k_system.cu k_pair_shift_df, k_pair_scan_df, k_pairs_to_A_df; the slab
    terms of csrc/k_linearize.cu k_jacobian_acc): every record moved once from c_lo to
    c_0, prefix and suffix sums about c_0, each block moved from c_0 to c_i; the slab
    terms formed from the rows about the pair origin and moved to the anchor centre."""
    N = int(prob.n_poses)
    P = 6 * N
    G = S.global_poses(prob.poses)
    lm, a, n = S._expand(prob)
    t_a, alpha, cams = S._camera_terms(prob, G, lm, a, n)
    Xw = np.einsum('oij,oj->oi', G[a][:, :3, :3], t_a) + G[a][:, :3, 3]   # world point
    Rw, cw = G[:, :3, :3], G[:, :3, 3]                                     # left cameras
    lo, hi = np.minimum(a, n), np.maximum(a, n)
    sgn = np.where(n > a, 1.0, -1.0)
    L = len(prob.host)

    # per-(lo, hi) records about the left centre of frame lo (the Jacobian pass)
    M = np.zeros((N + 1, N + 1, 6, 6))
    m = np.zeros((N + 1, N + 1, 6))
    # per-(landmark, pose) pose-depth columns about the anchor's left centre (the slab)
    b = np.zeros((L, N, 6))
    for res, Jp, Gn, R_an in cams:
        w2, _ = loss.weight2_and_rho(np.sum(res * res, -1), n, a)
        u = np.einsum('okj,oij->oki', Jp, Gn[:, :3, :3])                  # Jp R_n^T
        dta = -t_a / alpha[:, None]
        ja = np.einsum('oij,ojk,ok->oi', Jp, R_an, dta)                    # raw d r / d alpha
        for o in np.nonzero(lo != hi)[0]:
            K = np.concatenate([np.cross(Xw[o] - cw[lo[o]], u[o]), u[o]], -1)   # about c_lo
            M[lo[o], hi[o]] += w2[o] * K.T @ K
            m[lo[o], hi[o]] += sgn[o] * w2[o] * K.T @ res[o]
            if one_origin:
                q = sgn[o] * w2[o] * K.T @ ja[o]                                  # about c_lo
                q[:3] -= np.cross(cw[a[o]] - cw[lo[o]], q[3:])                    # to c_a
            else:
                Ka = np.concatenate([np.cross(Xw[o] - cw[a[o]], u[o]), u[o]], -1)   # about c_a
                q = sgn[o] * w2[o] * Ka.T @ ja[o]
            for i in range(lo[o], hi[o]):
                b[lm[o], i] += q

    # pass A: P(i, hi) = sum_{lo <= i} M(lo, hi), the running sum moved from c_{lo-1}
    # to c_lo before each record is added (every partial sum about its row's centre)
    Pf = np.zeros((N, N + 1, 6, 6))
    pf = np.zeros((N, N + 1, 6))
    for h in range(1, N + 1):
        acc, gacc = np.zeros((6, 6)), np.zeros(6)
        for lo_ in range(h):
            if one_origin:   # each record moved from c_lo to c_0, plain sums
                e = E(cw[lo_] - cw[0])
                acc, gacc = acc + e.T @ M[lo_, h] @ e, gacc + e.T @ m[lo_, h]
            else:
                if lo_ > 0:
                    e = E(cw[lo_ - 1] - cw[lo_])
                    acc, gacc = e.T @ acc @ e, e.T @ gacc
                acc, gacc = acc + M[lo_, h], gacc + m[lo_, h]
            Pf[lo_, h], pf[lo_, h] = acc, gacc
    if one_origin:   # each row's sums moved from c_0 to c_i
        for i in range(N):
            e = E(cw[0] - cw[i])
            for h in range(i + 1, N + 1):
                Pf[i, h], pf[i, h] = e.T @ Pf[i, h] @ e, e.T @ pf[i, h]
    # pass B: F(i, j) = sum_{hi > j} P(i, hi), all about c_i;  A(i, j) = Ad_i^T F Ad_j
    A = np.zeros((P, P))
    g = np.zeros(P)
    for i in range(N):
        for j in range(i, N):
            F = sum(Pf[i, h] for h in range(j + 1, N + 1))
            blk = Ad(Rw[i], cw[i], cw[i]).T @ F @ Ad(Rw[j], cw[j], cw[i])
            A[6 * i:6 * i + 6, 6 * j:6 * j + 6] = blk
            A[6 * j:6 * j + 6, 6 * i:6 * i + 6] = blk.T
        g[6 * i:6 * i + 6] = Ad(Rw[i], cw[i], cw[i]).T @ sum(pf[i, h] for h in range(i + 1, N + 1))
    # B_l(i) = Ad_i^T b_l(i) about the anchor centre
    B = np.zeros((P, L))
    host = np.asarray(prob.host)
    for l in range(L):
        for i in range(N):
            B[6 * i:6 * i + 6, l] = Ad(Rw[i], cw[i], cw[host[l]]).T @ b[l, i]
    return A, g, B


@pytest.mark.parametrize("one_origin", [False, True], ids=["chain", "one_origin"])
@pytest.mark.parametrize("loss", [S.Loss(), S.REFERENCE_GPU_LOSS, S.Loss(S.LOSS_HUBER, 2.0)],
                         ids=["l2", "cauchy_near_boost", "huber"])
def test_pair_assembly_matches_dense_products(loss, one_origin):
    p = scenes.circle_scene(5, 6, 60)
    lin = S.linearize(p, loss)
    A, g, B = pair_assembly(p, loss, one_origin)
    scale = lambda x: max(np.abs(x).max(), 1e-300)
    assert np.abs(A - lin.A).max() / scale(lin.A) < 1e-11
    assert np.abs(g - lin.g_T).max() / scale(lin.g_T) < 1e-11
    assert np.abs(B - lin.B).max() / scale(lin.B) < 1e-11


@pytest.mark.parametrize("one_origin", [False, True], ids=["chain", "one_origin"])
def test_pair_assembly_covisibility_window(one_origin):
    """A corridor with a 4-frame covisibility window: the records only span
    hi - lo <= window, and the prefix / suffix sums still give the dense blocks."""
    p = scenes.corridor_scene(3, 9, 120, window=4)
    lin = S.linearize(p, S.REFERENCE_GPU_LOSS)
    A, g, B = pair_assembly(p, S.REFERENCE_GPU_LOSS, one_origin)
    assert np.abs(A - lin.A).max() / np.abs(lin.A).max() < 1e-11
    assert np.abs(g - lin.g_T).max() / np.abs(lin.g_T).max() < 1e-11
    assert np.abs(B - lin.B).max() / np.abs(lin.B).max() < 1e-11


def test_recentring_steps_compose():
    """Moving a record by z1 then z2 is moving it by z1 + z2 (E(z1) E(z2) = E(z1 + z2)),
    so the prefix pass's step-by-step re-centring equals one move to row i's centre."""
    rng = np.random.default_rng(0)
    z1, z2 = rng.normal(size=3), rng.normal(size=3)
    assert np.abs(E(z1 + z2) - E(z1) @ E(z2)).max() < 1e-15
