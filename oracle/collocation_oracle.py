"""ORACLE — CPU restatement of the reference collocation solver, for testing only.

This module is test infrastructure.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm may import it, and only as the checker
or as the timed CPU baseline; the CUDA product never calls it.

It restates, in vectorised numpy (float64 throughout), the algorithm of
UW-OCP/Collocation-Solver-CUDA for one BVP-DAE instance, stage by stage, with
the reference's own structure and quirks:

  form_initial_input      collocation_solver_parallel_2d_shared.py:287-356
  compute_f_q             collocation_solver_parallel_2d_shared.py:399-559
  construct_jacobian      collocation_solver_parallel_2d_shared.py:611-797
  reduce_jacobian         collocation_solver_parallel_2d_shared.py:840-1001
                          (partial-pivot LU, matrix_factorization_cuda.py:91-165)
  partition_factorization solve_babd_system.py:93-258 (M = 8 partitions,
                          Householder QR with the sign rule of
                          matrix_factorization_cuda.py:5-82)
  reduced BABD solve      solve_babd_system.py:311-440 (numpy QR + solve)
  partition_backsub       solve_babd_system.py:495-572
  recover_delta_k         collocation_solver_parallel_2d_shared.py:1580-1650
  line search             collocation_solver_parallel_2d_shared.py:155-174
  segment_residual        collocation_solver_parallel_2d_shared.py:1770-1892
                          (residual_type 1 with the scale_by_time quirk: the
                          running sum is multiplied by h after every component)
  recover_solution        collocation_solver_parallel_2d_shared.py:2034-2075
  remesh                  collocation_solver_parallel_2d_shared.py:2106-2311
  solve (driver)          collocation_solver_parallel_2d_shared.py:36-251

Problem interface (duck-typed `prob`): sizes ny, nz, np; theta (constants);
vectorised f(y, z, p, th) -> (n, ny), g(y, z, p, th, alpha) -> (n, nz),
Df(y, z, p, th) -> (n, ny, ny+nz+np), Dg(y, z, p, th, alpha) -> (n, nz, ...),
r(y0, y1, p, th) -> (ny+np,), Dr(y0, y1, p, th) -> (ny+np, 2ny+np).

Collocation tables (Lobatto A, b, c; Gauss nodes/weights; the Lagrange basis
and its integral at the Gauss nodes) are passed in as `rk` and `seg` objects.

Pinned against the golden fixtures in tests/golden/, which were produced by
running the unmodified reference (tests/golden/make_golden.py).
"""
import numpy as np

EPS = np.finfo(np.float64).eps


# --------------------------------------------------------------- residual ---
def form_initial_input(prob, m, N, y0, z0, p, rk, alpha=None):
    """y' at the collocation points from linearly interpolated y, z (CS:287-356)."""
    ny, nz = prob.ny, prob.nz
    c = rk.c
    yl = (1.0 - c)[None, :, None] * y0[:-1, None, :] + c[None, :, None] * y0[1:, None, :]
    zl = (1.0 - c)[None, :, None] * z0[:-1, None, :] + c[None, :, None] * z0[1:, None, :]
    yt = yl.reshape((N - 1) * m, ny)
    zt = zl.reshape((N - 1) * m, nz)
    y_dot = prob.f(yt, zt, p, prob.theta)
    return y0.copy(), y_dot, zt.copy()


def collocation_update(m, N, A, t, y, y_dot):
    """y~_ij = y_i + h_i sum_k A_jk y'_ik (CS:520-559)."""
    ny = y.shape[1]
    h = t[1:] - t[:-1]
    yd = y_dot.reshape(N - 1, m, ny)
    s = np.zeros((N - 1, m, ny))
    for k in range(m):
        s += A[None, :, k, None] * yd[:, k, None, :]
    return (y[:-1, None, :] + h[:, None, None] * s).reshape((N - 1) * m, ny)


def compute_f_q(prob, m, N, rk, t, y, y_dot, z_tilde, p, alpha):
    """Residual pieces f_a, f_b, r_bc and the assembled vector (CS:399-512)."""
    ny, nz = prob.ny, prob.nz
    y_tilde = collocation_update(m, N, rk.A, t, y, y_dot)
    rh = prob.f(y_tilde, z_tilde, p, prob.theta) - y_dot
    rg = prob.g(y_tilde, z_tilde, p, prob.theta, alpha)
    f_a = np.concatenate([rh.reshape(N - 1, m, ny), rg.reshape(N - 1, m, nz)], axis=2).reshape(N - 1, m * (ny + nz))
    h = t[1:] - t[:-1]
    yd = y_dot.reshape(N - 1, m, ny)
    sb = np.zeros((N - 1, ny))
    for j in range(m):
        sb += rk.b[j] * yd[:, j, :]
    f_b = y[1:] - y[:-1] - h[:, None] * sb
    r_bc = prob.r(y[0], y[N - 1], p, prob.theta)
    f_q = np.concatenate([np.concatenate([f_a, f_b], axis=1).ravel(), r_bc])
    return f_q, y_tilde, f_a, f_b, r_bc


# --------------------------------------------------------------- jacobian ---
def interval_jacobian(prob, m, rk, h, y_tilde, z_tilde, p, alpha):
    """J, V, D, W of the intervals of widths h, from the stage values of
    those intervals (CS:680-797); every interval is computed on its own."""
    ny, nz, npar = prob.ny, prob.nz, prob.np
    n = len(h)
    s = m * (ny + nz)
    Df = prob.Df(y_tilde, z_tilde, p, prob.theta).reshape(n, m, ny, ny + nz + npar)
    Dg = prob.Dg(y_tilde, z_tilde, p, prob.theta, alpha).reshape(n, m, nz, ny + nz + npar)
    J = np.zeros((n, m, ny + nz, ny))
    V = np.zeros((n, m, ny + nz, npar))
    J[:, :, :ny, :] = Df[:, :, :, :ny]
    J[:, :, ny:, :] = Dg[:, :, :, :ny]
    V[:, :, :ny, :] = Df[:, :, :, ny + nz:]
    V[:, :, ny:, :] = Dg[:, :, :, ny + nz:]
    D = np.zeros((n, ny, m, ny + nz))
    for j in range(m):
        for k in range(ny):
            D[:, k, j, k] = h * rk.b[j]
    W = np.zeros((n, m, ny + nz, m, ny + nz))
    for j in range(m):
        for k in range(m):
            hA = (h * rk.A[j, k])[:, None, None]
            W[:, j, :ny, k, :ny] = hA * Df[:, j, :, :ny]
            W[:, j, ny:, k, :ny] = hA * Dg[:, j, :, :ny]
            if j == k:
                W[:, j, :ny, k, :ny] -= np.eye(ny)[None]
                W[:, j, :ny, k, ny:] = Df[:, j, :, ny:ny + nz]
                W[:, j, ny:, k, ny:] = Dg[:, j, :, ny:ny + nz]
    return J.reshape(n * s, ny), V.reshape(n * s, npar), D.reshape(n * ny, s), W.reshape(n * s, s)


def boundary_jacobian(prob, N, y, p):
    """B_0, B_n, V_n: the columns of Dr for y_0, y_n and p (CS:611-797)."""
    ny = prob.ny
    dr = prob.Dr(y[0], y[N - 1], p, prob.theta)
    return dr[:, 0:ny].copy(), dr[:, ny:2 * ny].copy(), dr[:, 2 * ny:].copy()


def construct_jacobian(prob, m, N, rk, t, y, y_tilde, z_tilde, p, alpha):
    """J, V, D, W per interval and B_0, B_n, V_n (CS:611-797)."""
    J, V, D, W = interval_jacobian(prob, m, rk, t[1:] - t[:-1], y_tilde, z_tilde, p, alpha)
    B_0, B_n, V_n = boundary_jacobian(prob, N, y, p)
    return J, V, D, W, B_0, B_n, V_n


def reduce_jacobian(ny, nz, npar, m, N, W, D, J, V, f_a, f_b):
    """Condensation of the stage unknowns (CS:840-1001):
    A = -I + D W^-1 J, C = I, H = D W^-1 V, b = -f_b - D W^-1 f_a."""
    s = m * (ny + nz)
    Wb = W.reshape(N - 1, s, s)
    rhs = np.concatenate([J.reshape(N - 1, s, ny), V.reshape(N - 1, s, npar), f_a.reshape(N - 1, s, 1)], axis=2)
    X = np.linalg.solve(Wb, rhs)
    DX = np.matmul(D.reshape(N - 1, ny, s), X)
    A = -np.eye(ny)[None] + DX[:, :, :ny]
    H = DX[:, :, ny:ny + npar]
    b = -f_b - DX[:, :, ny + npar]
    C = np.broadcast_to(np.eye(ny), (N - 1, ny, ny)).copy()
    return A.reshape((N - 1) * ny, ny), C.reshape((N - 1) * ny, ny), H.reshape((N - 1) * ny, npar), b


# ---------------------------------------------------------------- BABD ------
def householder_qr(a, eps=EPS):
    """Q (n x n), R (n x k) with a = Q R, Householder sign rule and early stop
    of matrix_factorization_cuda.py:5-82: v_k >= 0 -> s = +1, g = -s |v|,
    stop at the first column whose reflector has |v|^2 < eps."""
    n, k = a.shape
    cpy = a.astype(np.float64).copy()
    vs_list = []
    col = k
    for c in range(k):
        vv = cpy[c:, c].copy()
        s = 1.0 if vv[0] >= 0 else -1.0
        g = -s * np.sqrt(np.dot(vv, vv))
        vv[0] -= g
        vsq = np.dot(vv, vv)
        if vsq < eps:
            col = c
            break
        beta = -2.0 / vsq
        w = vv @ cpy[c:, c:]
        cpy[c:, c:] += beta * np.outer(vv, w)
        vs_list.append((c, vv, beta))
    R = np.zeros((n, k))
    R[:k, :] = cpy[:k, :]
    Q = np.eye(n)
    for c, vv, beta in reversed(vs_list[:col]):
        u = vv @ Q[c:, c:]
        Q[c:, c:] += beta * np.outer(vv, u)
    return Q, R


def partition_index(M, N):
    k = (N - 1) // M
    return np.array([i * k for i in range(M)] + [N - 1])


def partition_factorization(ny, npar, M, N, A, C, H, b):
    """Sequential QR sweep inside each of M partitions (SB:93-258)."""
    index = partition_index(M, N)
    A3 = A.reshape(N - 1, ny, ny)
    C3 = C.reshape(N - 1, ny, ny)
    H3 = H.reshape(N - 1, ny, npar)
    R = np.zeros((N - 1, ny, ny))
    E = np.zeros((N - 1, ny, ny))
    G = np.zeros((N - 1, ny, ny))
    Jr = np.zeros((N - 1, ny, npar))
    d = np.zeros((N - 1, ny))
    At = np.zeros((M, ny, ny))
    Ct = np.zeros((M, ny, ny))
    Ht = np.zeros((M, ny, npar))
    bt = np.zeros((M, ny))
    for i in range(M):
        r0, r1 = index[i], index[i + 1] - 1
        ct, gt, htl, btl = C3[r0].copy(), A3[r0].copy(), H3[r0].copy(), b[r0].copy()
        for j in range(r0, r1):
            Q, Rq = householder_qr(np.vstack([ct, A3[j + 1]]))
            Qt = Q.T
            ec = Qt[:, ny:] @ C3[j + 1]
            gg = Qt[:, :ny] @ gt
            jh = Qt[:, :ny] @ htl + Qt[:, ny:] @ H3[j + 1]
            db = Qt[:, :ny] @ btl + Qt[:, ny:] @ b[j + 1]
            E[j], ct = ec[:ny], ec[ny:]
            G[j], gt = gg[:ny], gg[ny:]
            Jr[j], htl = jh[:ny], jh[ny:]
            d[j], btl = db[:ny], db[ny:]
            R[j] = Rq[:ny]
        At[i], Ct[i], Ht[i], bt[i] = gt, ct, htl, btl
    return (index, R.reshape(-1, ny), E.reshape(-1, ny), Jr.reshape((N - 1) * ny, npar), G.reshape(-1, ny), d,
            At.reshape(-1, ny), Ct.reshape(-1, ny), Ht.reshape(M * ny, npar), bt)


def _solve_or_zero(Rm, rhs):
    try:
        return np.linalg.solve(Rm, rhs)
    except np.linalg.LinAlgError:
        return np.zeros(rhs.shape)


def reduced_babd_solve(ny, npar, M, A_t, C_t, H_t, b_t, B_0, B_n, V_n, b_n):
    """Reduced (M+1)-node system: sequential numpy QR sweep, final block QR and
    back substitution (SB:311-440, babd_node.py).  Returns delta_s (M+1, ny), delta_p."""
    At = A_t.reshape(M, ny, ny)
    Ct = C_t.reshape(M, ny, ny)
    Ht = H_t.reshape(M, ny, npar)
    c_t, g_t, h_t, bb_t = Ct[0], At[0], Ht[0], b_t[0]
    Rn, En, Gn, Kn, dn = {}, {}, {}, {}, {}
    for i in range(M - 1):
        Q, Rq = np.linalg.qr(np.vstack([c_t, At[i + 1]]), mode="complete")
        Rn[i] = Rq[:ny]
        ec = Q.T @ np.vstack([np.zeros((ny, ny)), Ct[i + 1]])
        En[i], c_t = ec[:ny], ec[ny:]
        gg = Q.T @ np.vstack([g_t, np.zeros((ny, ny))])
        Gn[i], g_t = gg[:ny], gg[ny:]
        jh = Q.T @ np.vstack([h_t, Ht[i + 1]])
        Kn[i], h_t = jh[:ny, :npar], jh[ny:, :npar]
        db = Q.T @ np.concatenate([bb_t, b_t[i + 1]])
        dn[i], bb_t = db[:ny], db[ny:]
    final = np.vstack([np.hstack([c_t, g_t, h_t]), np.hstack([B_n, B_0, V_n])])
    Q, Rq = np.linalg.qr(final, mode="complete")
    Rn[M - 1] = Rq[:ny, :ny]
    Gn[M - 1] = Rq[:ny, ny:2 * ny]
    Kn[M - 1] = Rq[:ny, 2 * ny:2 * ny + npar]
    RM = Rq[ny:2 * ny, ny:2 * ny]
    KM = Rq[ny:2 * ny, 2 * ny:2 * ny + npar]
    Rp = Rq[2 * ny:2 * ny + npar, 2 * ny:2 * ny + npar]
    dd = Q.T @ np.concatenate([bb_t, b_n])
    dn[M - 1] = dd[:ny]
    dM = dd[ny:2 * ny]
    dp = dd[2 * ny:2 * ny + npar]
    delta_p = _solve_or_zero(Rp, dp)
    ds = np.zeros((M + 1, ny))
    ds[0] = _solve_or_zero(RM, dM - KM @ delta_p)
    ds[M] = _solve_or_zero(Rn[M - 1], dn[M - 1] - Gn[M - 1] @ ds[0] - Kn[M - 1] @ delta_p)
    for i in range(M - 1, 0, -1):
        rhs = dn[i - 1] - En[i - 1] @ ds[i + 1] - Gn[i - 1] @ ds[0] - Kn[i - 1] @ delta_p
        ds[i] = _solve_or_zero(Rn[i - 1], rhs)
    return ds, delta_p.copy()


def partition_backward_substitution(ny, npar, M, N, index, delta_s_r, delta_p, R, G, E, J, d):
    """delta y at every node from the partition-boundary values (SB:495-572)."""
    R3 = R.reshape(N - 1, ny, ny)
    G3 = G.reshape(N - 1, ny, ny)
    E3 = E.reshape(N - 1, ny, ny)
    J3 = J.reshape(N - 1, ny, npar)
    ds = np.zeros((N, ny))
    for i in range(M):
        r0, r1 = index[i], index[i + 1] - 1
        ds[r0] = delta_s_r[i]
        ds[r1 + 1] = delta_s_r[i + 1]
        for j in range(r1, r0, -1):
            vec = d[j - 1] - G3[j - 1] @ ds[r0] - E3[j - 1] @ ds[j + 1] - J3[j - 1] @ delta_p
            ds[j] = np.linalg.solve(np.triu(R3[j - 1]), vec)
    return ds


def solve_babd(ny, npar, N, A, C, H, b, B_0, B_n, V_n, r_bc, M=8):
    index, R, E, Jr, G, d, At, Ct, Ht, bt = partition_factorization(ny, npar, M, N, A, C, H, b)
    ds_r, dp = reduced_babd_solve(ny, npar, M, At, Ct, Ht, bt, B_0, B_n, V_n, -r_bc)
    dy = partition_backward_substitution(ny, npar, M, N, index, ds_r, dp, R, G, E, Jr, d)
    return dy, dp


def recover_delta_k(ny, nz, m, N, delta_y, delta_p, f_a, J, V, W):
    """delta k_i = W_i^-1 (-f_a - J_i dy_i - V_i dp) (CS:1580-1650)."""
    s = m * (ny + nz)
    Jb = J.reshape(N - 1, s, ny)
    Vb = V.reshape(N - 1, s, -1)
    rhs = -f_a - np.einsum("isk,ik->is", Jb, delta_y[:-1]) - np.einsum("isk,k->is", Vb, delta_p)
    dk = np.linalg.solve(W.reshape(N - 1, s, s), rhs[..., None])[..., 0]
    dk3 = dk.reshape(N - 1, m, ny + nz)
    return dk, dk3[:, :, :ny].reshape((N - 1) * m, ny).copy(), dk3[:, :, ny:].reshape((N - 1) * m, nz).copy()


# ------------------------------------------------------------ mesh error ----
def segment_residual(prob, m, N, t, y, y_dot, z_tilde, p, alpha, tol, seg, residual_type=1, scale_by_time=True,
                     residual2=False):
    """Per-interval residual at the m+1 Gauss points and |r|_inf / tol at
    index N-1 (CS:1770-1892).  residual_type 1 (default, a weighted sum of
    |h - y'| and |g|), 2 (weighted squares, square root at the end) or 0 (a
    weighted maximum; its g part takes |h - y'| of the first nz components,
    as CS:1882-1883 does); with scale_by_time the running sum is multiplied
    by h after each component (CS:1868-1869, 1883-1884).  residual2
    (CS:1895-2013): max over the Gauss points and components of
    |h - y'| / (1 + max |y'|) and |g| / (1 + max |z|)."""
    ny, nz = prob.ny, prob.nz
    h = t[1:] - t[:-1]
    yd = y_dot.reshape(N - 1, m, ny)
    zt = z_tilde.reshape(N - 1, m, nz)
    rho_h = np.zeros(N - 1)
    rho_g = np.zeros(N - 1)
    pts = []
    for i in range(m + 1):
        L, I, w = seg["L"][i], seg["I"][i], seg["w"][i]
        ydot_t = np.einsum("k,ikl->il", L, yd)
        y_t = y[:-1] + h[:, None] * np.einsum("k,ikl->il", I, yd)
        z_t = np.einsum("k,ikl->il", L, zt)
        pts.append((w, ydot_t, y_t, z_t))
    if residual2:
        ydg = np.max([np.abs(q[1]) for q in pts], axis=0)
        zg = np.max([np.abs(q[3]) for q in pts], axis=0) if nz else None
        for w, ydot_t, y_t, z_t in pts:
            hres = prob.f(y_t, z_t, p, prob.theta) - ydot_t
            rho_h = np.maximum(rho_h, np.max(np.abs(hres) / (1.0 + ydg), axis=1))
            if nz > 0:
                gres = prob.g(y_t, z_t, p, prob.theta, alpha)
                rho_g = np.maximum(rho_g, np.max(np.abs(gres) / (1.0 + zg), axis=1))
        residual = np.zeros(N)
        residual[:N - 1] = np.maximum(rho_h, rho_g) / tol
    else:
        for w, ydot_t, y_t, z_t in pts:
            hres = prob.f(y_t, z_t, p, prob.theta) - ydot_t
            for k in range(ny):
                if residual_type == 2:
                    rho_h = rho_h + w * hres[:, k] * hres[:, k]
                elif residual_type == 1:
                    rho_h = rho_h + w * np.abs(hres[:, k])
                else:
                    rho_h = np.maximum(rho_h, w * np.abs(hres[:, k]))
                if scale_by_time:
                    rho_h = rho_h * h
            if nz > 0:
                gres = prob.g(y_t, z_t, p, prob.theta, alpha)
                for k in range(nz):
                    if residual_type == 2:
                        rho_g = rho_g + w * gres[:, k] * gres[:, k]
                    elif residual_type == 1:
                        rho_g = rho_g + w * np.abs(gres[:, k])
                    else:
                        rho_g = np.maximum(rho_g, w * np.abs(hres[:, k]))
                    if scale_by_time:
                        rho_g = rho_g * h
        residual = np.zeros(N)
        if residual_type == 2:
            residual[:N - 1] = np.sqrt(rho_h + rho_g) / tol
        elif residual_type == 1:
            residual[:N - 1] = (np.abs(rho_h) + np.abs(rho_g)) / tol
        else:
            residual[:N - 1] = np.maximum(rho_h, rho_g) / tol
    if prob.ny + prob.np > 0:
        r = prob.r(y[0], y[N - 1], p, prob.theta)
        residual[N - 1] = np.max(np.abs(r)) / tol
    return residual, float(np.max(residual))


def recover_solution(nz, m, N, z_tilde, seg):
    """z at the nodes from the stage values (CS:2034-2075)."""
    zt = z_tilde.reshape(N - 1, m, nz)
    z = np.zeros((N, nz))
    z[:N - 1] = np.einsum("k,ikl->il", seg["L0"], zt)
    z[N - 1] = np.einsum("k,kl->l", seg["L1"], zt[N - 2])
    return z


def remesh(ny, nz, N, tspan, y0, z0, residual):
    """Node deletion (5 quiet nodes -> keep 1st, 3rd, 5th) then insertion
    (res > 10: 3 equispaced nodes, res > 1: midpoint) (CS:2106-2311)."""
    keep = []
    i = 0
    thr = 1e-2
    while i < N - 4:
        if residual[i] <= thr and all(residual[i + q] <= thr for q in range(1, 5)):
            keep += [i, i + 2, i + 4]
            i += 5
        else:
            keep.append(i)
            i += 1
    while i < N:
        keep.append(i)
        i += 1
    tT = tspan[keep]
    yT = y0[keep]
    zT = z0[keep]
    rT = residual[keep]
    NT = len(keep)
    t_new, y_new, z_new = [], [], []
    for i in range(NT - 1):
        res = rT[i]
        if res > 1:
            q = 4 if res > 10 else 2
            dt = (tT[i + 1] - tT[i]) / q
            dy = (yT[i + 1] - yT[i]) / q
            dz = (zT[i + 1] - zT[i]) / q
            t_new.append(tT[i])
            y_new.append(yT[i])
            z_new.append(zT[i])
            for k in range(1, q):
                t_new.append(tT[i] + k * dt)
                y_new.append(yT[i] + k * dy)
                z_new.append(zT[i] + k * dz)
        else:
            t_new.append(tT[i])
            y_new.append(yT[i])
            z_new.append(zT[i])
    t_new.append(tT[NT - 1])
    y_new.append(yT[NT - 1])
    z_new.append(zT[NT - 1])
    return len(t_new), np.array(t_new), np.array(y_new).reshape(-1, ny), np.array(z_new).reshape(-1, nz)


# ----------------------------------------------------------------- driver ---
class SolveResult:
    pass


def newton_step(prob, m, N, rk, t, y, y_dot, z_tilde, p, alpha, f_a, f_b, r_bc, y_tilde, M=8, chunk=None):
    """Jacobian, condensation, partitioned BABD solve and recovery: the Newton
    direction (CS:121-152).

    chunk: intervals per pass of the Jacobian, condensation and recovery
    (default: all at once).  Each interval is computed on its own, so any
    chunk gives the same numbers; a chunk bounds the memory of the stage
    matrices W (s x s per interval: 38 GB for 16,384 intervals of s = 544),
    which the recovery forms again, as the reference re-factorises them."""
    ny, nz, npar = prob.ny, prob.nz, prob.np
    n_int = N - 1
    chunk = n_int if chunk is None else max(1, int(chunk))
    h = t[1:] - t[:-1]
    A = np.empty((n_int * ny, ny))
    C = np.empty((n_int * ny, ny))
    H = np.empty((n_int * ny, npar))
    b = np.empty((n_int, ny))

    def blocks(i0, i1):
        return interval_jacobian(prob, m, rk, h[i0:i1], y_tilde[i0 * m:i1 * m], z_tilde[i0 * m:i1 * m], p, alpha)

    for i0 in range(0, n_int, chunk):
        i1 = min(n_int, i0 + chunk)
        J, V, D, W = blocks(i0, i1)
        Ac, Cc, Hc, bc = reduce_jacobian(ny, nz, npar, m, i1 - i0 + 1, W, D, J, V, f_a[i0:i1], f_b[i0:i1])
        A[i0 * ny:i1 * ny], C[i0 * ny:i1 * ny], H[i0 * ny:i1 * ny], b[i0:i1] = Ac, Cc, Hc, bc
    B_0, B_n, V_n = boundary_jacobian(prob, N, y, p)
    dy, dp = solve_babd(ny, npar, N, A, C, H, b, B_0, B_n, V_n, r_bc, M=M)
    dyd = np.empty((n_int * m, ny))
    dzt = np.empty((n_int * m, nz))
    for i0 in range(0, n_int, chunk):
        i1 = min(n_int, i0 + chunk)
        J, V, D, W = blocks(i0, i1)
        _, dyd[i0 * m:i1 * m], dzt[i0 * m:i1 * m] = recover_delta_k(ny, nz, m, i1 - i0 + 1, dy[i0:i1 + 1], dp,
                                                                    f_a[i0:i1], J, V, W)
    return dy, dyd, dzt, dp


def solve(prob, m, rk, seg, T0=None, Y0=None, Z0=None, P0=None, verbose=False, M=8, residual_type=1,
          scale_by_time=True, residual2=False, chunk=None, trace=None):
    """The reference driver (CS:36-251): alpha continuation, damped Newton with
    a halving line search, segment residual and remesh.  Returns SolveResult.
    chunk: see newton_step.  trace(event, **data), when given, is called with
    ("direction", dy=, dp=) after every Newton direction (used to record the
    first direction of large fixtures)."""
    ny, nz, npar = prob.ny, prob.nz, prob.np
    t_span = np.array(prob.T0 if T0 is None else T0, dtype=np.float64).copy()
    y0 = np.array(prob.Y0 if Y0 is None else Y0, dtype=np.float64)
    z0 = np.array(prob.Z0 if Z0 is None else Z0, dtype=np.float64)
    p0 = np.array(prob.P0 if P0 is None else P0, dtype=np.float64)
    N = t_span.shape[0]
    tol = prob.tolerance
    max_iter = prob.maximum_newton_iterations
    max_mesh = prob.maximum_mesh_refinements
    max_nodes = prob.maximum_nodes
    min_nodes = 3
    max_linesearch = 20
    alpha = 0.1
    alpha_m = 1e-6 if (prob.size_inequality > 0 or prob.size_sv_inequality > 0) else 0.1
    beta = 0.9
    res = SolveResult()
    res.norms, res.nodes_after_remesh, res.alphas = [], [], []
    res.residual_count = res.jacobian_count = res.segment_count = 0
    para = p0.copy()
    max_residual = 1 / tol
    y, y_dot, z_tilde = form_initial_input(prob, m, N, y0, z0, para, rk)
    success = 1
    for alphacal in range(max_iter):
        res.alphas.append(alpha)
        mesh_it = 0
        iter_time = 0
        for iter_time in range(max_iter):
            f_q, y_tilde, f_a, f_b, r_bc = compute_f_q(prob, m, N, rk, t_span, y, y_dot, z_tilde, para, alpha)
            res.residual_count += 1
            norm = np.linalg.norm(f_q, np.inf)
            res.norms.append(norm)
            if verbose:
                print("\tnorm: {0:.8f}".format(norm))
            if norm < tol:
                break
            res.jacobian_count += 1
            dy, dyd, dzt, dp = newton_step(prob, m, N, rk, t_span, y, y_dot, z_tilde, para, alpha,
                                           f_a, f_b, r_bc, y_tilde, M=M, chunk=chunk)
            if trace is not None:
                trace("direction", dy=dy, dp=dp)
            a0 = 1.0
            for _ in range(max_linesearch):
                yn = y + a0 * dy
                ydn = y_dot + a0 * dyd
                ztn = z_tilde + a0 * dzt
                pn = para + a0 * dp
                fqn = compute_f_q(prob, m, N, rk, t_span, yn, ydn, ztn, pn, alpha)[0]
                res.residual_count += 1
                if np.linalg.norm(fqn, np.inf) < norm:
                    y, y_dot, z_tilde, para = yn, ydn, ztn, pn
                    break
                a0 /= 2
        if alphacal >= (max_iter - 1) or iter_time >= (max_iter - 1) \
                or N > max_nodes or mesh_it > max_mesh or N < min_nodes:
            success = 0
            break
        residual, max_residual = segment_residual(prob, m, N, t_span, y, y_dot, z_tilde, para, alpha, tol, seg,
                                                  residual_type, scale_by_time, residual2)
        res.segment_count += 1
        if max_residual > 1:
            z = recover_solution(nz, m, N, z_tilde, seg)
            N, t_span, y, z = remesh(ny, nz, N, t_span, y, z, residual)
            mesh_it += 1
            y, y_dot, z_tilde = form_initial_input(prob, m, N, y, z, para, rk)
            res.nodes_after_remesh.append(N)
            if mesh_it > max_mesh or N > max_nodes or N < min_nodes:
                success = 0
                break
        else:
            if alpha <= alpha_m:
                break
            alpha *= beta
    res.success = bool(alpha <= alpha_m and success)
    res.alpha = alpha
    res.N = N
    res.t = t_span
    res.y = y
    res.y_dot = y_dot
    res.z_tilde = z_tilde
    res.z = recover_solution(nz, m, N, z_tilde, seg)
    res.p = para
    res.max_residual = max_residual
    return res
