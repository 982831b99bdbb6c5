"""Matrix-free operator, k-line preconditioner and restarted GMRES (oracle only).

Test infrastructure.  The operator is the factorised form of the assembled
matrix of dg1d.get_sysm; the solver follows the semantics of the reference's
Krylov wrapper:
  * right preconditioning, RHS normalisation, warm start as a correction about
    rho0 with the tolerance rescaled to the same absolute target, and an
    independent true-residual check that downgrades flag 0
    (DG_code/solve_transport_DG_full2D.m:279-334, 422-506);
  * the k-line block preconditioner: for every k an upwind element sweep with
    N_K x N_K block inverses (get_LineTransversePreconditioner_full2D.m:174-239).
    In 1D the operator is already diagonal in k, so each k is one "line"; the
    line operator keeps the flux and the k-diagonal of the Wigner-potential term.
"""
import numpy as np

from . import dg1d


class Operator1D:
    """y = A x without assembly.

    Flux: per k, Q_diff/detJ * [(k K1 + |k| K2) x_e + (k K3 + |k| K4) x_{e-1}
    + (k K5 + |k| K6) x_{e+1}].
    Wigner potential: X^ = Phi X (per DG node), Y^_{e,a} = sum_b T(beta_{e,ab}) X^_{e,b}
    with T the xi-tridiagonal of C_q and beta_{e,ab}(s) = (dxi/4) sum_q
    Q_drift invM(a,b) w_q W(q,a) W(q,b) B(e,q,s); then y += i Phi^H Y^.
    """

    def __init__(self, mat, p, EM, mpc=1.0):
        self.p = p
        self.n_el, self.nK, self.nk = p["N_chi"], p["N_K_chi"], p["Nk"]
        self.N = self.n_el * self.nK * self.nk
        K = dg1d.k_blocks(p)
        self.K = K
        detJ = p["delta_chi"] / 2
        k = p["k"]
        qd = p["Q_diff"] / detJ * mpc
        # per-k element blocks (nk, nK, nK)
        self.Dk = qd * (k[:, None, None] * K["K1"] + np.abs(k)[:, None, None] * (K["K2L"] + K["K2R"]))
        self.Lk = qd * (k[:, None, None] * K["K3"] + np.abs(k)[:, None, None] * K["K4"])   # from e-1
        self.Uk = qd * (k[:, None, None] * K["K5"] + np.abs(k)[:, None, None] * K["K6"])   # from e+1
        B = dg1d.drift_b(mat, p, EM)
        W = dg1d.interp_w(p)
        w = p["w"]
        invM = K["invM"]
        kap = p["Q_drift"] * invM[:, :, None] * (w[None, None, :] * W.T[:, None, :] * W.T[None, :, :])
        Bq = B.reshape(self.n_el, dg1d.NQX, -1)
        # beta[e, a, b, s]
        self.beta = np.einsum("abq,eqs->eabs", kap, Bq) * (p["delta_xi"] / 4) * mpc
        self.phi = p["phi"]

    def apply_flux(self, x):
        X = x.reshape(self.n_el, self.nK, self.nk)
        y = np.einsum("jab,ebj->eaj", self.Dk, X)
        y[1:] += np.einsum("jab,ebj->eaj", self.Lk, X[:-1])
        y[:-1] += np.einsum("jab,ebj->eaj", self.Uk, X[1:])
        return y.ravel()

    def apply_drift(self, x):
        X = x.reshape(self.n_el, self.nK, self.nk)
        Xh = np.einsum("sj,ebj->ebs", self.phi, X)
        Xm = np.zeros_like(Xh); Xm[..., 1:] = Xh[..., :-1]
        Xp = np.zeros_like(Xh); Xp[..., :-1] = Xh[..., 1:]
        b0 = self.beta[..., :-1]
        b1 = self.beta[..., 1:]
        Yh = np.einsum("eabs,ebs->eas", b0, Xh + Xm) + np.einsum("eabs,ebs->eas", b1, Xh + Xp)
        Y = 1j * np.einsum("sj,eas->eaj", self.phi.conj(), Yh)
        return Y.ravel()

    def apply(self, x):
        return self.apply_flux(x) + self.apply_drift(x)

    def drift_kdiag(self):
        """k-diagonal of the potential term per element: (n_el, nk, nK, nK).

        [Phi^H T(beta) Phi]_jj = (1/L) [sum_s T_ss + 2 cos(k_j h) sum_s T_s,s+1]
        with h the xi spacing of Phi's rows."""
        L = self.p["L_xi"]
        h = self.p["xi_elem"][1] - self.p["xi_elem"][0]
        k = self.p["k"]
        b = self.beta
        main = 2 * b.sum(-1) - b[..., 0] - b[..., -1]
        off = b[..., 1:-1].sum(-1)
        out = np.empty((self.n_el, self.nk, self.nK, self.nK), dtype=complex)
        for j in range(self.nk):
            out[:, j] = 1j / L * (main + 2 * np.cos(k[j] * h) * off)
        return out


class KLinePreconditioner:
    """Exact inverse of the per-k block-bidiagonal line operator.

    Line operator for k_j: diagonal blocks D_e = flux(k_j) + G_kk(e) and the
    upwind coupling from e-1 (k>0) or e+1 (k<0).  Forward sweep for k>0,
    backward for k<0 (get_LineTransversePreconditioner_full2D.m:199-221).
    """

    def __init__(self, op: Operator1D, use_drift_diag=True, sigma=0.0):
        self.op = op
        blocks = np.broadcast_to(op.Dk[None], (op.n_el, op.nk, op.nK, op.nK)).copy()
        if use_drift_diag:
            blocks = blocks + op.drift_kdiag()
        if sigma:
            blocks = blocks + sigma * np.eye(op.nK)
        self.inv = np.linalg.inv(blocks)          # (n_el, nk, nK, nK)
        self.forward = op.p["k"] > 0

    def apply(self, r):
        op = self.op
        R = r.reshape(op.n_el, op.nK, op.nk)
        Z = np.zeros_like(R)
        fw = self.forward
        bw = ~fw
        prev = None
        for e in range(op.n_el):
            rhs = R[e][:, fw].T                      # (nkf, nK)
            if e > 0:
                rhs = rhs - np.einsum("jab,jb->ja", op.Lk[fw], Z[e - 1][:, fw].T)
            Z[e][:, fw] = np.einsum("jab,jb->ja", self.inv[e][fw], rhs).T
        for e in range(op.n_el - 1, -1, -1):
            rhs = R[e][:, bw].T
            if e < op.n_el - 1:
                rhs = rhs - np.einsum("jab,jb->ja", op.Uk[bw], Z[e + 1][:, bw].T)
            Z[e][:, bw] = np.einsum("jab,jb->ja", self.inv[e][bw], rhs).T
        return Z.ravel()


def gmres_right(apply_a, apply_m, b, restart=50, tol=1e-10, maxit=50, x0=None):
    """Restarted right-preconditioned GMRES(m) with modified Gram-Schmidt and
    Givens rotations; returns (x, flag, relres_true, iterations, resvec).

    Stopping test |r| <= tol |b| on the Arnoldi residual estimate; the warm
    start is a correction about x0 with the tolerance rescaled to the same
    absolute target (solve_transport_DG_full2D.m:462-484).
    """
    bnorm = np.linalg.norm(b)
    if bnorm == 0:
        return np.zeros_like(b), 0, 0.0, 0, [0.0]
    x = np.zeros_like(b) if x0 is None else x0.astype(complex).copy()
    r = b - apply_a(x) if x0 is not None else b.astype(complex).copy()
    target = tol * bnorm
    resvec = [np.linalg.norm(r)]
    total = 0
    flag = 1
    for cycle in range(maxit):
        beta = np.linalg.norm(r)
        if beta <= target:
            flag = 0
            break
        V = np.zeros((restart + 1, b.size), dtype=complex)
        H = np.zeros((restart + 1, restart), dtype=complex)
        cs = np.zeros(restart, dtype=complex)
        sn = np.zeros(restart, dtype=complex)
        g = np.zeros(restart + 1, dtype=complex)
        g[0] = beta
        V[0] = r / beta
        k_used = 0
        for k in range(restart):
            w = apply_a(apply_m(V[k]))
            for i in range(k + 1):
                H[i, k] = np.vdot(V[i], w)
                w = w - H[i, k] * V[i]
            H[k + 1, k] = np.linalg.norm(w)
            if H[k + 1, k] != 0:
                V[k + 1] = w / H[k + 1, k]
            for i in range(k):
                t = cs[i] * H[i, k] + sn[i] * H[i + 1, k]
                H[i + 1, k] = -np.conj(sn[i]) * H[i, k] + np.conj(cs[i]) * H[i + 1, k]
                H[i, k] = t
            a, bb = H[k, k], H[k + 1, k]
            den = np.sqrt(abs(a) ** 2 + abs(bb) ** 2)
            cs[k] = a / den if den else 1.0
            sn[k] = bb / den if den else 0.0
            # rotation [c s; -conj(s) conj(c)] with c = a/den, s = b/den (complex Givens)
            cs[k] = np.conj(cs[k]); sn[k] = np.conj(sn[k])
            H[k, k] = cs[k] * a + sn[k] * bb
            H[k + 1, k] = 0.0
            g[k + 1] = -np.conj(sn[k]) * g[k]
            g[k] = cs[k] * g[k]
            total += 1
            k_used = k + 1
            resvec.append(abs(g[k + 1]))
            if abs(g[k + 1]) <= target:
                break
        y = np.linalg.solve(np.triu(H[:k_used, :k_used]), g[:k_used])
        x = x + apply_m(V[:k_used].T @ y)
        r = b - apply_a(x)
        if np.linalg.norm(r) <= target:
            flag = 0
            break
    relres = np.linalg.norm(b - apply_a(x)) / bnorm
    if flag == 0 and relres > tol:
        flag = 1
    return x, flag, relres, total, resvec
