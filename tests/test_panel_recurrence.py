"""The blocked Householder reduction of the eigensolver (zlatrd-style panel
recurrence, lower formulation), restated in numpy in the order the kernels
run it, and checked against LAPACK's spectrum.

Per panel column i (k0 <= i < k0 + jb, jj = i - k0):
  column update   A(i:n, i) -= V(i:n, 0:jj) W(i, 0:jj)^H + W(i:n, 0:jj) V(i, 0:jj)^H
  reflector       v, tau from A(i+1:n, i)   (beta = -sign(Re alpha) |[alpha, x]|)
  mat-vec         y = A22 v with A22 the panel-start trailing matrix
  corrections     w = tau (y - W x1 - V x2), x1 = V^H v, x2 = W^H v
  completion      w += alpha v, alpha = -1/2 tau (w^H v)   (in the next column's update)
and after the panel the trailing update A22 -= V W^H + W V^H.

The kernels split the column update: the corrections kernel of column i
(which reads rows of V and W for W x1 + V x2) also applies panel columns
0 .. jj-1 to column i+1, and the next column update applies only column jj
(after completing w).  Both orders are restated here and must give the same
tridiagonal matrix, whose eigenvalues must be the input's."""
import numpy as np


def _hermitian(rng, n):
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (M + M.conj().T) / 2


def _reduce(A0, nb, fused):
    A = A0.astype(complex).copy()
    n = A.shape[0]
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 0))
    for k0 in range(0, n, nb):
        jb = min(nb, n - k0)
        W = np.zeros((n, jb), complex)
        A22 = A.copy()  # the mat-vec's matrix: the trailing block as the panel started
        pending = None  # (jj, alpha) of a w still to complete
        for jj in range(jb):
            i = k0 + jj
            V = A[:, k0:k0 + jj]  # Householder vectors of the panel's earlier columns
            if pending is not None:  # complete w of the previous column
                pj, alpha = pending
                W[:, pj] += alpha * A[:, k0 + pj]
                pending = None
            lo = (jj - 1) if (fused and jj > 0) else 0  # fused: columns < jj-1 were applied already
            for c in range(lo, jj):
                A[i:, i] -= A[i:, k0 + c] * np.conj(W[i, c]) + W[i:, c] * np.conj(A[i, k0 + c])
            d[i] = A[i, i].real
            if i == n - 1:
                break
            alpha_r = A[i + 1, i]
            x = A[i + 2:, i]
            xn = np.linalg.norm(x)
            if xn == 0 and alpha_r.imag == 0:
                tau, beta = 0.0, alpha_r.real
                v = np.zeros(n, complex)
                v[i + 1] = 1.0
            else:
                beta = -np.copysign(np.sqrt(abs(alpha_r) ** 2 + xn ** 2), alpha_r.real)
                tau = (beta - alpha_r.real) / beta - 1j * alpha_r.imag / beta
                v = np.zeros(n, complex)
                v[i + 1] = 1.0
                v[i + 2:] = x / (alpha_r - beta)
            e[i] = beta
            A[i + 1:, i] = v[i + 1:]
            y = np.zeros(n, complex)
            y[i + 1:] = A22[i + 1:, i + 1:] @ v[i + 1:]
            x1 = V[i + 1:].conj().T @ v[i + 1:]
            x2 = W[i + 1:, :jj].conj().T @ v[i + 1:]
            w = np.zeros(n, complex)
            w[i + 1:] = tau * (y[i + 1:] - W[i + 1:, :jj] @ x1 - V[i + 1:] @ x2)
            W[:, jj] = w
            alpha = -0.5 * tau * np.vdot(w[i + 1:], v[i + 1:])
            if fused and jj + 1 < jb:  # the corrections kernel's share of column i+1's update
                for c in range(jj):
                    A[i + 1:, i + 1] -= (A[i + 1:, k0 + c] * np.conj(W[i + 1, c]) +
                                         W[i + 1:, c] * np.conj(A[i + 1, k0 + c]))
            if jj == jb - 1 or i == n - 2:
                W[:, jj] += alpha * v  # last column of the panel (or matrix): completed at once
            else:
                pending = (jj, alpha)
        k1 = k0 + jb
        if k1 < n:
            Vp = A[k1:, k0:k1]
            Wp = W[k1:, :]
            A[k1:, k1:] -= Vp @ Wp.conj().T + Wp @ Vp.conj().T
    return d, e


def test_fused_and_plain_orders_give_the_same_tridiagonal():
    rng = np.random.default_rng(9)
    for n, nb in [(50, 8), (37, 32), (70, 16), (9, 4)]:
        A0 = _hermitian(rng, n)
        d0, e0 = _reduce(A0, nb, fused=False)
        d1, e1 = _reduce(A0, nb, fused=True)
        np.testing.assert_allclose(d1, d0, rtol=0, atol=1e-11 * np.abs(A0).max())
        np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-11 * np.abs(A0).max())
        T = np.diag(d1) + np.diag(e1, 1) + np.diag(e1, -1)
        np.testing.assert_allclose(np.linalg.eigvalsh(T), np.linalg.eigvalsh(A0), atol=1e-10 * np.abs(A0).max())
