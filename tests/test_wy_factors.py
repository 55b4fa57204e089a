"""The compact-WY factor of a panel of Householder reflectors, as the
back-transform forms it (k_wy_factors), restated in numpy and checked
against the explicit product of the reflectors.

A panel of jb reflectors H_a = I - tau_a v_a v_a^H (v_a zero above row
k0 + a + 1, one there, as the reduction stores them) multiplies out to
H_0 H_1 ... H_{jb-1} = I - V Tf V^H with Tf upper triangular from the
Gram matrix G = V^H V by zlarft's forward columnwise recurrence:
Tf(a, a) = tau_a, Tf(0:a, a) = -tau_a Tf(0:a, 0:a) G(0:a, a).  The
back-transform applies Q = I - V Tf V^H (mode 1, E <- Q E) and
Q^H = I - V Tf^H V^H (mode 2, the rows-only path).  Reflectors past a
matrix's own order carry tau = 0 and give zero columns of Tf."""
import numpy as np


def _panel(rng, n, k0, jb, zero_from=None):
    """Reflector vectors in the reduction's storage pattern; the recurrence is
    an identity for any complex tau, so tau is drawn at random (zlarfg's
    would make each H_a unitary)."""
    V = np.zeros((n, jb), complex)
    tau = np.zeros(jb, complex)
    for a in range(jb):
        r = k0 + a + 1
        if r >= n or (zero_from is not None and k0 + a >= zero_from):
            continue
        V[r, a] = 1.0
        V[r + 1:, a] = rng.standard_normal(n - r - 1) + 1j * rng.standard_normal(n - r - 1)
        tau[a] = rng.standard_normal() + 1j * rng.standard_normal()
    return V, tau


def _tf(V, tau):
    jb = V.shape[1]
    G = V.conj().T @ V
    T = np.zeros((jb, jb), complex)
    for jj in range(jb):
        acc = np.array([T[a, a:jj] @ G[a:jj, jj] for a in range(jj)], complex)
        T[:jj, jj] = -tau[jj] * acc
        T[jj, jj] = tau[jj]
    return T


def _product(V, tau):
    n = V.shape[0]
    Q = np.eye(n, dtype=complex)
    for a in range(V.shape[1]):
        Q = Q @ (np.eye(n) - tau[a] * np.outer(V[:, a], V[:, a].conj()))
    return Q


def test_wy_factor_reproduces_reflector_product():
    rng = np.random.default_rng(4)
    for n, k0, jb in [(40, 0, 32), (75, 32, 32), (50, 40, 9), (33, 0, 31)]:
        V, tau = _panel(rng, n, k0, jb)
        T = _tf(V, tau)
        assert np.allclose(np.tril(T, -1), 0)
        Q = _product(V, tau)
        np.testing.assert_allclose(np.eye(n) - V @ T @ V.conj().T, Q, atol=1e-12)
        # mode 2 applies Q^H with Tf^H
        np.testing.assert_allclose(np.eye(n) - V @ T.conj().T @ V.conj().T, Q.conj().T, atol=1e-12)


def test_wy_factor_zero_past_the_matrix_order():
    """A batch's panels follow its largest order; for a smaller matrix the
    reflectors from its own order on have tau = 0 (and zero vectors), so Tf
    has zero columns there and the panel acts as the identity on them."""
    rng = np.random.default_rng(5)
    n, k0, jb = 60, 32, 32
    V, tau = _panel(rng, n, k0, jb, zero_from=45)
    T = _tf(V, tau)
    assert np.all(T[:, 45 - k0:] == 0)
    np.testing.assert_allclose(np.eye(n) - V @ T @ V.conj().T, _product(V, tau), atol=1e-12)
