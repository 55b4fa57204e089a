"""Shared comparison rules for the GPU parity tests.

Frequencies: |dw| < 1e-4 cm^-1 absolute or 1e-8 relative for |w| >= W_MIN;
below W_MIN (acoustic modes at/near Gamma, where the square root amplifies
FP64 rounding) the eigenvalues of D are compared: |dlambda| <= 64 n eps ||D||.
Velocities: per mode |dv| <= 1e-6 max(|v|, 1e-3 max|v|) on modes whose
eigenvalue is separated from its neighbours by more than 1e-6 ||D||; inside
clusters closer than that (degenerate or nearly so) the per-mode velocity is
basis dependent and the cluster sums are compared with the same rule.
max|v| is taken over every mode and q-point of the compared set: at Gamma
all velocities are rounding noise divided by the reference's 1e-3 clamp, so
a per-q scale would ask for agreement of that noise.
Eigenvectors: residual ||D z - lambda z|| <= RES_TOL ||D|| and
||Z^H Z - I||_max <= ORTH_TOL, plus per-cluster projector distance.
"""
import numpy as np

from oracle import oracle as O

W_MIN = 1.0
W_ABS = 1e-4
W_REL = 1e-8
V_REL = 1e-6
GAP_REL = 1e-6


def clusters(lam, norm):
    groups, cur = [], [0]
    for j in range(1, len(lam)):
        if lam[j] - lam[j - 1] <= GAP_REL * norm:
            cur.append(j)
        else:
            groups.append(cur)
            cur = [j]
    groups.append(cur)
    return groups


def check_frequencies(w_gpu, w_ref, lam_ref, n, Dnorm):
    w_gpu = np.asarray(w_gpu)
    assert w_gpu.shape == w_ref.shape, (w_gpu.shape, w_ref.shape)
    big = np.abs(w_ref) >= W_MIN
    err = np.abs(w_gpu - w_ref)
    ok = (err <= W_ABS) | (err <= W_REL * np.abs(w_ref))
    bad = np.where(big & ~ok)[0]
    assert len(bad) == 0, f"frequency mismatch at modes {bad[:10]}: {err[bad[:10]]}"
    if (~big).any():
        lam_gpu = np.sign(w_gpu) * (w_gpu / (O.C1 * O.C2)) ** 2
        dl = np.abs(lam_gpu[~big] - lam_ref[~big])
        assert dl.max() <= 64 * n * np.finfo(float).eps * Dnorm, dl.max()
    return float(err[big].max()) if big.any() else 0.0


def check_velocities(v_gpu, v_ref, lam_ref, Dnorm, vmax):
    floor = max(1e-3 * vmax, 1e-6)
    worst = 0.0
    for g in clusters(lam_ref, Dnorm):
        a = v_gpu[g].sum(axis=0)
        b = v_ref[g].sum(axis=0)
        tol = V_REL * np.maximum(np.abs(b), floor)
        rel = np.abs(a - b) / np.maximum(np.abs(b), floor)
        worst = max(worst, float(rel.max()))
        assert np.all(np.abs(a - b) <= tol), (g, a, b)
    return worst


def check_vectors(Z, lam, D, res_tol, orth_tol):
    if Z.shape[1] == 0:
        return 0.0, 0.0
    Dn = np.abs(np.linalg.eigvalsh(D)).max()
    R = D @ Z - Z * lam[None, :]
    res = np.linalg.norm(R, axis=0).max() / Dn
    orth = np.abs(Z.conj().T @ Z - np.eye(Z.shape[1])).max()
    assert res <= res_tol, res
    assert orth <= orth_tol, orth
    return res, orth
