"""Shared comparison rules for the GPU parity tests.

Frequencies: |dw| < 1e-4 cm^-1 absolute or 1e-8 relative for |w| >= W_MIN;
below W_MIN (acoustic modes at/near Gamma, where the square root amplifies
FP64 rounding) the eigenvalues of D are compared: |dlambda| <= 64 n eps ||D||.
Velocities: per mode |dv| <= 1e-6 max(|v|, 1e-3 max|v|) on modes whose
eigenvalue is separated from its neighbours by more than 1e-6 ||D||; inside
clusters closer than that (degenerate or nearly so) the per-mode velocity is
basis dependent and the cluster sums are compared with the same rule.
max|v| is taken over every mode and q-point of the compared set.  Modes at
the reference's clamp (2|w| < 1e-3 cm^-1: the acoustic modes at Gamma) have
a numerator at the eigensolver's backward-error level divided by the clamp
constant, i.e. rounding noise: a normwise perturbation of 1e-15 ||D|| moves
their cluster sum by ~1e-6 m/s, 1e-14 by ~3e-5 m/s.  They are compared with
|dv| <= 1e-7 max|v| (a few mm/s on a 2e4 m/s band).
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
CLAMP = 1e-3      # write_output.F90:443: v = Re(e^H dD e) / max(2|w|, 1e-3)
V_CLAMP = 1e-7


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
    w_ref = np.sign(lam_ref) * np.sqrt(np.abs(lam_ref)) * O.C1 * O.C2
    worst = 0.0
    for g in clusters(lam_ref, Dnorm):
        a = v_gpu[g].sum(axis=0)
        b = v_ref[g].sum(axis=0)
        if np.all(2.0 * np.abs(w_ref[g]) < CLAMP):
            # the reference divides by its clamp constant: rounding noise only
            assert np.all(np.abs(a - b) <= V_CLAMP * vmax), (g, a, b)
            continue
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
