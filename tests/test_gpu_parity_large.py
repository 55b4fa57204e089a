"""Oracle parity at the sizes the benchmark is quoted on.

* N = 868 (theta = 3.89 deg, n = 2604): 3 q-points on the band path,
  eigenvectors + analytic group velocities, both precision forms.
* N = 1588 (theta = 2.88 deg, n = 4764): 1 q-point off Gamma, frequencies +
  analytic group velocities without eigenvector output (the rows-only
  back-transform the benchmark times), both precision forms.

Same rules as the small-cell tests (tests/parity.py): |dw| < 1e-4 cm^-1 or
1e-8 relative (lambda-space rule below 1 cm^-1), per-mode velocities to
1e-6 relative with cluster sums inside near-degenerate clusters, residual
and orthogonality of the eigenvectors.  The oracle (LAPACK zheevx on the C
restatement of D(q)) runs once per q and serves both forms.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import api, synth
from tests import parity

pytestmark = pytest.mark.gpu

PRECS = [api.PP_PREC_FP64, api.PP_PREC_MIXED]


def _cell(m):
    c = synth.tblg_cell(m)
    phi = synth.spring_force_constants(c, seed=0)
    return c, phi


@pytest.fixture(scope="module")
def n868():
    c, phi = _cell(8)
    S = O.System.from_cell(c, phi)
    qs = synth.band_path(128)[[5, 47, 90]]
    refs = [O.solve_q(S, q, jobz="V", vel=True, vel_method="A") for q in qs]
    ctx = api.PhononContext.from_cell(c, phi)
    yield S, ctx, qs, refs
    ctx.close()


@pytest.fixture(scope="module")
def n1588():
    c, phi = _cell(11)
    S = O.System.from_cell(c, phi)
    qs = synth.band_path(128)[[3]]   # the benchmark's own sample q, off Gamma
    refs = [O.solve_q(S, q, vel=True, vel_method="A") for q in qs]
    ctx = api.PhononContext.from_cell(c, phi)
    yield S, ctx, qs, refs
    ctx.close()


def _check(S, qs, refs, res, vectors):
    n = S.n
    vmax = max(np.abs(r["vel"]).max() for r in refs)
    out = []
    for t, q in enumerate(qs):
        ref = refs[t]
        assert res.m[t] == n and res.info[t] == 0
        D = S.dynmat(q)
        Dn = np.abs(ref["lam"]).max()
        st = {"dw": parity.check_frequencies(res.w[t, :n], ref["w_cm"], ref["lam"], n, Dn),
              "dv": parity.check_velocities(res.vel[t, :n], ref["vel"], ref["lam"], Dn, vmax)}
        if vectors:
            assert res.nz[t] == n
            st["res"], st["orth"] = parity.check_vectors(res.z[t][:, :n], ref["lam"], D, 1e-11, 1e-10)
        out.append(st)
    return out


@pytest.mark.parametrize("prec", PRECS)
def test_n868_vectors_and_velocities(n868, prec):
    S, ctx, qs, refs = n868
    res = ctx.solve(qs, api.EigOpts(jobz="V", vel=True, vel_method="A", precision=prec))
    print(prec, _check(S, qs, refs, res, vectors=True))


@pytest.mark.parametrize("prec", PRECS)
def test_n1588_frequencies_and_velocities(n1588, prec):
    S, ctx, qs, refs = n1588
    res = ctx.solve(qs, api.EigOpts(jobz="N", vel=True, vel_method="A", precision=prec), want_z=False)
    print(prec, _check(S, qs, refs, res, vectors=False))


def test_n1588_vectors_with_subnormal_tails():
    """Band-path q-points 64 and 80 at N=1588 have eigenvectors whose far
    components fall below the single-precision normal range at some stage
    of the back-transform; the tensor-core long-K slicing scales such row
    chunks in two exact steps.  Every column must be finite and the pairs
    must keep their residual and orthogonality (mixed form, full vectors)."""
    import torch
    c, phi = _cell(11)
    ctx = api.PhononContext.from_cell(c, phi)
    try:
        qs = synth.band_path(128)[[64, 80]]
        res = ctx.solve(qs, api.EigOpts(jobz="V", precision=api.PP_PREC_MIXED))
        dev = torch.device("cuda")
        cw = float(np.float32(15.633302)) * float(np.float32(33.35641))
        for t in range(len(qs)):
            n = ctx.n
            assert res.m[t] == n and res.info[t] == 0
            Z = torch.as_tensor(res.z[t][:, :n], device=dev)
            assert bool(torch.isfinite(Z.real).all()) and bool(torch.isfinite(Z.imag).all())
            D = torch.as_tensor(ctx.dynamical_matrix(qs[t]), device=dev)
            lam = torch.as_tensor(np.sign(res.w[t, :n]) * (res.w[t, :n] / cw) ** 2, device=dev)
            dn = float(torch.abs(D).sum(dim=0).max())
            resid = float((torch.linalg.vector_norm(D @ Z - Z * lam[None, :], dim=0).max() / dn))
            orth = float(torch.abs(Z.conj().T @ Z - torch.eye(n, dtype=Z.dtype, device=dev)).max())
            assert resid < 1e-11 and orth < 1e-10, (resid, orth)
    finally:
        ctx.close()
