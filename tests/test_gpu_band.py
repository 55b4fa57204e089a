"""The two-stage reduction (dense -> band -> tridiagonal, mixed form) against
the oracle: frequencies, per-mode velocities (rows-only back-transform
through both stages), eigenvectors (full back-transform through both
stages), range I; and the same results as the one-stage reduction."""
import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import api, synth
from tests import parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cell148():
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    S = O.System.from_cell(c, phi)
    ctx = api.PhononContext.from_cell(c, phi)
    yield S, ctx
    ctx.close()


def _check(S, ctx, qs, opts, want_z):
    res = ctx.solve(qs, opts, want_z=want_z)
    refs = [O.solve_q(S, q, jobz="V" if (opts.jobz == "V" or opts.vel) else "N", rng=opts.range, il=opts.il,
                      iu=opts.iu, vel=opts.vel, vel_method=opts.vel_method) for q in qs]
    vmax = max(np.abs(r["vel"]).max() for r in refs) if opts.vel else 0.0
    out = []
    for t, q in enumerate(qs):
        ref = refs[t]
        m = len(ref["w_cm"])
        assert res.m[t] == m and res.info[t] == 0, (res.m[t], m, res.info[t])
        Dn = np.abs(np.linalg.eigvalsh(S.dynmat(q))).max()
        st = {"dw": parity.check_frequencies(res.w[t, :m], ref["w_cm"], ref["lam"], S.n, Dn)}
        if want_z and (opts.jobz == "V" or opts.vel):
            st["res"], st["orth"] = parity.check_vectors(res.z[t][:, :m], ref["lam"], S.dynmat(q), 1e-11, 1e-10)
        if opts.vel:
            st["dv"] = parity.check_velocities(res.vel[t, :m], ref["vel"], ref["lam"], Dn, vmax)
        out.append(st)
    return out


def test_band_velocities_rows_only(cell148, monkeypatch):
    monkeypatch.setenv("PARPHOM_GPU_BAND", "1")
    S, ctx = cell148
    qs = synth.random_qpoints(3, seed=41)
    print(_check(S, ctx, qs, api.EigOpts(jobz="N", vel=True, precision=api.PP_PREC_MIXED), want_z=False))


def test_band_vectors_and_range_index(cell148, monkeypatch):
    monkeypatch.setenv("PARPHOM_GPU_BAND", "1")
    S, ctx = cell148
    qs = synth.band_path(9)[[2, 5]]
    print(_check(S, ctx, qs, api.EigOpts(jobz="V", vel=True, precision=api.PP_PREC_MIXED), want_z=True))
    print(_check(S, ctx, qs, api.EigOpts(jobz="V", range="I", il=3, iu=80, vel=True, precision=api.PP_PREC_MIXED),
                 want_z=True))


def test_band_matches_one_stage_n1092(monkeypatch):
    c = synth.tblg_cell(5)
    phi = synth.spring_force_constants(c, seed=0)
    qs = synth.random_qpoints(4, seed=43)
    opts = api.EigOpts(jobz="N", vel=True, precision=api.PP_PREC_MIXED)
    with api.PhononContext.from_cell(c, phi) as ctx:
        monkeypatch.setenv("PARPHOM_GPU_BAND", "0")
        one = ctx.solve(qs, opts, want_z=False)
        monkeypatch.setenv("PARPHOM_GPU_BAND", "1")
        two = ctx.solve(qs, opts, want_z=False)
    assert np.all(two.info == 0)
    big = np.abs(one.w) >= 1.0
    assert np.abs(one.w - two.w)[big].max() < 1e-6
    vmax = np.abs(one.vel).max()
    assert np.abs(one.vel - two.vel).max() < 1e-5 * vmax
