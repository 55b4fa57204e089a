"""GPU path (C-ABI library) against the oracle, same inputs."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import api, geometry, synth
from tests import parity

pytestmark = pytest.mark.gpu

PRECS = [api.PP_PREC_FP64, api.PP_PREC_MIXED]


@pytest.fixture(scope="module")
def tblg28(golden_dir):
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    S = O.System(z["lat"], z["real_pos"], z["masses"], z["at_types"], z["phi"])
    ctx = api.PhononContext(z["lat"], S.crys, z["real_pos"], z["masses"], z["at_types"], z["phi"])
    yield S, ctx, z
    ctx.close()


@pytest.fixture(scope="module")
def cell148():
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    S = O.System.from_cell(c, phi)
    ctx = api.PhononContext.from_cell(c, phi)
    yield S, ctx
    ctx.close()


@pytest.mark.parametrize("deriv,method", [(0, "A"), (1, "A"), (2, "A"), (3, "A"), (1, "C"), (2, "C")])
def test_dynamical_matrix_elements(tblg28, cell148, deriv, method):
    for S, ctx in ((tblg28[0], tblg28[1]), cell148):
        for q in ([0.0, 0.0, 0.0], [0.31, -0.12, 0.0], [2 / 3, 1 / 3, 0.0]):
            Dg = ctx.dynamical_matrix(q, deriv, method)
            Dr = S.dynmat(q, deriv, method)
            scale = np.abs(Dr).max()
            tol = (1e-13 if method == "A" else 1e-7) * scale
            assert np.abs(Dg - Dr).max() <= tol, (deriv, method, np.abs(Dg - Dr).max() / scale)


def _solve_and_check(S, ctx, qs, prec, vel_method="A", rng="A", il=1, iu=1, vl=0.0, vu=0.0, jobz="V", vel=True):
    opts = api.EigOpts(jobz=jobz, range=rng, il=il, iu=iu, vl=vl, vu=vu, vel=vel, vel_method=vel_method,
                       precision=prec)
    res = ctx.solve(qs, opts)
    n = S.n
    stats = []
    refs = [O.solve_q(S, q, jobz=jobz, rng=rng, il=il, iu=iu, vl=vl, vu=vu, vel=vel, vel_method=vel_method)
            for q in qs]
    # velocity scale of the whole q set (at Gamma every velocity is rounding noise)
    vmax = max(np.abs(r["vel"]).max() for r in refs) if vel else 0.0
    for t, q in enumerate(qs):
        ref = refs[t]
        m = len(ref["w_cm"])
        assert res.m[t] == m
        assert res.info[t] == 0
        D = S.dynmat(q)
        Dn = np.abs(np.linalg.eigvalsh(D)).max()
        werr = parity.check_frequencies(res.w[t, :m], ref["w_cm"], ref["lam"], n, Dn)
        st = {"werr": werr}
        if jobz == "V" or vel:
            assert res.nz[t] == m
            Z = res.z[t][:, :m]
            st["res"], st["orth"] = parity.check_vectors(Z, ref["lam"], D, 1e-11, 1e-10)
        if vel:
            st["vrel"] = parity.check_velocities(res.vel[t, :m], ref["vel"], ref["lam"], Dn, vmax)
        stats.append(st)
    return res, stats


@pytest.mark.parametrize("prec", PRECS)
def test_shipped_cell_bands(tblg28, prec):
    S, ctx, z = tblg28
    qs = np.vstack([z["q_symm"], [[0, 0, 0]], z["q_band"][[17, 133, 250]]])
    _, st = _solve_and_check(S, ctx, qs, prec)
    print(prec, st)


@pytest.mark.parametrize("prec", PRECS)
def test_synthetic_148_band_path(cell148, prec):
    S, ctx = cell148
    qs = synth.band_path(7)
    _, st = _solve_and_check(S, ctx, qs, prec)
    print(prec, st)


@pytest.mark.parametrize("prec", PRECS)
def test_central_difference_velocities(cell148, prec):
    S, ctx = cell148
    qs = synth.random_qpoints(3, seed=5)
    _solve_and_check(S, ctx, qs, prec, vel_method="C")


@pytest.mark.parametrize("prec", PRECS)
def test_range_index(cell148, prec):
    S, ctx = cell148
    qs = synth.random_qpoints(2, seed=6)
    _solve_and_check(S, ctx, qs, prec, rng="I", il=5, iu=60, jobz="N", vel=False)
    _solve_and_check(S, ctx, qs, prec, rng="I", il=100, iu=180, jobz="V", vel=True)


@pytest.mark.parametrize("prec", PRECS)
def test_range_value(cell148, prec):
    S, ctx = cell148
    qs = synth.random_qpoints(2, seed=7)
    # bounds in the reference's units: they are divided by 15.633302*33.35641
    # and compared with lambda = omega^2, so lambda in (0.5, 3.0] here
    _solve_and_check(S, ctx, qs, prec, rng="V", vl=0.5 * O.C_RANGE, vu=3.0 * O.C_RANGE, jobz="V", vel=True)
    # an empty interval gives m = 0
    res = ctx.solve(qs[:1], api.EigOpts(range="V", vl=1e-9, vu=2e-9, jobz="N", precision=prec))
    assert res.m[0] == 0 and res.info[0] == 0


def test_eigenvalues_only_many_q(cell148):
    S, ctx = cell148
    qs = synth.uniform_grid(4)
    _solve_and_check(S, ctx, qs, api.PP_PREC_FP64, jobz="N", vel=False)


def test_errors(cell148):
    S, ctx = cell148
    with pytest.raises(api.PPError) as e:
        ctx.solve([[0, 0, 0]], api.EigOpts(range="I", il=5, iu=2))
    assert e.value.code == -5
    with pytest.raises(api.PPError) as e:
        ctx.solve([[np.nan, 0, 0]], api.EigOpts())
    assert e.value.code == 1003
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c)
    phi[0, 5] = np.inf
    with pytest.raises(api.PPError) as e:
        api.PhononContext.from_cell(c, phi)
    assert e.value.code == 1003


@pytest.mark.parametrize("prec", PRECS)
def test_velocities_without_vectors(cell148, prec):
    """Velocities when no eigenvectors are returned use only the eigenvector
    rows of atoms in boundary blocks (Q^H P^T, then X^H Z); same results."""
    S, ctx = cell148
    qs = synth.random_qpoints(3, seed=9)
    for rng, il, iu in (("A", 1, 1), ("I", 40, 200)):
        opts = api.EigOpts(jobz="N", range=rng, il=il, iu=iu, vel=True, vel_method="A", precision=prec)
        res = ctx.solve(qs, opts, want_z=False)
        full = ctx.solve(qs, opts, want_z=True)
        refs = [O.solve_q(S, q, rng=rng, il=il, iu=iu, vel=True) for q in qs]
        vmax = max(np.abs(r["vel"]).max() for r in refs)
        for t, q in enumerate(qs):
            ref = refs[t]
            m = len(ref["w_cm"])
            assert res.m[t] == m and res.info[t] == 0
            Dn = np.abs(np.linalg.eigvalsh(S.dynmat(q))).max()
            parity.check_velocities(res.vel[t, :m], ref["vel"], ref["lam"], Dn, vmax)
            np.testing.assert_allclose(res.vel[t, :m], full.vel[t, :m], rtol=0, atol=1e-7 * vmax)


@pytest.mark.parametrize("prec", PRECS)
def test_uneven_cells_one_batch(tblg28, cell148, prec):
    """pp_solve_multi: q-points of three cells of different size (N = 28,
    148, 364) interleaved, solved in shared batches; each result must equal
    the single-cell solve of the same q."""
    S28, ctx28, _ = tblg28
    S148, ctx148 = cell148
    c364 = synth.tblg_cell(5)
    phi364 = synth.spring_force_constants(c364, seed=0)
    ctx364 = api.PhononContext.from_cell(c364, phi364)
    ctxs = [ctx28, ctx148, ctx364]
    rng = np.random.default_rng(12)
    cell = rng.integers(0, 3, 9)
    q = synth.random_qpoints(9, seed=13)
    for want_z in (False, True):
        opts = api.EigOpts(jobz="V" if want_z else "N", vel=True, vel_method="A", precision=prec)
        res = api.solve_multi(ctxs, cell, q, opts, want_z=want_z)
        for t in range(9):
            c = ctxs[cell[t]]
            single = c.solve(q[t:t + 1], opts, want_z=want_z)
            n = c.n
            assert res.m[t] == n and res.info[t] == 0
            np.testing.assert_allclose(res.w[t, :n], single.w[0, :n], rtol=1e-12, atol=1e-9)
            vmax = np.abs(single.vel[0, :n]).max()
            np.testing.assert_allclose(res.vel[t, :n], single.vel[0, :n], rtol=0, atol=1e-9 * vmax)
            if want_z:
                Z, Zs = res.z[t][:n, :n], single.z[0][:, :n]
                ov = np.abs(np.einsum("ij,ij->j", Z.conj(), Zs))
                assert np.abs(ov - 1).max() < 1e-9
    ctx364.close()


@pytest.mark.parametrize("prec", PRECS)
def test_error_estimates(cell148, prec):
    """Per-eigenpair error estimates (want_resid): the residual equals an
    independent FP64 residual of the returned pair, the frequency bound covers
    the difference to the oracle, and the eigenvector bound covers the angle
    to the oracle's eigenvector for well-separated modes."""
    S, ctx = cell148
    qs = synth.random_qpoints(2, seed=21)
    res = ctx.solve(qs, api.EigOpts(jobz="V", vel=True, want_resid=True, precision=prec))
    fast = ctx.solve(qs, api.EigOpts(jobz="N", vel=True, want_resid=True, precision=prec), want_z=False)
    n = S.n
    eps = np.finfo(float).eps
    cw = O.C1 * O.C2
    for t, q in enumerate(qs):
        ref = O.solve_q(S, q, jobz="V")
        D = S.dynmat(q)
        lam_ref = ref["lam"]
        Dn = np.abs(lam_ref).max()
        w, z = res.w[t, :n], res.z[t][:, :n]
        lam = np.sign(w) * (w / cw) ** 2
        # the estimates come with or without returned eigenvectors (values at
        # the rounding level of the FP64 residual product: compared loosely)
        assert np.all(np.isfinite(fast.werr[t, :n])) and fast.resid[t, :n].max() <= 1e-11 * Dn
        assert np.all(np.abs(fast.werr[t, :n] - res.werr[t, :n]) <= 0.5 * res.werr[t, :n] + 1e-12)
        r_np = np.linalg.norm(D @ z - z * lam[None, :], axis=0)
        assert np.all(np.abs(res.resid[t, :n] - r_np) <= 0.2 * r_np + 1e-14 * Dn), \
            np.abs(res.resid[t, :n] - r_np).max()
        assert res.resid[t, :n].max() <= 1e-11 * Dn
        # frequency bound vs the oracle (its own error: a few n eps ||D|| in lambda)
        big = np.abs(ref["w_cm"]) >= 1.0
        dlo = 4 * n * eps * Dn
        oracle_w = cw * dlo / (2 * np.sqrt(np.abs(lam_ref)))
        dw = np.abs(w - ref["w_cm"])
        assert np.all((dw <= res.werr[t, :n] + oracle_w)[big])
        assert res.werr[t, :n][big].max() <= 1e-4
        # eigenvector bound on well-separated modes
        gaps = np.minimum(np.diff(lam_ref, prepend=-np.inf), np.diff(lam_ref, append=np.inf))
        sep = gaps > 1e-6 * Dn
        # sin(angle) as the norm of the part of z orthogonal to the oracle's
        # vector (no cancellation, unlike sqrt(1 - |z^H z_ref|^2))
        zh = z / np.linalg.norm(z, axis=0)[None, :]
        proj = ref["z"] * np.einsum("ij,ij->j", ref["z"].conj(), zh)[None, :]
        sin = np.linalg.norm(zh - proj, axis=0)
        oracle_z = 4 * n * eps * Dn / gaps
        assert np.all((sin <= res.zerr[t, :n] + oracle_z + 1e-7)[sep])
