"""Differentiation: dL/dq and dL/dPhi of L = sum (w - w_target)^2 through the
torch.autograd.Function, against central finite differences of the same GPU
forward and against an FP64 gradient built from the oracle's eigenvectors
(M = Z diag(dL/dlambda) Z^H, G = Re(M^T o P)).

The finite differences use h = 1e-5 with one Richardson step,
(4 d(h/2) - d(h)) / 3: near avoided crossings (pairs 0.1 cm^-1 apart in this
cell) the plain central difference carries an O(h^2) error of up to 4e-4
relative at h = 1e-5, which the extrapolation removes."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import api, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(golden_dir):
    import torch
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    phi = z["phi"]
    phi_t = synth.spring_force_constants  # noqa: F841  (target from a seeded perturbation below)
    rng = np.random.default_rng(11)
    pert = 1.0 + 0.03 * rng.uniform(-1, 1, phi.shape)
    pert = 0.5 * (pert + pert.T)
    target_phi = phi * pert
    q = np.array([[0.137, 0.071, 0.0], [0.41, -0.23, 0.0]])
    S = O.System(z["lat"], z["real_pos"], z["masses"], z["at_types"], target_phi)
    target = np.stack([O.solve_q(S, qq)["w_cm"] for qq in q])
    return z, phi, q, torch.tensor(target)


def _loss(spec, q, phi, target):
    w = spec.frequencies(q, phi)
    return ((w - target) ** 2).sum()


def _fd(f, x, d, h=1e-5):
    """Richardson-extrapolated central difference of f along d at x."""
    def cd(hh):
        return (f(x + hh * d) - f(x - hh * d)) / (2 * hh)
    return (4 * cd(h / 2) - cd(h)) / 3


@pytest.mark.parametrize("prec", [api.PP_PREC_FP64, api.PP_PREC_MIXED])
def test_grad_q_and_phi_vs_fd(setup, prec):
    import torch
    from parphom_gb300.autograd import PhononSpectrum
    z, phi, q, target = setup
    spec = PhononSpectrum(z["lat"], z["real_pos"], z["masses"], z["at_types"], precision=prec, batch=2)
    qt = torch.tensor(q, requires_grad=True)
    pt = torch.tensor(phi, requires_grad=True)
    L = _loss(spec, qt, pt, target)
    L.backward()
    gq, gp = qt.grad.numpy(), pt.grad.numpy()
    assert np.allclose(gp, gp.T)
    # finite differences of the FP64 forward (differences of the mixed forward
    # are limited by its ~1e-10 cm^-1 rounding noise divided by h)
    ref = PhononSpectrum(z["lat"], z["real_pos"], z["masses"], z["at_types"], precision=api.PP_PREC_FP64, batch=2)
    Lq = lambda x: _loss(ref, torch.tensor(x), torch.tensor(phi), target).item()  # noqa: E731
    Lp = lambda x: _loss(ref, torch.tensor(q), torch.tensor(x), target).item()  # noqa: E731
    # dL/dq in each in-plane reduced coordinate (kz does not enter: 2D cell)
    for t in range(q.shape[0]):
        for k in range(2):
            d = np.zeros_like(q)
            d[t, k] = 1.0
            fd = _fd(Lq, q, d)
            assert abs(fd - gq[t, k]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(gq).max()), (t, k, fd, gq[t, k])
    # dL/dPhi: directional derivatives along random symmetric directions
    rng = np.random.default_rng(3)
    for _ in range(3):
        d = rng.standard_normal(phi.shape)
        d = 0.5 * (d + d.T)
        fd = _fd(Lp, phi, d)
        an = float((gp * d).sum())
        assert abs(fd - an) <= 1e-6 * abs(fd), (fd, an)


def test_grad_phi_vs_fp64_oracle(setup):
    import torch
    from parphom_gb300.autograd import PhononSpectrum, C_OMEGA
    z, phi, q, target = setup
    spec = PhononSpectrum(z["lat"], z["real_pos"], z["masses"], z["at_types"], precision=api.PP_PREC_MIXED)
    pt = torch.tensor(phi, requires_grad=True)
    L = _loss(spec, torch.tensor(q), pt, target)
    L.backward()
    G = pt.grad.numpy()
    # oracle gradient
    S = O.System(z["lat"], z["real_pos"], z["masses"], z["at_types"], phi)
    S1 = O.System(z["lat"], z["real_pos"], z["masses"], z["at_types"], np.ones_like(phi))
    Gref = np.zeros_like(phi)
    for t, qq in enumerate(q):
        r = O.solve_q(S, qq, jobz="V")
        w = r["w_cm"]
        gw = 2 * (w - target[t].numpy())
        c = gw * C_OMEGA ** 2 / np.maximum(2 * np.abs(w), 1e-3)
        M = (r["z"] * c[None, :]) @ r["z"].conj().T
        P = S1.dynmat(qq)                      # phase/mass factor of each element
        Pu = np.triu(P) + np.triu(P, 1).conj().T   # upper triangle defines D
        Gref += np.real(M.T * Pu)
    scale = np.abs(Gref).max()
    assert np.abs(G - Gref).max() <= 1e-8 * scale, np.abs(G - Gref).max() / scale


def test_grad_q_vs_cd_velocities_n148():
    """dL/dq at N = 148 (device tensors end to end) against the
    central-difference group velocities of the library: for L = sum g_j w_j,
    dL/dq = sum_j g_j dw_j/dq with dw_j/dk the CD velocity over the
    reference's unit factor; g is constant over degenerate clusters (where
    only the cluster sums are basis independent)."""
    import torch
    from parphom_gb300.autograd import PhononSpectrum, C_OMEGA, VEL_FACTOR, cluster_mean
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    dev = torch.device("cuda", 0)
    spec = PhononSpectrum.from_cell(c, precision=api.PP_PREC_MIXED, batch=4)
    qs = synth.random_qpoints(5, seed=17)
    q = torch.tensor(qs, device=dev, requires_grad=True)
    pt = torch.tensor(phi, device=dev)
    w = spec.frequencies(q, pt)
    assert w.is_cuda
    lam = torch.sign(w.detach()) * (w.detach() / C_OMEGA) ** 2
    g = cluster_mean(lam, torch.linspace(-1.0, 1.0, w.shape[1], device=dev, dtype=torch.float64).expand_as(w))
    (g * w).sum().backward()
    assert q.grad.is_cuda
    with api.PhononContext.from_cell(c, phi) as ctx:
        r = ctx.solve(qs, api.EigOpts(jobz="N", vel=True, vel_method="C", precision=api.PP_PREC_FP64),
                      want_z=False)
    a = np.abs(r.w)
    dwdk = r.vel * (C_OMEGA ** 2 / VEL_FACTOR) * (np.maximum(2 * a, 1e-3) / np.maximum(2 * a, 1e-300))[..., None]
    dwdq = dwdk @ spec.rec_lat.T
    expect = np.einsum("tn,tnk->tk", g.cpu().numpy(), dwdq)
    got = q.grad.cpu().numpy()
    scale = np.abs(expect).max()
    assert np.abs(got - expect).max() <= 1e-6 * scale, np.abs(got - expect).max() / scale
    # a second forward with changed force constants reuses the context
    h = spec._ctx._h.value
    w2 = spec.frequencies(q.detach(), pt * 1.01)
    assert spec._ctx._h.value == h
    np.testing.assert_allclose(w2.cpu().numpy(), w.detach().cpu().numpy() * np.sqrt(1.01), rtol=1e-9)
    spec.close()
