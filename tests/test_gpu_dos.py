"""GPU density of states against the oracle restatement of the reference's
BZ-integration routines, on frequencies computed by the GPU path for a
6x6 grid of the shipped 28-atom cell."""
import os

import numpy as np
import pytest

from oracle import dos_ref
from parphom_gb300 import api, dos, geometry, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid_freqs(golden_dir):
    z = np.load(os.path.join(golden_dir, "tblg21_8_inputs.npz"))
    crys = geometry.crys_from_positions(z["lat"], z["real_pos"])
    with api.PhononContext(z["lat"], crys, z["real_pos"], z["masses"], z["at_types"], z["phi"]) as ctx:
        g = synth.uniform_grid(6)
        r = ctx.solve(g, api.EigOpts(jobz="N", precision=api.PP_PREC_FP64))
    rec = geometry.reciprocal_lattice(z["lat"])
    return z, g, r.w, rec


def test_linear_triangulation(grid_freqs):
    z, g, w, rec = grid_freqs
    tri = dos.triangulate(g, rec)
    freq = w[:, :12]                       # 12 lowest bands keep the oracle loop short
    rng = np.random.default_rng(4)
    func = rng.uniform(0.5, 1.5, freq.shape)
    E = np.linspace(freq.min() - 5, freq.max() + 5, 37)
    d_gpu, n_gpu = dos.linear_triangulation(freq, tri, E, func)
    d_ref, n_ref = dos_ref.linear_triangulation(freq, func, tri, E)
    np.testing.assert_allclose(d_gpu, d_ref, rtol=1e-10, atol=1e-12 * np.abs(d_ref).max())
    np.testing.assert_allclose(n_gpu, n_ref, rtol=1e-10, atol=1e-12 * np.abs(n_ref).max())
    # above every band each triangle contributes the sum of its vertex weights
    expect = sum(func[t].sum() for t in tri)
    assert abs(n_gpu[-1] - expect) <= 1e-12 * expect and d_gpu[-1] == 0.0
    D, N = dos.density_of_states(freq, tri, E, z["lat"], 28)
    assert np.all(np.isfinite(D)) and N[-1] > 0


@pytest.mark.parametrize("method,mid", [("gaussian", 1), ("lorentzian", 2)])
def test_smearing(grid_freqs, method, mid):
    z, g, w, rec = grid_freqs
    weights = np.full(len(g), 1.0 / len(g))
    E = np.linspace(-10, 1800, 181)
    out = dos.smearing_dos(w, weights, E, 8.0, 28, method)
    ref = dos_ref.smearing(mid, w, weights, 8.0, E, 28)
    np.testing.assert_allclose(out, ref, rtol=1e-10, atol=1e-14)


def test_device_resident_dos_and_transport_dos():
    """DOS and velocity-weighted (transport) DOS computed on the device from
    the outputs of pp_solve_batch_device for an N = 148 grid, against the
    oracle port on the same frequencies and weights copied to the host."""
    import torch
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    g = synth.uniform_grid(6)
    nq, nb = len(g), 40                    # the 40 lowest bands keep the oracle loop short
    dev = torch.device("cuda", 0)
    with api.PhononContext.from_cell(c, phi) as ctx:
        n = ctx.n
        q_dev = torch.tensor(np.asfortranarray(g).ravel(order="F"), dtype=torch.float64, device=dev)
        w_dev = torch.zeros((nq, n), dtype=torch.float64, device=dev)
        v_dev = torch.zeros((nq, n, 3), dtype=torch.float64, device=dev)
        m_dev = torch.zeros(nq, dtype=torch.int64, device=dev)
        nz_dev, info_dev = torch.zeros_like(m_dev), torch.zeros_like(m_dev)
        s = torch.cuda.current_stream().cuda_stream
        ctx.solve_device(q_dev, api.EigOpts(jobz="N", vel=True, precision=api.PP_PREC_MIXED), w_dev, m_dev, nz_dev,
                         info_dev, vel_dev=v_dev, stream=s)
        rec = geometry.reciprocal_lattice(c.lat)
        tri = dos.triangulate(g, rec)
        tri_dev = torch.as_tensor(tri, device=dev)
        w_h = w_dev.cpu().numpy()
        E = np.linspace(w_h[:, :nb].min() - 2, w_h[:, :nb].max() + 2, 23)
        E_dev = torch.as_tensor(E, device=dev)
        d_gpu, n_gpu = dos.linear_triangulation_device(w_dev, tri_dev, E_dev, nbands=nb, stream=s)
        func_dev = dos.velocity_weights_device(v_dev, 0, 0, nbands=nb, stream=s)
        t_gpu, tn_gpu = dos.linear_triangulation_device(w_dev, tri_dev, E_dev, nbands=nb, func_dev=func_dev,
                                                        stream=s)
        weights = torch.full((nq,), 1.0 / nq, dtype=torch.float64, device=dev)
        sm_gpu = dos.smearing_dos_device(w_dev, weights, E_dev, 4.0, c.natom, "gaussian", nbands=nb, stream=s)
        torch.cuda.synchronize()
    assert int(info_dev.max()) == 0 and int(m_dev.min()) == n
    freq = w_h[:, :nb]
    vx2 = v_dev.cpu().numpy()[:, :nb, 0] ** 2
    np.testing.assert_allclose(func_dev.cpu().numpy(), vx2, rtol=0, atol=0)
    d_ref, n_ref = dos_ref.linear_triangulation(freq, np.ones_like(freq), tri, E)
    t_ref, tn_ref = dos_ref.linear_triangulation(freq, vx2, tri, E)
    for a, b in ((d_gpu, d_ref), (n_gpu, n_ref), (t_gpu, t_ref), (tn_gpu, tn_ref)):
        b = np.asarray(b)
        np.testing.assert_allclose(a.cpu().numpy(), b, rtol=1e-10, atol=1e-12 * max(np.abs(b).max(), 1e-300))
    assert np.abs(t_ref).max() > 0     # the transport weights change the result
    sm_ref = dos_ref.smearing(1, freq, np.full(nq, 1.0 / nq), 4.0, E, c.natom)
    np.testing.assert_allclose(sm_gpu.cpu().numpy(), sm_ref, rtol=1e-10, atol=1e-14)
