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
