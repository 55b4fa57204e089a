"""The entry point that allocates nothing, checked against the regular one.

pp_heevx_values_noalloc is for callers that cannot allocate device memory
(drivers that hand over a fixed device pool and forbid hidden allocations,
stream-ordered pipelines they do not own, long runs that must not grow the
device footprint): it takes the Hermitian matrix and the output buffers from
the caller and keeps its scratch in a fixed array compiled into the library.
Here it must give the eigenvalues that pp_solve_batch gives for the same
D(q), within the lambda-space tolerance of the parity tests
(64 n eps ||D||), on two calls in a row (the second one sees whatever the
first left in the shared scratch array).  This file is collected last so
that a failure here does not hide the other tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_eigenvalues_match_solve_batch():
    import torch
    from parphom_gb300 import api, synth

    cell = synth.tblg_cell(3)   # N = 148, n = 444 (limit 1536)
    phi = synth.spring_force_constants(cell, seed=0)
    with api.PhononContext.from_cell(cell, phi) as ctx:
        q = np.array([[0.21, -0.13, 0.0]])
        ref = ctx.solve(q, api.EigOpts(jobz="N", raw_lambda=True, precision=api.PP_PREC_FP64))
        D = ctx.dynamical_matrix(q[0])
    n = D.shape[0]
    lam_ref = ref.w[0, :n]
    tol = 64 * n * np.finfo(float).eps * np.abs(lam_ref).max()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    outs = []
    for call in range(2):
        a = torch.from_numpy(np.ascontiguousarray(D.T)).to(dev)   # column-major D(q)
        w = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
        m = torch.zeros(1, dtype=torch.int64, device=dev)
        info = torch.full((1,), -1, dtype=torch.int64, device=dev)
        rc = api.heevx_values_noalloc(a.data_ptr(), n, n, w.data_ptr(), m.data_ptr(), info.data_ptr(),
                                      stream=stream.cuda_stream)
        torch.cuda.synchronize()
        assert rc == 0, api.strerror(rc)
        assert int(m.item()) == n and int(info.item()) == 0
        lam = w.cpu().numpy()
        assert np.abs(lam - lam_ref).max() <= tol, (call, np.abs(lam - lam_ref).max(), tol)
        outs.append(lam)
    assert np.array_equal(outs[0], outs[1])


def _call(D, rng="A", vl=0.0, vu=0.0, il=1, iu=1):
    """Two calls on fresh copies of D; the device's free memory is read around
    the second one (the first may load the library's kernels lazily)."""
    import torch
    from parphom_gb300 import api
    n = D.shape[0]
    dev = torch.device("cuda", 0)
    outs = []
    for call in range(2):
        a = torch.from_numpy(np.ascontiguousarray(D.T)).to(dev)
        w = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
        m = torch.zeros(1, dtype=torch.int64, device=dev)
        info = torch.full((1,), -1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        rc = api.heevx_values_noalloc(a.data_ptr(), n, n, w.data_ptr(), m.data_ptr(), info.data_ptr(), range=rng,
                                      vl=vl, vu=vu, il=il, iu=iu, stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(dev)[0]
        assert rc == 0, api.strerror(rc)
        outs.append((w.cpu().numpy(), int(m.item()), int(info.item()), free0 - free1))
    (w0, m0, i0, _), (w1, m1, i1, dfree) = outs
    assert m0 == m1 and i0 == i1 and np.array_equal(w0[:m0], w1[:m1])
    return w1, m1, i1, dfree


def test_noalloc_index_and_value_ranges():
    """Ranges 'I' and 'V' give the same m and eigenvalues as pp_solve_batch,
    and no call changes the device's free memory."""
    from parphom_gb300 import api, synth

    cell = synth.tblg_cell(3)
    phi = synth.spring_force_constants(cell, seed=0)
    q = np.array([[0.37, 0.05, 0.0]])
    with api.PhononContext.from_cell(cell, phi) as ctx:
        D = ctx.dynamical_matrix(q[0])
        n = D.shape[0]
        full = ctx.solve(q, api.EigOpts(jobz="N", raw_lambda=True, precision=api.PP_PREC_FP64)).w[0, :n]
        tol = 64 * n * np.finfo(float).eps * np.abs(full).max()
        # range I: indices 20..90
        w, m, info, dfree = _call(D, "I", il=20, iu=90)
        assert info == 0 and m == 71 and dfree == 0
        assert np.abs(w[:m] - full[19:90]).max() <= tol
        # range V: eigenvalues in (vl, vu] in the matrix's own units (no
        # cm^-1 conversion here), between two well separated eigenvalues
        j0 = 90 + int(np.argmax(np.diff(full[90:111])))     # widest gap near index 100
        j1 = 290 + int(np.argmax(np.diff(full[290:311])))   # and near index 300
        lo, hi = 0.5 * (full[j0] + full[j0 + 1]), 0.5 * (full[j1] + full[j1 + 1])
        w, m, info, dfree = _call(D, "V", vl=lo, vu=hi)
        assert info == 0 and m == j1 - j0 and dfree == 0
        assert np.abs(w[:m] - full[j0 + 1:j1 + 1]).max() <= tol


def test_noalloc_flags_non_finite_input():
    """A non-finite element of the upper triangle is reported in info
    (PP_INFO_NAN) with no eigenvalues; the next call is clean again."""
    from parphom_gb300 import api, synth

    cell = synth.tblg_cell(3)
    phi = synth.spring_force_constants(cell, seed=0)
    with api.PhononContext.from_cell(cell, phi) as ctx:
        D = ctx.dynamical_matrix([0.1, 0.2, 0.0])
        lam = ctx.solve([[0.1, 0.2, 0.0]], api.EigOpts(jobz="N", raw_lambda=True)).w[0]
    bad = D.copy()
    bad[3, 17] = np.nan
    _, m, info, _ = _call(bad)
    assert m == 0 and info & api.INFO_NAN
    w, m, info, _ = _call(D)
    n = D.shape[0]
    assert m == n and info == 0
    assert np.abs(w - lam[:n]).max() <= 64 * n * np.finfo(float).eps * np.abs(lam).max()


def test_noalloc_rejects_oversize():
    from parphom_gb300 import api
    n = api.PP_NOALLOC_MAX_N + 1
    # rejected before any device work: no buffers are touched
    rc = api.heevx_values_noalloc(1, n, n, 1, 1, 1)
    assert rc == api.PP_ERR_SIZE
    assert "capacity" in api.strerror(rc)
