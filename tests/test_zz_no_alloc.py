"""The entry point that allocates nothing, checked against the regular one.

pp_heevx_values_noalloc is for callers that cannot allocate device memory
(inside a stream capture or a pipeline they do not own, or with a fixed
device pool): it takes the Hermitian matrix and the output buffers from the
caller and keeps its scratch in a fixed array compiled into the library.
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


def test_noalloc_rejects_oversize():
    from parphom_gb300 import api
    n = api.PP_NOALLOC_MAX_N + 1
    # rejected before any device work: no buffers are touched
    rc = api.heevx_values_noalloc(1, n, n, 1, 1, 1)
    assert rc == api.PP_ERR_SIZE
    assert "capacity" in api.strerror(rc)
