"""A bounded device wait that runs out, made to run out on purpose.

The tensor-core kernels of the mixed form wait on mbarriers with a limit;
when a wait gives up, the kernel flags its matrix, waits (bounded) for its
own copies in flight, frees its tensor memory and returns, later launches
skip the matrix, and its info carries PP_INFO_TIMEOUT.  The test hook
pp_debug_stall_tc_wait makes one trailing-update launch wait on a barrier
that nothing completes, for ~1 ms of SM clocks: no fault, no hang.  The
other matrices of the batch must be unaffected, and the next clean solve of
the same q-points must be correct again.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parphom_gb300 import api, synth
from tests import parity

pytestmark = pytest.mark.gpu


def test_tc_wait_timeout_flags_only_its_matrix():
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    S = O.System.from_cell(c, phi)
    qs = synth.random_qpoints(3, seed=31)
    refs = [O.solve_q(S, q) for q in qs]
    n = S.n
    opts = api.EigOpts(jobz="N", precision=api.PP_PREC_MIXED)
    with api.PhononContext.from_cell(c, phi) as ctx:
        api.debug_stall_tc_wait(1, 2_000_000)
        bad = ctx.solve(qs, opts, want_z=False)
        assert bad.info[1] & api.INFO_TIMEOUT
        for t in (0, 2):
            assert bad.info[t] == 0
            Dn = np.abs(refs[t]["lam"]).max()
            parity.check_frequencies(bad.w[t, :n], refs[t]["w_cm"], refs[t]["lam"], n, Dn)
        good = ctx.solve(qs, opts, want_z=False)
        for t in range(3):
            assert good.info[t] == 0
            Dn = np.abs(refs[t]["lam"]).max()
            parity.check_frequencies(good.w[t, :n], refs[t]["w_cm"], refs[t]["lam"], n, Dn)
    api.debug_stall_tc_wait(-1, 0)
