"""The launch-configuration autotuner: the first solve of a (order, batch,
options) combination times its candidates on the GPU and records a choice;
the results do not depend on the configuration chosen."""
import numpy as np
import pytest

from parphom_gb300 import api, synth

pytestmark = pytest.mark.gpu


def test_autotune_records_a_choice_and_keeps_results(monkeypatch):
    c = synth.tblg_cell(3)
    phi = synth.spring_force_constants(c, seed=0)
    qs = synth.random_qpoints(8, seed=51)
    opts = api.EigOpts(jobz="N", vel=True, precision=api.PP_PREC_MIXED)
    with api.PhononContext.from_cell(c, phi) as ctx:
        monkeypatch.setenv("PARPHOM_GPU_TUNE", "0")
        ref = ctx.solve(qs, opts, want_z=False)
        monkeypatch.setenv("PARPHOM_GPU_TUNE", "1")
        before = len(api.autotune_report())
        tuned = ctx.solve(qs, opts, want_z=False)
        again = ctx.solve(qs, opts, want_z=False)
    rep = api.autotune_report()
    assert len(rep) == before + 1
    line = rep[-1]
    assert "n=444" in line and "B=8" in line and "split=" in line and "hemv_blocks_per_sm=" in line
    assert float(line.split("batch_ms=")[1]) > 0.0
    n = c.n
    for r in (tuned, again):
        assert np.all(r.info == 0)
        np.testing.assert_allclose(r.w[:, :n], ref.w[:, :n], rtol=1e-12, atol=1e-9)
        vmax = np.abs(ref.vel).max()
        np.testing.assert_allclose(r.vel, ref.vel, rtol=0, atol=1e-9 * vmax)
