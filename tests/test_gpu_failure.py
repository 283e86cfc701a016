"""Failure detection of the device waits, without a GPU fault.

The tiled Chebyshev step waits on mbarriers for its bulk copies. Each wait
gives up after the context's poll limit (or two seconds), records a status
word and drains its own copies before the block exits. The test hook
`test_unsatisfied_wait` makes every block first wait on a barrier that nobody
completes, so the wait must run out: the call reports LEO2D_ERR_TIMEOUT and
the context keeps working afterwards.
"""
import numpy as np
import pytest

import leo2d_gb300 as L

pytestmark = pytest.mark.gpu


def test_wait_runs_out_then_context_recovers():
    with L.Context(0) as ctx:
        g = L.make_geom(model=L.MODEL_SIMPLE, size=22, angles_deg=(0.0, 3.0), energy_rescale=1.0)
        csr = ctx.build_csr(ctx.prepare(g))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        cfg = L.kpm_cfg(32, R=4, seed=5, block=8)
        ctx.set_option("step_kernel", 0)
        before = csr.kpm_dos(cfg)
        ctx.set_spin_limit(2000)
        ctx.set_option("test_unsatisfied_wait", 1)
        with pytest.raises(L.Leo2dError) as e:
            csr.kpm_dos(cfg)
        assert e.value.status == L._abi.ERR_TIMEOUT
        assert "wait ran out" in str(e.value)
        ctx.set_option("test_unsatisfied_wait", 0)
        ctx.set_spin_limit(0)
        after = csr.kpm_dos(cfg)
        np.testing.assert_array_equal(after, before)
