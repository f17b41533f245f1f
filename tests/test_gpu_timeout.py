"""Failure detection of the tensor-core kernels without a GPU fault.

Every wait between the roles of k_local_tc (TMA issue, A producers, MMA issue,
accumulator drains) is bounded by %globaltimer.  With a limit far below one
pipeline stage (100 ns against ~1.2 us per stage) some wait must run out: the
kernel then stops issuing, lets its copies and MMAs in flight finish, frees
its tensor memory and reports LELPH_GPU_ERR_TIMEOUT, which the host returns as
a status.  The same context then runs again with the default limit and gives
the same matrix elements as before."""
import numpy as np
import pytest

from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphError, LelphGPU

pytestmark = pytest.mark.gpu

ERR_TIMEOUT = -4


def test_short_wait_limit_reports_timeout_and_context_recovers():
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]})
    ks = list(range(s.nk_bz))
    with LelphGPU(s, "mixed", route="real") as ctx:
        ctx.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g0 = ctx.run([0] * len(ks), ks)
        ctx.set_wait_limit(100)
        with pytest.raises(LelphError) as e:
            ctx.run([0] * len(ks), ks)
        assert e.value.status == ERR_TIMEOUT
        ctx.set_wait_limit(0)
        g1 = ctx.run([0] * len(ks), ks)
    assert np.isfinite(g1).all()
    assert np.array_equal(g0, g1)   # the same kernels on the same inputs: the same bits


def test_projections_short_wait_limit_reports_timeout_and_context_recovers():
    """The tensor-core KB projections (prepare) under the same short limit: the
    MMA thread gives up on the first stage, the producers find their slots
    never freed and leave together at their next barrier, the drains give up
    on the accumulators; prepare returns LELPH_GPU_ERR_TIMEOUT and prepares
    again, to the same bits, once the default limit is back."""
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]})
    ks = list(range(s.nk_bz))
    with LelphGPU(s, "mixed", route="real") as ctx:
        ctx.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g0 = ctx.run([0] * len(ks), ks)
        ctx.set_wavefunctions(s.wfc)  # the next run prepares again
        ctx.set_wait_limit(100)
        with pytest.raises(LelphError) as e:
            ctx.prepare()
        assert e.value.status == ERR_TIMEOUT
        ctx.set_wait_limit(0)
        ctx.prepare()
        g1 = ctx.run([0] * len(ks), ks)
    assert np.isfinite(g1).all()
    assert np.array_equal(g0, g1)
