"""Bounded device waits give up and report, without faulting the GPU.

The TMA-staged FP16 hopping kernel waits on mbarriers for its copies; every
such wait is bounded (0.5 s of the device timer), after which the thread sets
the context's device error flag and stops waiting.  `wd_debug_expire_wait`
runs that same bounded wait on a barrier nothing completes: the wait must
give up after its bound, `wd_context_device_check` must then report
WD_ERR_TIMEOUT once and clear the flag, and the context must stay usable."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_timeout_then_clears(wd, ctx, oracle):
    ctx.device_check()  # nothing pending
    waited = ctx.debug_expire_wait()
    assert 0.45 < waited < 5.0, waited
    with pytest.raises(wd.WilsonError) as e:
        ctx.device_check()
    assert e.value.status == wd.TIMEOUT
    ctx.device_check()  # the flag was cleared
    # the context still computes correctly
    dims = (8, 4, 4, 4)
    gauge = wd.gen_gauge(dims, seed=31)
    src = wd.gen_source(dims, seed=31)
    lat = ctx.lattice(dims, gauge)
    fo = lat.field()
    lat.dslash_offd(lat.field(src), fo, 0, 1)
    assert rel_l2(fo.download(), oracle.dslash_offd(src, gauge, dims, 0, 1)) < 1e-13
    ctx.device_check()
