"""Failure detection without a GPU fault: the tensor-core kernels' waits on
mbarriers are bounded.  A self-test kernel waits, with a short poll limit,
on a barrier that nothing completes; the wait runs out, the kernel leaves
the time-out bit in the device status word and returns, and the context
stays usable (a render afterwards succeeds)."""
import ctypes as C

import pytest

import lisa_gb300 as L
from lisa_gb300 import _native as N
from lisa_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_context_stays_usable(gpu):
    v = C.c_uint32(0)
    N.check(N.lib().lisa_selftest_wait_timeout(1 << 8, C.byref(v)))
    assert v.value & N.LISA_STATUS_WAIT_TIMEOUT
    sc = scenes.cornell_box(width=16, height=16, num_samples=1, num_bounces=2)
    r = L.Renderer(L.params_from_scene(sc))
    st = r.render()
    assert st.device_status == 0 and st.rays_primary == 16 * 16
