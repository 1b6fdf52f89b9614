"""A device wait that runs out.

The bulk-copy shapes of the mixed pair kernel (17 and 18) wait on an
mbarrier for each j tile's copies, each wait bounded by about 2 s of SM
clock.  The NBG_OPT_TEST_WAIT_STALL hook arms every mbarrier for 16 bytes
more than its copies bring, so no wait completes: a flag that nothing sets,
with every copy finished.  The cycle must fail with NBG_E_TIMEOUT (what 8),
change nothing, and leave the context stepping on exactly as a fresh one.
"""
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import NbgError, Simulation

from helpers import assert_states_identical

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [17])
def test_bulk_copy_wait_runs_out_and_the_context_recovers(shape):
    b = W.plummer(4096, seed=11)
    with Simulation("mixed") as ref:
        ref.set_option(A.OPT_MIX_SHAPE, shape)
        ref.set_bodies(b)
        ref.step(0.01, 1.0, 2)
        exp = ref.state()
    with Simulation("mixed") as s:
        s.set_option(A.OPT_MIX_SHAPE, shape)
        s.set_bodies(b)
        s.set_option(A.OPT_TEST_WAIT_STALL, 1)
        with pytest.raises(NbgError) as e:
            s.step(0.01, 1.0, 1)
        assert e.value.code == A.NBG_E_TIMEOUT
        assert "what 8" in str(e.value)
        s.set_option(A.OPT_TEST_WAIT_STALL, 0)
        s.step(0.01, 1.0, 2)
        got = s.state()
    assert_states_identical(got, exp, where="after a cycle whose waits ran out")


def test_wait_stall_hook_takes_only_0_or_1():
    with Simulation("mixed") as s:
        with pytest.raises(NbgError):
            s.set_option(A.OPT_TEST_WAIT_STALL, 2)
