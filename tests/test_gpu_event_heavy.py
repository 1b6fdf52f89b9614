"""Cycles with more events than one block sorts in shared memory (4,096):
the multi-block radix sort of the event keys, the one-block global-memory
sort and the automatic choice between them must all give the oracle's
events and state bit for bit, on a dense cluster whose busiest cycles detect
more than 10^5 events, and on a large body absorbing the bodies of a disk
(one body in thousands of events, resolved in the reference's order)."""
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W

from test_gpu_plain_parity import dense_cluster, run_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_dense_cluster_beyond_the_block_sort(mode):
    """3,000 bodies of every behaviour: cycles 3 and 4 detect 149k and 273k
    events (oracle counts)."""
    b = dense_cluster(3000, seed=107)
    sim, ora = run_both(b, 0.03, 0.8, 5, gpu_opts={A.OPT_EVENT_SORT: mode})
    assert len(ora.events()) > 100000


@pytest.mark.parametrize("mode", [1, 2])
def test_large_body_absorbs_a_disk(mode):
    """A central body of radius 400 inside a disk of 24,000 bodies
    (r 100-1000), everything subsume: 7,446 events in the first cycle, every
    one on the central body, which absorbs 3,712 bodies."""
    b = W.disk(n=24000, seed=5)
    b["radius"][0] = 400.0
    b["collision"][:] = A.SUBSUME
    sim, ora = run_both(b, 0.005, 1.0, 2, gpu_opts={A.OPT_EVENT_SORT: mode})
    assert ora.count() == 20288
