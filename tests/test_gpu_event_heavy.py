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


@pytest.mark.parametrize("mode", [1, 2])
def test_batched_clusters_beyond_the_block_sort(mode):
    """Two dense clusters in one batched context: their events (well over
    4,096 a cycle together) go through the multi-block sort (mode 1) or the
    one-block sort (mode 2) and one resolution over both collections; each
    collection stays bit-identical to its own oracle run (fragment ids
    aside: a batch draws them from one counter)."""
    import numpy as np

    from nbodygo_gb300.api import Simulation
    from oracle.oracle import OracleSim

    from helpers import assert_states_identical
    from test_gpu_batch import split_state

    sims = [dense_cluster(1500, seed=108), dense_cluster(1200, seed=109)]
    gpu = Simulation("fp64", seed=77)
    gpu.set_option(A.OPT_EVENT_SORT, mode)
    gpu.set_collections(sims)
    oracles = []
    for b in sims:
        o = OracleSim(seed=77, threads=8)
        o.set_bodies(b)
        oracles.append(o)
    busiest = 0
    for c in range(4):
        info = gpu.step(0.03, 0.8, 1)
        for o in oracles:
            o.step(0.03, 0.8, 1)
        busiest = max(busiest, info["events"])
        counts = gpu.sim_counts()
        assert list(counts) == [o.count() for o in oracles], f"cycle {c}"
        for q, (got, o) in enumerate(zip(split_state(gpu.state(), counts), oracles)):
            assert_states_identical(got, o.state(), fields=[k for k in got if k != "id"],
                                    where=f"mode {mode} cycle {c} collection {q}")
    assert busiest > 4096
    gpu.close()
