"""Render ring (nbg_set_render_ring): every cycle's renderables written by the
integration kernel straight into mapped host memory, the path of the
reference's result queue (computation-runner.go:316-321,
resultqueue.go:97-129) without a copy call."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation

pytestmark = pytest.mark.gpu


def same_rend(a, b):
    for f in ("id", "x", "y", "z", "flags", "radius"):
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_slots_hold_each_cycles_renderables(precision):
    b = W.disk(n=700, seed=3)
    with Simulation(precision) as sim:
        sim.set_bodies(b)
        head, rend = sim.set_render_ring(slots=4, slot_cap=1024)
        assert np.all(head["cycle"] == -1)
        for c in range(6):
            sim.step(0.005, 1.0, 1)
            s = c % 4
            assert head[s]["cycle"] == c
            n = head[s]["count"]
            assert head[s]["written"] == n == len(sim.renderables())
            same_rend(rend[s, :n], sim.renderables())


def test_ring_from_a_graph_replay_and_a_short_slot():
    b = W.plummer(3000, seed=4)
    with Simulation("mixed") as sim:
        sim.set_bodies(b)
        head, rend = sim.set_render_ring(slots=3, slot_cap=2000)
        sim.step(0.01, 1.0, 7)  # cycles 0..6 in one call (a graph replay)
        assert sorted(head["cycle"].tolist()) == [4, 5, 6]
        last = int(np.argmax(head["cycle"]))
        assert head[last]["count"] == 3000 and head[last]["written"] == 2000
        same_rend(rend[last, :2000], sim.renderables()[:2000])
        sim.clear_render_ring()
        sim.step(0.01, 1.0, 2)  # detached: stepping goes on without the ring


def test_ring_attach_needs_sizes():
    from nbodygo_gb300.api import NbgError
    with Simulation("fp64") as sim:
        with pytest.raises(NbgError):
            sim.set_render_ring(slots=0, slot_cap=10)


@pytest.mark.parametrize("bh", [False, True])
def test_ring_with_several_collections(bh):
    """A batched context (direct sum or one Barnes-Hut tree per collection)
    writes every collection's renderables into the ring, in body order."""
    sims = [W.disk(n=400, seed=5), W.plummer(500, seed=6)]
    with Simulation("mixed") as sim:
        if bh:
            sim.set_option(A.OPT_BARNES_HUT, 1)
        sim.set_collections(sims)
        head, rend = sim.set_render_ring(slots=2, slot_cap=2048)
        for c in range(3):
            sim.step(0.005, 1.0, 1)
            s = c % 2
            n = head[s]["count"]
            assert head[s]["cycle"] == c and n == sim.count() and head[s]["written"] == n
            same_rend(rend[s, :n], sim.renderables())
