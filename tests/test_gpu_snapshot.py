"""Snapshots (nbg_save_state / nbg_load_state): a run stopped after some
cycles, saved, loaded into a fresh context and continued must repeat the
uninterrupted run bit for bit - body state, private fields (fragmenting and
fragInfo, collided, r, the stale force), ids, the NextId counter and the
fragment generator's cycle key - and, in the plain form, the CPU oracle's
run too.  The reference's CSV format (cmd/sim/fromcsv.go:46-116) holds the
public fields only, which cannot resume a trajectory."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import NbgError, Simulation
from oracle.oracle import OracleSim

from helpers import assert_events_identical, assert_states_identical
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu


def resumed(make, load, first, then, dt, R, adds=None):
    """(uninterrupted simulation, resumed simulation): both ran first + then
    cycles; the second was saved after `first`, loaded into a new context
    and continued.  `adds(sim)` stages host adds just before the save."""
    a = make()
    load(a)
    a.step(dt, R, first)
    if adds:
        adds(a)
    snap = a.save_state()
    a.step(dt, R, then)
    b = make()
    b.load_state(snap)
    b.step(dt, R, then)
    return a, b, snap


def test_disk_resumed_at_100_of_200_cycles_matches_uninterrupted_and_oracle():
    bodies = W.disk(seed=1)
    a, b, _ = resumed(lambda: Simulation("fp64", seed=9), lambda s: s.set_bodies(bodies), 100, 100, 0.005, 1.0)
    assert_states_identical(b.state(), a.state(), where="resumed vs uninterrupted")
    assert b.next_id() == a.next_id()
    ora = OracleSim(seed=9, threads=8)
    ora.set_bodies(bodies)
    ora.step(0.005, 1.0, 200)
    assert_states_identical(b.state(), ora.state(), where="resumed vs oracle")


def test_fragmenting_cluster_with_staged_adds_resumes_bit_exact():
    """Saved while bodies are fragmenting (fragInfo, stale forces, collided
    flags live) and with host adds staged for the next Cycle."""
    bodies = dense_cluster(300, seed=32, behaviors=(A.ELASTIC, A.FRAGMENT))
    extra = dense_cluster(7, seed=99)
    extra["id"][:] = np.arange(7) + 5000

    def adds(s):
        s.add_bodies(extra)

    a, b, _ = resumed(lambda: Simulation("fp64", seed=4), lambda s: s.set_bodies(bodies), 6, 12, 0.05, 1.0, adds)
    st = a.state()
    assert_states_identical(b.state(), st, where="resumed vs uninterrupted")
    assert_events_identical(b.events(), a.events(), where="last cycle's events")
    assert b.next_id() == a.next_id()
    assert np.isin(np.arange(5000, 5007), st["id"]).all(), "the staged adds arrived after the load"
    ora = OracleSim(seed=4, threads=8)
    ora.set_bodies(bodies)
    ora.step(0.05, 1.0, 6)
    ora.add_bodies(extra)
    ora.step(0.05, 1.0, 12)
    assert_states_identical(b.state(), ora.state(), where="resumed vs oracle")


def test_snapshot_taken_mid_fragmentation_holds_fragment_state():
    bodies = dense_cluster(300, seed=32, behaviors=(A.ELASTIC, A.FRAGMENT))
    with Simulation("fp64", seed=4) as s:
        s.set_bodies(bodies)
        for _ in range(12):
            s.step(0.05, 1.0, 1)
            if np.any(s.state()["flags"] & A.F_FRAGMENTING):
                break
        st = s.state()
        assert np.any(st["flags"] & A.F_FRAGMENTING), "the cluster fragments within 12 cycles"
        snap = s.save_state()
    with Simulation("mixed") as t:  # another form: the snapshot's form wins
        t.load_state(snap)
        assert_states_identical(t.state(), st, where="loaded state")


@pytest.mark.parametrize("shape", [0, A.MIX_SYM, 17])
def test_mixed_form_resumes_bit_exact_between_sorts(shape):
    """The mixed form keeps its Morton order for 4 cycles; a snapshot taken
    mid-interval carries the order and the kernel shape (one-sided,
    symmetric, bulk-copied tiles), so the FP32 sums group the same bodies."""
    bodies = W.plummer_disk(n_each=4096, seed=8)

    made = []

    def make():
        s = Simulation("mixed")
        if not made:  # the resumed context takes its shape from the snapshot
            s.set_option(A.OPT_MIX_SHAPE, shape)
        made.append(s)
        return s

    a, b, _ = resumed(make, lambda s: s.set_bodies(bodies), 6, 7, 0.01, 1.0)
    assert_states_identical(b.state(), a.state(), where=f"mixed shape {shape} resumed vs uninterrupted")


def test_batched_context_with_staged_adds_resumes_bit_exact():
    sims = [W.disk(n=300, seed=1), dense_cluster(150, seed=2), W.plummer(n=257, seed=3, behavior=A.SUBSUME,
                                                                          radius_range=(0.5, 3.0))]

    def adds(s):
        e1 = dense_cluster(3, seed=61)
        e1["id"][:] = [7001, 7002, 7003]
        e2 = dense_cluster(2, seed=62)
        e2["id"][:] = [8001, 8002]
        s.add_bodies(e1, sim=2)
        s.add_bodies(e2, sim=0)

    a, b, _ = resumed(lambda: Simulation("fp64", seed=3), lambda s: s.set_collections(sims), 4, 6, 0.02, 0.9, adds)
    assert list(b.sim_counts()) == list(a.sim_counts())
    assert_states_identical(b.state(), a.state(), where="batched resumed vs uninterrupted")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_barnes_hut_context_resumes_bit_exact(prec):
    """The octree is rebuilt from the body state every cycle, so a
    Barnes-Hut run resumes bit for bit too, in both precisions, through
    collisions of every behaviour."""
    bodies = dense_cluster(400, seed=41)

    def make():
        s = Simulation(prec, seed=6)
        s.set_option(A.OPT_BARNES_HUT, 1)
        return s

    a, b, _ = resumed(make, lambda s: s.set_bodies(bodies), 5, 7, 0.05, 0.9)
    assert_states_identical(b.state(), a.state(), where=f"{prec} Barnes-Hut resumed vs uninterrupted")
    assert_events_identical(b.events(), a.events(), where="last cycle")


def test_batched_barnes_hut_context_resumes_bit_exact():
    """One tree per collection, rebuilt every cycle: a batched Barnes-Hut
    run resumes bit for bit too."""
    sims = [dense_cluster(250, seed=42), W.plummer(n=700, seed=43, radius_range=(0.3, 1.5))]

    def make():
        s = Simulation("mixed", seed=6)
        s.set_option(A.OPT_BARNES_HUT, 1)
        return s

    a, b, _ = resumed(make, lambda s: s.set_collections(sims), 4, 5, 0.05, 0.9)
    assert list(b.sim_counts()) == list(a.sim_counts())
    assert_states_identical(b.state(), a.state(), where="batched Barnes-Hut resumed vs uninterrupted")


def test_snapshot_size_query_and_rejections():
    bodies = W.disk(n=100, seed=3)
    import ctypes as C

    with Simulation("fp64") as s:
        s.set_bodies(bodies)
        s.step(0.005, 1.0, 3)
        snap = s.save_state()
        before = s.state()
        lib, ctx = s.lib, s.ctx
        size = C.c_int64()
        assert lib.nbg_save_state(ctx, None, 0, C.byref(size)) == A.NBG_OK and size.value == len(snap)
        small = C.create_string_buffer(16)
        assert lib.nbg_save_state(ctx, small, 16, C.byref(size)) == A.NBG_E_OVERFLOW
        with pytest.raises(NbgError):
            s.load_state(snap[:-8])  # truncated
        bad = bytearray(snap)
        bad[0:8] = b"NOTASNAP"
        with pytest.raises(NbgError):
            s.load_state(bytes(bad))
        # a refused load leaves the context as it was
        assert_states_identical(s.state(), before, where="after refused loads")


def test_snapshot_carries_its_form_into_a_context_of_the_other():
    """A mixed run's snapshot loaded into a context created for the plain
    form resumes the mixed run (the form, the kernel shape and the Morton
    order travel with it), bit for bit; and the other way round."""
    bodies = W.plummer_disk(n_each=3000, seed=12)
    for first, other in (("mixed", "fp64"), ("fp64", "mixed")):
        a = Simulation(first, seed=2)
        a.set_bodies(bodies)
        a.step(0.01, 1.0, 5)
        snap = a.save_state()
        a.step(0.01, 1.0, 6)
        b = Simulation(other, seed=2)
        b.load_state(snap)
        assert b.precision == first
        b.step(0.01, 1.0, 6)
        assert_states_identical(b.state(), a.state(), where=f"{first} snapshot in a {other} context")
        a.close()
        b.close()


def test_batched_mixed_context_resumes_bit_exact():
    """Several collections in the mixed form: the Morton order travels with
    the snapshot, each collection's positions over its own bodies."""
    sims = [W.plummer(n=1500, seed=1, behavior=A.SUBSUME, radius_range=(0.5, 3.0)), W.disk(n=700, seed=2),
            W.uniform_ball(n=2100, seed=3, R=300.0)]
    a, b, _ = resumed(lambda: Simulation("mixed", seed=3), lambda s: s.set_collections(sims), 5, 6, 0.01, 1.0)
    assert list(b.sim_counts()) == list(a.sim_counts())
    assert_states_identical(b.state(), a.state(), where="batched mixed resumed vs uninterrupted")


def test_snapshot_with_a_broken_order_is_refused():
    """The kernels index the bodies through the snapshot's order, so a load
    checks that it is a permutation of each collection: an index past the
    collection or a repeated one is refused, and the context stays as it
    was."""
    bodies = W.plummer_disk(n_each=2000, seed=4)
    with Simulation("mixed") as s:
        s.set_bodies(bodies)
        s.step(0.01, 1.0, 5)
        snap = s.save_state()
        n = s.count()
        before = s.state()
        start = len(snap) - (n * 4 + 7) // 8 * 8  # the order is the last section
        order = np.frombuffer(snap, dtype=np.uint32, count=n, offset=start)
        assert sorted(order.tolist()) == list(range(n))
        for k, v in ((0, n), (1, int(order[0])), (n - 1, 0xFFFFFFFF)):
            o = order.copy()
            o[k] = v
            with pytest.raises(NbgError) as e:
                s.load_state(snap[:start] + o.tobytes() + snap[start + 4 * n:])
            assert e.value.code == A.NBG_E_ARG and "order" in str(e.value)
        assert_states_identical(s.state(), before, where="after refused loads")
        s.load_state(snap)
