"""Batched form: many independent collections in one context
(nbg_set_collections).  Each collection must evolve exactly as it would alone:
bit-identical to its own oracle run in the plain form, and within the mixed
tolerance of its own FP64 forces in the mixed form."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import assert_states_identical, rel_l2
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu


def small_ensemble():
    sims = [
        W.disk(n=300, seed=1),
        dense_cluster(150, seed=2),                       # every behaviour, removals, fragments
        W.plummer(n=257, seed=3, behavior=A.SUBSUME, radius_range=(0.5, 3.0)),
        W.uniform_ball(n=64, seed=4, R=50.0, radius=1.0, behavior=A.ELASTIC),
        dense_cluster(1, seed=5),                         # a single body
        W.plummer(n=1000, seed=6),
    ]
    return sims


def split_state(st, counts):
    out, o = [], 0
    for c in counts:
        out.append({k: v[o:o + c] for k, v in st.items()})
        o += c
    return out


def test_plain_batch_matches_each_sim_alone():
    sims = small_ensemble()
    first_new_id = 1_000_000
    gpu = Simulation("fp64", seed=77)
    gpu.set_collections(sims)
    gpu.set_next_id(first_new_id)
    oracles = []
    for b in sims:
        o = OracleSim(seed=77, threads=4)
        o.set_bodies(b)
        o.set_next_id(first_new_id)
        oracles.append(o)
    dt, R = 0.02, 0.9
    for cycle in range(12):
        info = gpu.step(dt, R, 1)
        exp_inter = 0
        for o in oracles:
            n = o.count()
            exp_inter += n * (n - 1)
            o.step(dt, R, 1)
        assert info["interactions"] == exp_inter
        counts = gpu.sim_counts()
        assert list(counts) == [o.count() for o in oracles], f"cycle {cycle}"
        parts = split_state(gpu.state(), counts)
        for s, (got, o) in enumerate(zip(parts, oracles)):
            exp = o.state()
            # fragment ids come from one counter shared by all sims; the rest
            # of the state must be bit-identical
            fields = [f for f in got if f != "id"]
            assert_states_identical(got, exp, fields=fields, where=f"cycle {cycle} sim {s}")
            orig = exp["id"] < first_new_id
            assert np.array_equal(got["id"][orig], exp["id"][orig])
            assert np.all(got["id"][~orig] >= first_new_id)


def test_plain_batch_graph_replay():
    sims = small_ensemble()
    a = Simulation("fp64")
    a.set_collections(sims)
    a.step(0.02, 1.0, 10)
    b = Simulation("fp64")
    b.set_collections(sims)
    for _ in range(10):
        b.step(0.02, 1.0, 1)
    assert_states_identical(a.state(), b.state(), where="graph vs direct")
    assert list(a.sim_counts()) == list(b.sim_counts())


def test_mixed_batch_forces_per_sim():
    sims = [W.plummer(n=n, seed=10 + n) for n in (256, 700, 2048, 4096)] + [W.disk(n=999, seed=3)]
    gpu = Simulation("mixed")
    gpu.set_collections(sims)
    f = gpu.force_pass()
    o = 0
    for s, b in enumerate(sims):
        n = len(b["x"])
        ora = OracleSim(threads=8)
        ora.set_bodies(b)
        g = ora.forces()
        err = rel_l2([c[o:o + n] for c in f], g)
        assert err <= 1e-6, f"sim {s}: rel L2 {err:.3e}"
        o += n


def test_mixed_batch_events_and_counts():
    sims = [dense_cluster(200, seed=s) for s in (21, 22, 23)]
    gpu = Simulation("mixed", seed=9)
    gpu.set_collections(sims)
    gpu.step(0.05, 1.0, 1)
    ev = gpu.events()
    total = 0
    for b in sims:
        o = OracleSim(seed=9, threads=4)
        o.set_bodies(b)
        o.step(0.05, 1.0, 1)
        total += len(o.events())
    assert len(ev) == total
    counts = gpu.sim_counts()
    assert len(counts) == 3 and counts.sum() == gpu.count()


def test_batch_rejects_single_collection_operations():
    gpu = Simulation("fp64")
    gpu.set_collections([W.disk(n=50, seed=1), W.disk(n=60, seed=2)])
    from nbodygo_gb300.api import NbgError
    with pytest.raises(NbgError):
        gpu.remove_bodies(3)
    with pytest.raises(NbgError):
        gpu.add_bodies(W.disk(n=2, seed=3))


def test_flat_collections_match_separate_parts():
    """The flat form (collections one after another in one set of pinned
    arrays, as nbg_set_collections takes them) loads the same bodies as the
    list-of-parts form: the same state, bit for bit, after three cycles."""
    import torch

    sims = small_ensemble()
    a = Simulation("fp64")
    a.set_collections(sims)
    counts = np.array([len(b["x"]) for b in sims], dtype=np.int64)
    keys = set(sims[0])
    for b in sims[1:]:
        keys &= set(b)
    flat, keep = {}, []
    for k in keys:
        v = np.concatenate([np.asarray(b[k]) for b in sims])
        tdt = torch.int32 if v.dtype == np.uint32 else getattr(torch, str(v.dtype))
        t = torch.empty(len(v), dtype=tdt, pin_memory=True)
        keep.append(t)
        arr = t.numpy().view(v.dtype)
        arr[:] = v
        flat[k] = arr
    b = Simulation("fp64")
    b.set_collections_flat(flat, counts)
    assert list(b.sim_counts()) == list(counts)
    a.step(0.01, 1.0, 3)
    b.step(0.01, 1.0, 3)
    assert list(a.sim_counts()) == list(b.sim_counts())
    assert_states_identical(a.state(), b.state())
    with pytest.raises(ValueError):
        b.set_collections_flat(flat, counts[:-1])


@pytest.mark.parametrize("interval,shape", [(1, 0), (4, 0), (4, A.MIX_SYM), (4, 17)])
def test_mixed_batch_graph_replay_equals_single_cycles(interval, shape):
    """The mixed form decides on the device when to sort and carries the
    order through compaction; with collisions in some collection every
    cycle, ten cycles replayed as one CUDA graph, as two graphs of five and
    as ten single cycles give the same state bit for bit."""
    sims = small_ensemble()
    runs = []
    for cycles_per_graph, calls in ((10, [10]), (5, [5, 5]), (1, [1] * 10)):
        gpu = Simulation("mixed", seed=9)
        gpu.set_option(A.OPT_MIX_SHAPE, shape)
        gpu.set_option(A.OPT_SORT_INTERVAL, interval)
        gpu.set_option(A.OPT_GRAPH_CYCLES, cycles_per_graph)
        gpu.set_collections(sims)
        removed = 0
        for k in calls:
            info = gpu.step(0.02, 0.9, k)
            removed += info["removed"]
        runs.append((gpu.state(), list(gpu.sim_counts()), removed))
    assert runs[0][2] > 0  # bodies left some collection: compaction ran
    for st, counts, _ in runs[1:]:
        assert counts == runs[0][1]
        assert_states_identical(st, runs[0][0], where="graph replay vs single cycles")


def test_ensemble_full_run_conserves_mass_per_collection():
    """Config 3 for its full length (512 collections, 200 cycles, graphs of
    10, mixed form): every collection keeps its mass through merges and
    fragments, every state stays finite, and the collection sizes account
    for the removals and fragments reported."""
    sims = W.ensemble()
    gpu = Simulation("mixed", seed=5, capacity=sum(len(s["x"]) for s in sims) + 65536)
    gpu.set_option(A.OPT_GRAPH_CYCLES, 10)
    gpu.set_collections(sims)
    m0 = np.array([s["mass"].sum() for s in sims])
    n0 = sum(len(s["x"]) for s in sims)
    info = gpu.step(0.01, 1.0, 200)
    assert info["steps_done"] == 200
    st = gpu.state()
    counts = gpu.sim_counts()
    assert len(counts) == len(sims) and counts.sum() == len(st["x"])
    assert len(st["x"]) == n0 - info["removed"] + info["fragments_emitted"]
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        assert np.all(np.isfinite(st[f])), f
    o = 0
    for s, c in enumerate(counts):
        m1 = st["mass"][o:o + c].sum()
        assert abs(m1 - m0[s]) <= 1e-12 * m0[s], f"collection {s}: mass {m1!r} != {m0[s]!r}"
        o += c


def _empty_like(b):
    return {k: np.asarray(v)[:0] for k, v in b.items()}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_empty_collections_in_a_batch(prec):
    """Collections with no bodies at the start, in the middle and at the end
    of a batch: the others step exactly as alone (plain: bit for bit against
    their oracles; mixed: forces within the tolerance of FP64), the empty
    ones stay empty, and an add into an empty one lands there alone."""
    full = [W.disk(n=300, seed=11), dense_cluster(120, seed=12), W.plummer(n=500, seed=13)]
    e = _empty_like(full[0])
    sims = [e, full[0], e, e, full[1], full[2], e]
    counts0 = [len(b["x"]) for b in sims]
    dt, R = 0.02, 0.9
    with Simulation(prec, seed=77) as gpu:
        gpu.set_collections(sims)
        assert list(gpu.sim_counts()) == counts0
        if prec == "mixed":
            f = np.array(gpu.force_pass())
            with Simulation("fp64") as p:
                p.set_collections(sims)
                g = np.array(p.force_pass())
            assert rel_l2(f, g) <= 1e-6
        oracles = []
        for b in sims:
            o = OracleSim(seed=77, threads=2)
            o.set_bodies(b)
            oracles.append(o)
        for cycle in range(6):
            gpu.step(dt, R, 1)
            for o in oracles:
                o.step(dt, R, 1)
            counts = gpu.sim_counts()
            # the mixed form's events are exact on a given state; its states
            # drift from FP64 within the tolerance, so only the first cycle's
            # counts must agree there
            if prec == "fp64" or cycle == 0:
                assert list(counts) == [o.count() for o in oracles], f"cycle {cycle}"
            assert counts[0] == counts[2] == counts[3] == counts[6] == 0
            if prec == "fp64":
                parts = split_state(gpu.state(), counts)
                for s, (got, o) in enumerate(zip(parts, oracles)):
                    if counts[s]:
                        fields = [k for k in got if k != "id"]
                        assert_states_identical(got, o.state(), fields=fields, where=f"cycle {cycle} sim {s}")
        add = W.uniform_ball(n=5, seed=14, R=20.0, radius=0.5)
        gpu.add_bodies(add, sim=2)
        gpu.step(dt, R, 1)
        counts = gpu.sim_counts()
        assert counts[2] == 5 and counts[0] == 0 and counts[3] == 0 and counts[6] == 0
        part = split_state(gpu.state(), counts)[2]
        assert np.all(np.isin(part["mass"], add["mass"]))


def _tiny_sets(count, seed):
    """count small collections of 0-16 bodies (some empty), every behaviour"""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(0, 17, count)
    sets = []
    for s, k in enumerate(sizes):
        b = dense_cluster(max(int(k), 1), seed=1000 + s)
        if k == 0:
            b = {f: np.asarray(v)[:0] for f, v in b.items()}
        sets.append(b)
    return sets


def test_the_most_collections_a_context_takes():
    """2,048 collections (the Morton key's 11-bit collection field, the
    largest count nbg_set_collections takes), of 0-16 bodies each: plain
    cycles stay bit-identical to each collection's oracle run, the mixed
    forces and the Barnes-Hut forests agree with FP64, and 2,049 are
    refused."""
    from nbodygo_gb300.api import NbgError

    sets = _tiny_sets(2048, 5)
    gpu = Simulation("fp64", seed=3)
    gpu.set_collections(sets)
    oracles = []
    for b in sets:
        o = OracleSim(seed=3, threads=1)
        o.set_bodies(b)
        oracles.append(o)
    for c in range(3):
        gpu.step(0.05, 0.9, 1)
        for o in oracles:
            o.step(0.05, 0.9, 1)
        counts = gpu.sim_counts()
        assert list(counts) == [o.count() for o in oracles], f"cycle {c}"
        for q, (got, o) in enumerate(zip(split_state(gpu.state(), counts), oracles)):
            if counts[q]:
                assert_states_identical(got, o.state(), fields=[k for k in got if k != "id"],
                                        where=f"cycle {c} collection {q}")
    g = np.array(gpu.force_pass())
    parts = split_state(gpu.state(), gpu.sim_counts())
    gpu.close()

    def forces(prec, bh):
        with Simulation(prec) as s:
            if bh:
                s.set_option(A.OPT_BARNES_HUT, 1)
            s.set_collections(parts)
            return np.array(s.force_pass())

    assert rel_l2(forces("mixed", False), g) <= 1e-6
    # one tree per collection: against the oracle's octree of each
    t = forces("fp64", True)
    want = []
    for b in parts:
        if len(b["x"]):
            o = OracleSim(threads=1)
            o.set_barnes_hut(True)
            o.set_bodies(b)
            want.append(np.array(o.forces()))
    assert rel_l2(t, np.concatenate(want, axis=1)) <= 1e-12
    assert rel_l2(forces("mixed", True), t) <= 1e-6
    with pytest.raises(NbgError):
        with Simulation("mixed") as s:
            s.set_collections(_tiny_sets(2049, 6))
