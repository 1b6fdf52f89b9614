"""Cycle-boundary controls addressed to one collection of a batched context
(nbg_add_bodies_to, nbg_remove_bodies_from, nbg_apply_edits_in,
nbg_get_body_in): the gRPC AddBody / RemoveBodies / ModBody / GetBody of one
simulation (cmd/sim/grpcsimcb.go:15-70) when many share a context.  Each
collection must stay bit-identical to its own oracle run given the same
controls; the others must not notice."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import NbgError, Simulation
from oracle.oracle import OracleSim

from helpers import assert_states_identical, rel_l2
from test_gpu_batch import split_state
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu
FIRST_NEW_ID = 1_000_000


def collections():
    return [W.disk(n=300, seed=1), dense_cluster(150, seed=2),
            W.plummer(n=257, seed=3, behavior=A.SUBSUME, radius_range=(0.5, 3.0)),
            W.uniform_ball(n=64, seed=4, R=50.0, radius=1.0, behavior=A.ELASTIC)]


def compare(gpu, oracles, where):
    counts = gpu.sim_counts()
    assert list(counts) == [o.count() for o in oracles], where
    for s, (got, o) in enumerate(zip(split_state(gpu.state(), counts), oracles)):
        exp = o.state()
        # fragment ids come from the context's one counter; everything else,
        # and every id given by the host, must match
        assert_states_identical(got, exp, fields=[f for f in got if f != "id"], where=f"{where} sim {s}")
        orig = exp["id"] < FIRST_NEW_ID
        assert np.array_equal(got["id"][orig], exp["id"][orig]), f"{where} sim {s}: ids"


def with_ids(b, first):
    b["id"][:] = np.arange(len(b["x"])) + first
    return b


def test_edits_addressed_to_one_collection_match_its_oracle():
    sims = collections()
    gpu = Simulation("fp64", seed=5)
    gpu.set_collections(sims)
    gpu.set_next_id(FIRST_NEW_ID)
    oracles = []
    for b in sims:
        o = OracleSim(seed=5, threads=4)
        o.set_bodies(b)
        o.set_next_id(FIRST_NEW_ID)
        oracles.append(o)
    dt, R = 0.02, 0.9

    def step(k):
        for _ in range(k):
            gpu.step(dt, R, 1)
            for o in oracles:
                o.step(dt, R, 1)

    step(3)
    compare(gpu, oracles, "before the controls")
    # adds to collection 2, then 0 (staged before 2's in the buffer), then 2
    # and 3 again: each collection's adds arrive newest first at its Cycle
    staged = [(2, with_ids(dense_cluster(3, seed=71), 9001)), (0, with_ids(dense_cluster(2, seed=72), 9101)),
              (2, with_ids(dense_cluster(1, seed=73), 9201)), (3, with_ids(dense_cluster(4, seed=74), 9301))]
    for s, b in staged:
        ids = gpu.add_bodies(b, sim=s)
        assert np.array_equal(ids, b["id"])
        oracles[s].add_bodies(b)
    # processDeletes on collection 1 alone
    assert gpu.remove_bodies(5, sim=1) == oracles[1].remove_bodies(5)
    # ModBody of id 5 in collection 3 only; of id 7 in every collection
    e5 = [{"id": 5, "mask": A.M_VX | A.M_MASS, "vx": 1.25, "mass": 3.5e11}]
    e7 = [{"id": 7, "mask": A.M_X | A.M_RADIUS, "x": 2.0, "radius": 0.75}]
    assert list(gpu.apply_edits(e5, sim=3)) == [1]
    oracles[3].apply_edits(e5)
    assert list(gpu.apply_edits(e7)) == [len(sims)]
    for o in oracles:
        o.apply_edits(e7)
    step(1)
    compare(gpu, oracles, "after the controls")
    step(4)
    compare(gpu, oracles, "4 cycles later")
    # GetBody within one collection: id 9001 lives in collection 2 only, and
    # id 5 of collection 3 is the one the edit gave mass 3.5e11
    got = gpu.get_body(9001, sim=2)
    assert got is not None and got["id"] == 9001
    assert gpu.get_body(9001, sim=1) is None
    c3 = split_state(gpu.state(), gpu.sim_counts())[3]
    k = int(np.flatnonzero(c3["id"] == 5)[0])
    assert gpu.get_body(5, sim=3)["mass"] == c3["mass"][k]
    assert gpu.get_body(5, sim=0)["mass"] == sims[0]["mass"][5]  # collection 0's id 5 was not edited
    gpu.close()


def test_collection_index_is_checked():
    with Simulation("fp64") as gpu:
        gpu.set_collections(collections())
        b = dense_cluster(2, seed=1)
        with pytest.raises(NbgError) as e:
            gpu.add_bodies(b)  # several collections: one must be named
        assert e.value.code == A.NBG_E_STATE
        with pytest.raises(NbgError) as e:
            gpu.add_bodies(b, sim=4)
        assert e.value.code == A.NBG_E_ARG
        with pytest.raises(NbgError) as e:
            gpu.remove_bodies(3)
        assert e.value.code == A.NBG_E_STATE
        with pytest.raises(NbgError) as e:
            gpu.remove_bodies(3, sim=-1)
        assert e.value.code == A.NBG_E_ARG


@pytest.mark.parametrize("shape", [0, 7, A.MIX_SYM])
def test_mixed_batch_stays_right_through_edits(shape):
    """The mixed form carries a Morton order between sorts; removals, adds
    and edits addressed to single collections change bodies' indices and
    positions.  After them the mixed forces must still be those of the
    bodies now in the context: within 1e-6 of an FP64 force pass of the
    same state."""
    sims = [W.plummer(n=800, seed=s) for s in (71, 72, 73)]
    m = Simulation("mixed", seed=5)
    m.set_option(A.OPT_MIX_SHAPE, shape)
    m.set_collections(sims)
    m.step(0.01, 1.0, 2)
    m.remove_bodies(100, sim=1)
    m.add_bodies(W.plummer(n=50, seed=74), sim=2)
    m.apply_edits([dict(id=int(sims[0]["id"][5]), mask=A.M_X | A.M_MASS, x=123.0, mass=5e13)], sim=0)
    m.step(0.01, 1.0, 1)
    counts = m.sim_counts()
    assert counts[1] < 800 and counts[2] > 800
    f = np.array(m.force_pass())
    st = m.state()
    with Simulation("fp64") as p:
        p.set_collections(split_state(st, counts))
        g = np.array(p.force_pass())
    assert rel_l2(f, g) <= 1e-6
    m.close()
