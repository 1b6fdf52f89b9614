"""The reference's own tests for this path, restated against the CPU oracle.

Each test names the Go test it restates.  Where the Go test only checks a
property (e.g. "Vx != 0"), the restatement also pins the exact value, derived
here independently with Python floats (IEEE doubles, no fused operations).
"""
import math

import numpy as np

from nbodygo_gb300 import _abi as A
from oracle.oracle import OracleSim

G = 6.673e-11


def create_test_bodies(cnt):
    """createTestBodies / createTestBody (cmd/body/body_collection_test.go:15-56):
    body i has every numeric field equal to i, Elastic, r = 1."""
    i = np.arange(cnt, dtype=np.float64)
    return {
        "id": np.arange(cnt, dtype=np.int64),
        "x": i.copy(), "y": i.copy(), "z": i.copy(),
        "vx": i.copy(), "vy": i.copy(), "vz": i.copy(),
        "radius": i.copy(), "mass": i.copy(),
        "frag_factor": i.copy(), "frag_step": i.copy(),
        "collision": np.full(cnt, A.ELASTIC, dtype=np.int32),
        "flags": np.full(cnt, A.F_EXISTS, dtype=np.uint32),
        "r": np.ones(cnt),
    }


def test_wp_compute_exact():
    """TestWpCompute (cmd/runner/workpool_test.go:41-56): two bodies at (1,1,1)
    and (22,22,22), m=1, r=1, v=0; Compute then Update(1, 1): Vx != 0."""
    b = create_test_bodies(2)
    for k, (p, bid) in enumerate(((1.0, 1), (22.0, 2))):
        b["x"][k] = b["y"][k] = b["z"][k] = p
        b["vx"][k] = b["vy"][k] = b["vz"][k] = 0.0
        b["mass"][k] = 1.0
        b["radius"][k] = 1.0
        b["frag_factor"][k] = b["frag_step"][k] = 0.0
        b["id"][k] = bid
    o = OracleSim()
    o.set_bodies(b)
    o.compute(threads=1)
    o.update(1.0, 1.0)
    s = o.state()
    assert s["vx"][0] != 0 and s["vx"][1] != 0
    # exact value: calcForceFrom + Update with Go's operation order
    dx = 22.0 - 1.0
    dist = math.sqrt(dx * dx + dx * dx + dx * dx)
    force = G * 1.0 * 1.0 / (dist * dist)
    f = force * dx / dist
    v = 0.0 + 1.0 * f / 1.0
    assert s["vx"][0] == v and s["vy"][0] == v and s["vz"][0] == v
    assert s["vx"][1] == -v
    assert s["x"][0] == 1.0 + 1.0 * v


def test_collide_coincident_bodies():
    """TestCollide (body_collection_test.go:319-344): two bodies at the same
    point; after ProcessMods both are marked collided.  With d = 0, acos(0/0)
    is NaN, the NaN comparisons fall through, and the velocities become NaN."""
    b = create_test_bodies(5000)
    for idx in (2999, 3999):
        b["x"][idx] = b["y"][idx] = b["z"][idx] = 500.0
    o = OracleSim()
    o.set_bodies(b)
    o.enqueue_event(A.EV_COLLISION, 2999, 3999)
    o.process_mods()
    s = o.state()
    assert s["flags"][2999] & A.F_COLLIDED and s["flags"][3999] & A.F_COLLIDED
    assert np.isnan(s["vx"][2999]) and np.isnan(s["vz"][3999])
    ev = o.events()
    assert len(ev) == 1 and ev["id1"][0] == 2999 and ev["id2"][0] == 3999


def test_subsume():
    """TestSubsume (body_collection_test.go:288-313)."""
    b = create_test_bodies(500)
    o = OracleSim()
    o.set_bodies(b)
    o.enqueue_event(A.EV_SUBSUME, 10, 444)
    o.process_mods()
    s = o.state()
    assert s["flags"][10] & A.F_EXISTS
    assert not (s["flags"][444] & A.F_EXISTS)
    assert s["mass"][10] == 10.0 + 444.0 and s["mass"][444] == 0.0


def test_remove():
    """TestRemove (body_collection_test.go:73-88): Cycle compacts."""
    b = create_test_bodies(1000)
    b["flags"][10] = 0
    o = OracleSim()
    o.set_bodies(b)
    o.cycle(1.0)
    s = o.state()
    assert o.count() == 999
    assert 10 not in set(s["id"].tolist())
    assert np.array_equal(s["id"], np.delete(np.arange(1000), 10))


def test_adds():
    """TestAdds (body_collection_test.go:268-281): an enqueued add appears
    after Cycle, with r = R."""
    o = OracleSim()
    o.set_bodies(create_test_bodies(500))
    add = create_test_bodies(601)
    add = {k: v[600:601] for k, v in add.items()}
    o.add_bodies(add)
    o.cycle(0.25)
    s = o.state()
    assert o.count() == 501 and s["id"][500] == 600 and s["r"][500] == 0.25


def test_adds_newest_first():
    """Cycle appends adds in events-list order, and the list is built with
    PushFront (body_collection.go:100, 283-290): newest first."""
    o = OracleSim()
    o.set_bodies(create_test_bodies(3))
    add = create_test_bodies(3)
    add["id"][:] = -1
    ids = o.add_bodies(add)
    o.cycle(1.0)
    s = o.state()
    assert list(s["id"][3:]) == list(ids[::-1])


def test_init_size():
    """TestInitSize (body_collection_test.go:61-67): 1M bodies, none lost."""
    o = OracleSim()
    o.set_bodies(create_test_bodies(1_000_000))
    assert o.count() == 1_000_000


def test_id_gen():
    """TestIdGen (body_test.go:50-67): 10 x 1000 NextId calls, then 10000."""
    o = OracleSim()
    o.set_bodies(create_test_bodies(1))
    for _ in range(10):
        add = create_test_bodies(1000)
        add["id"][:] = -1
        o.add_bodies(add)
    assert o.next_id() == 10_000


def test_remove_bodies_stride():
    """processDeletes (computation-runner.go:176-216): every Count()/n-th body
    (or the next unpinned, existing one) is removed; the walk does not stop at
    n, and pinned bodies are skipped."""
    b = create_test_bodies(105)
    b["flags"][20] |= A.F_PINNED
    o = OracleSim()
    o.set_bodies(b)
    removed = o.remove_bodies(10)
    s = o.state()
    gone = [int(i) for i in s["id"][(s["flags"] & A.F_EXISTS) == 0]]
    # step = 105 // 10 = 10; body 20 is pinned so 21 goes instead; 100 is the 11th
    assert gone == [0, 10, 21, 30, 40, 50, 60, 70, 80, 90, 100]
    assert removed == 11
    assert all(s["mass"][i] == 0 for i in gone)
    o2 = OracleSim()
    o2.set_bodies(create_test_bodies(7))
    assert o2.remove_bodies(-1) == 7


def test_self_collision_events_are_no_ops():
    """Compute enqueues collision(b, b) for every Elastic body every cycle
    (Collided(b, b) is true, d = 0); resolving it is a no-op because the
    relative speed is 0 (collisioncalc.go:89-92)."""
    b = create_test_bodies(4)
    b["x"][:] = [0.0, 100.0, 200.0, 300.0]
    b["y"][:] = 0
    b["z"][:] = 0
    b["radius"][:] = 1.0
    b["mass"][:] = 1.0
    o = OracleSim()
    o.set_bodies(b)
    before = o.state()
    for i in range(4):
        o.enqueue_event(A.EV_COLLISION, i, i)
    o.process_mods()
    after = o.state()
    for f in ("vx", "vy", "vz", "mass", "flags"):
        assert np.array_equal(before[f], after[f])
    assert len(o.events()) == 0  # self events are not reported
