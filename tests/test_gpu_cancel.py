"""Stopping a long nbg_step at a cycle boundary: nbg_cancel from another
thread, or the per-call deadline (NBG_OPT_STEP_DEADLINE_MS).  The call
returns NBG_E_CANCELLED or NBG_E_TIMEOUT with the cycles it ran, and the
state is exactly that of a run of that many cycles - the context stays
usable.  No device wait is involved: the host stops launching."""
import threading
import time

import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation

from helpers import assert_states_identical

pytestmark = pytest.mark.gpu


def reference_state(bodies, cycles, seed=3):
    with Simulation("fp64", seed=seed) as s:
        s.set_bodies(bodies)
        if cycles:
            s.step(0.01, 1.0, cycles)
        return s.state()


def test_deadline_stops_at_a_cycle_boundary():
    bodies = W.plummer(n=4096, seed=12)
    with Simulation("fp64", seed=3) as s:
        s.set_bodies(bodies)
        s.step(0.01, 1.0, 1)  # warm: graphs and buffers exist
        s.set_option(A.OPT_STEP_DEADLINE_MS, 30)
        t0 = time.perf_counter()
        info, rc = s.step_until(0.01, 1.0, 20000)
        wall = time.perf_counter() - t0
        assert rc == A.NBG_E_TIMEOUT
        assert 0 < info["steps_done"] < 20000
        assert wall < 5.0, f"{wall:.2f} s"
        done = 1 + info["steps_done"]
        got = s.state()
        # the context stays usable: lift the deadline, run two more cycles
        s.set_option(A.OPT_STEP_DEADLINE_MS, 0)
        info2, rc2 = s.step_until(0.01, 1.0, 2)
        assert rc2 == A.NBG_OK and info2["steps_done"] == 2
        after = s.state()
    assert_states_identical(got, reference_state(bodies, done), where=f"after {done} cycles")
    assert_states_identical(after, reference_state(bodies, done + 2), where=f"after {done + 2} cycles")


def test_cancel_from_another_thread():
    bodies = W.plummer(n=4096, seed=13)
    with Simulation("fp64", seed=3) as s:
        s.set_bodies(bodies)
        s.set_option(A.OPT_GRAPH_CYCLES, 5)
        s.step(0.01, 1.0, 5)
        t = threading.Timer(0.05, s.cancel)
        t.start()
        info, rc = s.step_until(0.01, 1.0, 20000)
        t.join()
        assert rc == A.NBG_E_CANCELLED
        done = 5 + info["steps_done"]
        assert info["steps_done"] < 20000
        got = s.state()
        # a cancel is consumed by the call it stopped
        info2, rc2 = s.step_until(0.01, 1.0, 3)
        assert rc2 == A.NBG_OK and info2["steps_done"] == 3
    assert_states_identical(got, reference_state(bodies, done), where=f"after {done} cycles")


def test_cancel_before_a_call_stops_it_at_once():
    bodies = W.disk(n=200, seed=2)
    with Simulation("fp64") as s:
        s.set_bodies(bodies)
        before = s.state()
        s.cancel()
        info, rc = s.step_until(0.005, 1.0, 10)
        assert rc == A.NBG_E_CANCELLED and info["steps_done"] == 0
        assert_states_identical(s.state(), before, where="no cycle ran")
