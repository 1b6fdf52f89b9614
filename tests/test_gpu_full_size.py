"""The mixed form at the full sizes of the measured workloads, each against an
FP64 reference:

- the 512-collection ensemble (3.3 M bodies): mixed forces against the plain
  FP64 GPU forces (bit-identical to the oracle), relative L2 <= 1e-6 in every
  collection and over all of them;
- the 2^20-body uniform ball: 1,024 bodies spread over the ball against the
  CPU oracle's FP64 forces;
- the 131,072-body Plummer sphere + disk over its stated 1,000 cycles: the
  subsume events conserve mass to 1e-12, and the first 10 cycles resolve the
  same events and remove the same bodies as the plain FP64 form.
"""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-6


def test_ensemble_mixed_against_fp64_in_every_collection():
    sims = W.ensemble()
    n = sum(len(s["x"]) for s in sims)
    with Simulation("mixed", capacity=n) as m:
        m.set_collections(sims)
        f = m.force_pass()
    with Simulation("fp64", capacity=n) as p:
        p.set_collections(sims)
        g = p.force_pass()
    assert rel_l2(f, g) <= TOL
    o, worst = 0, 0.0
    for s in sims:
        k = len(s["x"])
        worst = max(worst, rel_l2([c[o:o + k] for c in f], [c[o:o + k] for c in g]))
        o += k
    assert worst <= TOL, f"worst collection rel L2 {worst:.3e}"


def test_uniform_ball_1024_bodies_against_the_oracle():
    b = W.uniform_ball()
    with Simulation("mixed", capacity=len(b["x"])) as m:
        m.set_bodies(b)
        f = m.force_pass()
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    idx = np.arange(1024) * (len(b["x"]) // 1024) + 511
    g = ora.forces_subset(idx)
    err = rel_l2([c[idx] for c in f], g)
    assert err <= TOL, f"rel L2 {err:.3e}"


def test_plummer_disk_1000_cycles_conserve_mass_and_match_fp64_events():
    b = W.plummer_disk()
    dt = 0.01
    m = Simulation("mixed", capacity=len(b["x"]) + 4096)
    p = Simulation("fp64", capacity=len(b["x"]) + 4096)
    m.set_bodies(b)
    p.set_bodies(b)
    m0 = float(np.sum(b["mass"]))
    for c in range(10):
        im, ip = m.step(dt, 1.0, 1), p.step(dt, 1.0, 1)
        assert (im["events"], im["removed"], im["n_bodies"]) == (ip["events"], ip["removed"], ip["n_bodies"]), \
            f"cycle {c}"
        em, ep = m.events(), p.events()
        assert np.array_equal(em["id1"], ep["id1"]) and np.array_equal(em["id2"], ep["id2"]), f"cycle {c}"
    p.close()
    m.set_option(A.OPT_GRAPH_CYCLES, 10)
    done, events = 10, 0
    while done < 1000:
        info = m.step(dt, 1.0, 10)
        done += info["steps_done"]
        events += info["events"]
    st = m.state()
    live = (st["flags"] & A.F_EXISTS) != 0
    drift = abs(float(np.sum(st["mass"][live])) - m0) / m0
    assert events > 100
    assert drift <= 1e-12, f"mass drift {drift:.3e} over 1,000 cycles"
    m.close()
