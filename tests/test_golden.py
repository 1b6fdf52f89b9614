"""Golden fixtures (tests/golden/*.json, made by tests/golden/make_golden.py,
an independent pure-Python restatement of the reference's cycle): the C
oracle (CPU) and the plain FP64 GPU path must reproduce every cycle bit for
bit, events included."""
import glob
import json
import os

import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from oracle.oracle import OracleSim

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.json")))
INT_FIELDS = {"id": np.int64, "collision": np.int32, "flags": np.uint32, "frag_fragments": np.int64}


def to_arrays(rows):
    out = {}
    for f, _, dt, _ in A.SOA_FIELDS:
        if f in INT_FIELDS:
            out[f] = np.array([r[f] for r in rows], dtype=INT_FIELDS[f])
        else:
            out[f] = np.array([float.fromhex(r[f]) for r in rows], dtype=np.float64)
    return out


def check_state(got, rows, where):
    exp = to_arrays(rows)
    assert len(got["x"]) == len(exp["x"]), f"{where}: count"
    for f in exp:
        a, b = np.asarray(got[f]), exp[f]
        if a.dtype.kind == "f":
            same = (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))
        else:
            same = a == b
        assert np.all(same), f"{where}: {f} differs at {np.flatnonzero(~same)[:5]}: {a[~same][:3]} vs {b[~same][:3]}"


def check_events(ev, exp, where):
    assert len(ev) == len(exp), f"{where}: {len(ev)} events, expected {len(exp)}"
    for k, (i1, i2, t) in enumerate(exp):
        assert (ev["id1"][k], ev["id2"][k], ev["type"][k]) == (i1, i2, t), f"{where}: event {k}"


def load(path):
    with open(path) as fh:
        return json.load(fh)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-5] for p in FIXTURES])
def test_oracle_matches_golden(path):
    fx = load(path)
    o = OracleSim(seed=fx["seed"])
    o.set_bodies(to_arrays(fx["bodies"]))
    o.set_next_id(fx["next_id"])
    for k, st in enumerate(fx["steps"]):
        o.step(fx["dt"], fx["R"], 1)
        check_events(o.events(), st["events"], f"cycle {k}")
        check_state(o.state(), st["state"], f"cycle {k}")
        assert o.next_id() == st["next_id"]


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-5] for p in FIXTURES])
def test_gpu_plain_matches_golden(path):
    from nbodygo_gb300.api import Simulation

    fx = load(path)
    sim = Simulation("fp64", seed=fx["seed"])
    sim.set_bodies(to_arrays(fx["bodies"]))
    sim.set_next_id(fx["next_id"])
    for k, st in enumerate(fx["steps"]):
        sim.step(fx["dt"], fx["R"], 1)
        check_events(sim.events(), st["events"], f"cycle {k}")
        check_state(sim.state(), st["state"], f"cycle {k}")
        assert sim.next_id() == st["next_id"]
