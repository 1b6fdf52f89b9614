"""Loading and reading back a collection through pinned host arrays (one
copy kernel over the host link) gives exactly what pageable arrays (DMA
copies) give."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation

pytestmark = pytest.mark.gpu


def pinned_copy(torch, arrays, extra=0):
    out, keep = {}, []
    for k, v in arrays.items():
        tdt = torch.int32 if v.dtype == np.uint32 else getattr(torch, str(v.dtype))
        t = torch.zeros(len(v) + extra, dtype=tdt, pin_memory=True)
        keep.append(t)
        a = t.numpy().view(v.dtype)
        a[:len(v)] = v
        out[k] = a
    return out, keep


def test_pinned_and_pageable_io_agree():
    torch = pytest.importorskip("torch")
    b = W.plummer_disk(2000, seed=5)
    pinned, keep = pinned_copy(torch, b)
    ref = Simulation("mixed")
    ref.set_bodies(b)
    ref.step(0.01, 1.0, 3)
    got = Simulation("mixed")
    got.set_bodies(pinned)
    got.step(0.01, 1.0, 3)
    pageable = ref.state()
    out, keep2 = pinned_copy(torch, A.empty_state(len(pageable["x"])), extra=16)
    pin = got.state(out=out)
    for f in pageable:
        a, c = np.asarray(pageable[f]), np.asarray(pin[f])
        assert len(a) == len(c)
        if a.dtype.kind == "f":
            assert np.array_equal(a.view(np.uint64), c.view(np.uint64)), f
        else:
            assert np.array_equal(a, c), f


def test_pinned_flag_fields_every_behaviour():
    """The flag byte and the collision behaviour reach pinned outputs through
    the copy kernel's split; a pinned/pageable mix goes through the staging
    path.  Both equal the pageable read of a collection holding every
    behaviour after removals and fragments."""
    torch = pytest.importorskip("torch")
    from test_gpu_plain_parity import dense_cluster

    sim = Simulation("fp64")
    sim.set_bodies(dense_cluster(300, seed=11))
    sim.step(0.01, 1.0, 4)
    ref = sim.state()
    assert len(set(ref["collision"].tolist())) > 1
    n = len(ref["x"])
    out, keep = pinned_copy(torch, A.empty_state(n), extra=8)
    got = sim.state(out=out)
    for f in ("flags", "collision", "id", "x"):
        assert np.array_equal(np.asarray(ref[f]), np.asarray(got[f])), f
    mixed = dict(out)
    mixed["collision"] = np.zeros(n + 8, dtype=ref["collision"].dtype)  # pageable
    got = sim.state(out=mixed)
    for f in ("flags", "collision"):
        assert np.array_equal(np.asarray(ref[f]), np.asarray(got[f])), f
