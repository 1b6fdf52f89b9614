"""nbg_forces_mixed_noalloc: the force pass for callers that cannot allocate
device memory (their memory pool owns the device, or they run where the
allocator must not be entered).  The caller passes device arrays; the library
works in its static scratch array.

Called through the C ABI twice in a row, its forces must agree with the
context entry point's (nbg_force_pass) within the mixed form's tolerance, at
a ragged size (not a multiple of the 512-body i-tile), a tile multiple and
the largest size the static array holds; on a small case they must also agree
with the CPU oracle's FP64 forces directly.  Sizes beyond the maximum must be
refused.  Calls of different sizes follow each other, so a call must not
depend on what an earlier one left in the shared array.

This file is collected last on purpose (tests run in file-name order)."""
import ctypes as C

import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation, load_library

pytestmark = pytest.mark.gpu
TOL = 1e-6  # relative L2, as for the mixed form elsewhere
MAX_BODIES = 65536


def rel_l2(a, b):
    num = np.sqrt(sum(np.sum((x - y) ** 2) for x, y in zip(a, b)))
    den = np.sqrt(sum(np.sum(y ** 2) for y in b))
    return num / den


def noalloc_calls(b, calls=2):
    """Forces of `calls` consecutive nbg_forces_mixed_noalloc calls on the
    body set b, each from freshly zeroed output arrays."""
    torch = pytest.importorskip("torch")
    lib = load_library()
    n = len(b["x"])
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(b[k])).to(dev) for k in ("x", "y", "z", "mass", "radius")}
    t["flags"] = torch.from_numpy(b["flags"].view(np.int32).copy()).to(dev)
    out = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(3)]
    ptr = lambda v: C.c_void_p(v.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream or None)
    results = []
    for _ in range(calls):
        for o in out:
            o.fill_(0.0)
        rc = lib.nbg_forces_mixed_noalloc(ptr(t["x"]), ptr(t["y"]), ptr(t["z"]), ptr(t["mass"]), ptr(t["radius"]),
                                          ptr(t["flags"]), n, ptr(out[0]), ptr(out[1]), ptr(out[2]), stream)
        torch.cuda.synchronize()
        assert rc == A.NBG_OK, lib.nbg_last_error(None)
        results.append([o.cpu().numpy() for o in out])
    return results


def live_mask(b):
    return (b["flags"] & (A.F_EXISTS | A.F_FRAGMENTING)) == A.F_EXISTS


# 1,000 bodies: a ragged last i-tile; 16,384: tile multiples; 65,536: the
# largest size the static array is laid out for
@pytest.mark.parametrize("n_each", [500, 8192, MAX_BODIES // 2])
def test_noalloc_force_pass_matches_context_entry_point(n_each):
    b = W.plummer_disk(n_each=n_each, seed=21)
    b["flags"][::97] = 0  # some bodies that do not exist
    assert len(b["x"]) == 2 * n_each
    with Simulation("mixed") as sim:
        sim.set_bodies(b)
        want = sim.force_pass()
    live = live_mask(b)
    for call, got in enumerate(noalloc_calls(b)):
        err = rel_l2([g[live] for g in got], [w[live] for w in want])
        assert err <= TOL, f"call {call}: rel L2 {err:.3e}"
        assert all(np.all(g[~live] == 0.0) for g in got), "bodies that do not exist must be left alone"


def test_noalloc_matches_oracle_fp64_forces():
    """Straight against the CPU oracle's FP64 force pass (the restatement of
    calcForceFrom), not through another entry point of this library; after
    the largest size has run, so the smaller call starts from whatever that
    call left in the shared array."""
    from oracle.oracle import OracleSim

    b = W.disk(n=1000, seed=23)
    b["flags"][5::131] |= A.F_FRAGMENTING  # fragmenting bodies get no force and exert none
    ref = OracleSim(threads=4)
    ref.set_bodies(b)
    want = ref.forces()
    live = live_mask(b)
    for call, got in enumerate(noalloc_calls(b)):
        err = rel_l2([g[live] for g in got], [w[live] for w in want])
        assert err <= TOL, f"call {call}: rel L2 {err:.3e} against the oracle"
        assert all(np.all(g[~live] == 0.0) for g in got)


def test_noalloc_rejects_sizes_beyond_the_maximum():
    lib = load_library()
    big = MAX_BODIES + 1
    rc = lib.nbg_forces_mixed_noalloc(*([C.c_void_p(8)] * 6), big, *([C.c_void_p(8)] * 3), None)
    assert rc == A.NBG_E_ARG
    assert b"65536" in lib.nbg_last_error(None)
