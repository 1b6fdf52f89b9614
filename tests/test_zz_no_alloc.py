"""nbg_forces_mixed_noalloc: the force pass for callers that cannot allocate
device memory (their memory pool owns the device, or they run where the
allocator must not be entered).  The caller passes device arrays; the library
works in its static scratch array.  Called through the C ABI twice in a row,
its forces must agree with the context entry point's (nbg_force_pass) within
the mixed form's tolerance, and sizes beyond the maximum must be refused.

This file is collected last on purpose (tests run in file-name order)."""
import ctypes as C

import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation, load_library

pytestmark = pytest.mark.gpu
TOL = 1e-6  # relative L2, as for the mixed form elsewhere


def rel_l2(a, b):
    num = np.sqrt(sum(np.sum((x - y) ** 2) for x, y in zip(a, b)))
    den = np.sqrt(sum(np.sum(y ** 2) for y in b))
    return num / den


def test_noalloc_force_pass_matches_context_entry_point():
    torch = pytest.importorskip("torch")
    lib = load_library()
    b = W.plummer_disk(n_each=8192, seed=21)
    b["flags"][::97] = 0  # some bodies that do not exist
    n = len(b["x"])
    with Simulation("mixed") as sim:
        sim.set_bodies(b)
        want = sim.force_pass()
    live = (b["flags"] & (A.F_EXISTS | A.F_FRAGMENTING)) == A.F_EXISTS
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(b[k])).to(dev) for k in ("x", "y", "z", "mass", "radius")}
    t["flags"] = torch.from_numpy(b["flags"].view(np.int32).copy()).to(dev)
    out = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(3)]
    ptr = lambda v: C.c_void_p(v.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream or None)
    for call in range(2):
        for o in out:
            o.fill_(0.0)
        rc = lib.nbg_forces_mixed_noalloc(ptr(t["x"]), ptr(t["y"]), ptr(t["z"]), ptr(t["mass"]), ptr(t["radius"]),
                                          ptr(t["flags"]), n, ptr(out[0]), ptr(out[1]), ptr(out[2]), stream)
        torch.cuda.synchronize()
        assert rc == A.NBG_OK, lib.nbg_last_error(None)
        got = [o.cpu().numpy() for o in out]
        err = rel_l2([g[live] for g in got], [w[live] for w in want])
        assert err <= TOL, f"call {call}: rel L2 {err:.3e}"
        assert all(np.all(g[~live] == 0.0) for g in got), "bodies that do not exist must be left alone"


def test_noalloc_rejects_sizes_beyond_the_maximum():
    lib = load_library()
    big = 65536 + 1
    rc = lib.nbg_forces_mixed_noalloc(*([C.c_void_p(8)] * 6), big, *([C.c_void_p(8)] * 3), None)
    assert rc == A.NBG_E_ARG
    assert b"65536" in lib.nbg_last_error(None)
