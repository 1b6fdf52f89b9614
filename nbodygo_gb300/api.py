"""Python host binding of libnbgpu.so.

`Simulation` owns one nbg_ctx: the device copy of a body collection and the
compute cycle on it.  Every method is a thin call into the C ABI
(include/nbgpu.h); there is no CPU code path - if the CUDA library is missing
or no GPU is visible, the constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libnbgpu.so")


class NbgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nbg status {code}: {msg}")
        self.code = code


def load_library(path=None):
    """Loads libnbgpu.so (built in-tree by nbodygo_gb300.build); raises if absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} not found: run `python -m nbodygo_gb300.build` (the CUDA library is required)")
    lib = C.CDLL(p)
    A.declare(lib)
    if path is None:
        _LIB = lib
    return lib


def probe_peaks(device=0):
    """(fp32 FLOP/s, fp64 FLOP/s, SM MHz) measured by FMA-chain kernels."""
    lib = load_library()
    f32, f64, mhz = C.c_double(), C.c_double(), C.c_double()
    rc = lib.nbg_probe_peaks(device, C.byref(f32), C.byref(f64), C.byref(mhz))
    if rc != A.NBG_OK:
        raise NbgError(rc, "peak probe failed")
    return f32.value, f64.value, mhz.value


def _adjacent(sims, k):
    """Field k of every collection as one array: a view when the collections'
    arrays already lie one after another in one buffer (no host copy), else
    their concatenation."""
    parts = [np.asarray(b[k]) for b in sims]
    first = parts[0]
    if all(p.flags.c_contiguous and p.dtype == first.dtype for p in parts):
        addr, ok = first.ctypes.data, True
        for p in parts:
            if p.ctypes.data != addr:
                ok = False
                break
            addr += p.nbytes
        if ok and first.ndim == 1:
            # every part is a live array and they tile one address range, so
            # the span from the first part's start is valid memory
            total = sum(len(p) for p in parts)
            return np.lib.stride_tricks.as_strided(first, shape=(total,), strides=(first.itemsize,))
    return np.concatenate(parts)


class Simulation:
    """A body collection on one GPU with the nbodygo compute cycle."""

    def __init__(self, precision="fp64", capacity=0, device=0, seed=None):
        self.lib = load_library()
        self.precision = precision
        p = A.PRECISION_MIXED if precision == "mixed" else A.PRECISION_FP64
        ctx = C.c_void_p()
        rc = self.lib.nbg_create(device, p, int(capacity), C.byref(ctx))
        if rc != A.NBG_OK:
            raise NbgError(rc, self.lib.nbg_last_error(None).decode())
        self.ctx = ctx
        if seed is not None:
            self._check(self.lib.nbg_set_seed(self.ctx, int(seed) & (2 ** 64 - 1)))

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.nbg_destroy(self.ctx)
            self.ctx = None
        self._ring = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != A.NBG_OK:
            raise NbgError(rc, self.lib.nbg_last_error(self.ctx).decode())

    # ---- configuration ----
    def set_precision(self, precision):
        self.precision = precision
        self._check(self.lib.nbg_set_precision(self.ctx, A.PRECISION_MIXED if precision == "mixed" else A.PRECISION_FP64))

    def set_stream(self, stream_handle):
        """Run on an external cudaStream_t (an int handle; 0/None = own stream)."""
        self._check(self.lib.nbg_set_stream(self.ctx, C.c_void_p(stream_handle or None)))

    def set_next_id(self, next_id):
        self._check(self.lib.nbg_set_next_id(self.ctx, int(next_id)))

    def next_id(self):
        v = C.c_int64()
        self._check(self.lib.nbg_get_next_id(self.ctx, C.byref(v)))
        return v.value

    def set_cycle(self, cycle):
        self._check(self.lib.nbg_set_cycle(self.ctx, int(cycle)))

    def set_option(self, key, value):
        self._check(self.lib.nbg_set_option(self.ctx, int(key), int(value)))

    def autotune(self, cache_path=None):
        """Times every compiled shape of the mixed pair kernel on the current
        collection and keeps the fastest; returns (shape, ms)."""
        v, ms = C.c_int32(), C.c_double()
        path = cache_path.encode() if cache_path else None
        self._check(self.lib.nbg_autotune(self.ctx, path, C.byref(v), C.byref(ms)))
        return v.value, ms.value

    def enable_timing(self, on=True):
        self._check(self.lib.nbg_enable_timing(self.ctx, 1 if on else 0))

    def timing(self):
        t = A.NbgTiming()
        self._check(self.lib.nbg_get_timing(self.ctx, C.byref(t)))
        return {"pair_ms": t.pair_ms, "other_ms": t.other_ms, "pair_launches": t.pair_launches,
                "kernel_launches": t.kernel_launches}

    # ---- body set ----
    def set_bodies(self, bodies):
        n = len(bodies["x"])
        soa, keep = A.soa_from_arrays(bodies)
        self._check(self.lib.nbg_set_bodies(self.ctx, C.byref(soa), n))
        del keep

    def set_collections(self, sims):
        """Several independent collections in one context (a list of body
        dicts); one step advances all of them, and they never interact."""
        counts = np.array([len(b["x"]) for b in sims], dtype=np.int64)
        keys = set(sims[0])
        for b in sims[1:]:
            keys &= set(b)
        cat = {k: _adjacent(sims, k) for k in keys}
        self.set_collections_flat(cat, counts)

    def set_collections_flat(self, bodies, counts):
        """Several collections given as one body dict whose arrays hold the
        collections one after another (collection s has counts[s] bodies):
        the layout nbg_set_collections takes, so nothing is copied on the
        host.  Pinned arrays go to the device through the copy kernel."""
        counts = np.ascontiguousarray(counts, dtype=np.int64)
        n = int(counts.sum())
        if any(len(v) != n for v in bodies.values()):
            raise ValueError("every array must hold sum(counts) bodies")
        soa, keep = A.soa_from_arrays(bodies)
        self._check(self.lib.nbg_set_collections(self.ctx, len(counts), counts.ctypes.data_as(C.POINTER(C.c_int64)),
                                                 C.byref(soa)))
        del keep

    def sim_counts(self):
        ns = C.c_int64()
        self._check(self.lib.nbg_sim_counts(self.ctx, None, 0, C.byref(ns)))
        out = np.zeros(max(1, ns.value), dtype=np.int64)
        self._check(self.lib.nbg_sim_counts(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int64)), ns.value,
                                            C.byref(ns)))
        return out[:ns.value]

    def count(self):
        v = C.c_int64()
        self._check(self.lib.nbg_count(self.ctx, C.byref(v)))
        return v.value

    def state(self, fields=None, out=None):
        """Body state as a dict of numpy arrays.  With `out` (a dict of
        contiguous arrays, e.g. in pinned memory) the state is copied into
        them, up to their length, and views of the filled part are returned."""
        if out is None:
            n = self.count()
            out = A.empty_state(n) if fields is None else {f: np.zeros(n, dtype=A.FIELD_DTYPES[f]) for f in fields}
            cap = n
        else:
            cap = min(len(v) for v in out.values())
        soa, keep = A.soa_from_arrays(out)
        got = C.c_int64()
        self._check(self.lib.nbg_get_state(self.ctx, C.byref(soa), cap, C.byref(got)))
        del keep
        m = min(cap, got.value)
        return {k: v[:m] for k, v in out.items()}

    def add_bodies(self, bodies, sim=None):
        """Enqueue(NewAdd) for every body; `sim` names one collection of a
        context holding several (nbg_add_bodies_to).  Returns the ids."""
        n = len(bodies["x"])
        soa, keep = A.soa_from_arrays(bodies)
        ids = np.zeros(max(n, 1), dtype=np.int64)
        pids = ids.ctypes.data_as(C.POINTER(C.c_int64))
        if sim is None:
            self._check(self.lib.nbg_add_bodies(self.ctx, C.byref(soa), n, pids))
        else:
            self._check(self.lib.nbg_add_bodies_to(self.ctx, int(sim), C.byref(soa), n, pids))
        del keep
        return ids[:n]

    def apply_edits(self, edits, sim=None):
        """ModBody by id; `sim` limits the edits to one collection."""
        arr = A.edit_array(edits)
        res = np.zeros(max(1, len(edits)), dtype=np.int32)
        pres = res.ctypes.data_as(C.POINTER(C.c_int32))
        if sim is None:
            self._check(self.lib.nbg_apply_edits(self.ctx, arr, len(edits), pres))
        else:
            self._check(self.lib.nbg_apply_edits_in(self.ctx, int(sim), arr, len(edits), pres))
        return res[:len(edits)]

    def remove_bodies(self, count, sim=None):
        """processDeletes; `sim` names one collection of several."""
        v = C.c_int64()
        if sim is None:
            self._check(self.lib.nbg_remove_bodies(self.ctx, int(count), C.byref(v)))
        else:
            self._check(self.lib.nbg_remove_bodies_from(self.ctx, int(sim), int(count), C.byref(v)))
        return v.value

    def get_body(self, body_id, sim=None):
        out = A.empty_state(1)
        soa, keep = A.soa_from_arrays(out)
        found = C.c_int32()
        if sim is None:
            self._check(self.lib.nbg_get_body(self.ctx, int(body_id), C.byref(soa), C.byref(found)))
        else:
            self._check(self.lib.nbg_get_body_in(self.ctx, int(sim), int(body_id), C.byref(soa), C.byref(found)))
        del keep
        if not found.value:
            return None
        return {k: v[0] for k, v in out.items()}

    # ---- snapshots ----
    def save_state(self):
        """The context's full state as a snapshot (bytes), to resume later
        with load_state in this or another context."""
        size = C.c_int64()
        self._check(self.lib.nbg_save_state(self.ctx, None, 0, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        self._check(self.lib.nbg_save_state(self.ctx, buf, size.value, C.byref(size)))
        return buf.raw[:size.value]

    def load_state(self, snapshot):
        data = bytes(snapshot)
        self._check(self.lib.nbg_load_state(self.ctx, data, len(data)))
        # the snapshot carries the form of the run it came from
        p = C.c_int()
        self._check(self.lib.nbg_get_precision(self.ctx, C.byref(p)))
        self.precision = "mixed" if p.value == A.PRECISION_MIXED else "fp64"

    # ---- the cycle ----
    def step(self, dt, R=1.0, nsteps=1):
        info = A.NbgStepInfo()
        self._check(self.lib.nbg_step(self.ctx, float(dt), float(R), int(nsteps), C.byref(info)))
        return {f: getattr(info, f) for f, _ in A.NbgStepInfo._fields_}

    def step_until(self, dt, R=1.0, nsteps=1):
        """Like step, but a call stopped by cancel() or the deadline option
        (OPT_STEP_DEADLINE_MS) returns (info, status) instead of raising:
        status is NBG_OK, NBG_E_CANCELLED or NBG_E_TIMEOUT, and info counts
        the cycles that ran."""
        info = A.NbgStepInfo()
        rc = self.lib.nbg_step(self.ctx, float(dt), float(R), int(nsteps), C.byref(info))
        if rc not in (A.NBG_OK, A.NBG_E_CANCELLED, A.NBG_E_TIMEOUT):
            self._check(rc)
        return {f: getattr(info, f) for f, _ in A.NbgStepInfo._fields_}, rc

    def cancel(self):
        """Stops the running (or next) step call at a cycle boundary; safe
        from another thread."""
        self._check(self.lib.nbg_cancel(self.ctx))

    def force_pass(self):
        """Recomputes the forces of the current state (no other change)."""
        self._check(self.lib.nbg_force_pass(self.ctx))
        return self.forces()

    def renderables(self):
        n = C.c_int64()
        self._check(self.lib.nbg_get_renderables(self.ctx, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=A.RENDERABLE_DTYPE)
        self._check(self.lib.nbg_get_renderables(self.ctx, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return out

    def set_render_ring(self, slots, slot_cap):
        """Attaches a render ring of `slots` slots of `slot_cap` renderables in
        host memory owned here; returns (headers, renderables) numpy views:
        headers[s] describes slot s, renderables[s, :written] its bodies."""
        nbytes = slots * A.RING_SLOT_DTYPE.itemsize + slots * slot_cap * A.RENDERABLE_DTYPE.itemsize
        buf = np.zeros(nbytes, dtype=np.uint8)
        self._check(self.lib.nbg_set_render_ring(self.ctx, buf.ctypes.data_as(C.c_void_p), int(slot_cap), int(slots)))
        self._ring = buf
        head = buf[:slots * A.RING_SLOT_DTYPE.itemsize].view(A.RING_SLOT_DTYPE)
        rend = buf[slots * A.RING_SLOT_DTYPE.itemsize:].view(A.RENDERABLE_DTYPE).reshape(slots, slot_cap)
        return head, rend

    def clear_render_ring(self):
        self._check(self.lib.nbg_set_render_ring(self.ctx, None, 0, 0))
        self._ring = None

    def events(self):
        n = C.c_int64()
        self._check(self.lib.nbg_get_events(self.ctx, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=A.EVENT_DTYPE)
        self._check(self.lib.nbg_get_events(self.ctx, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return out

    def forces(self):
        n = self.count()
        fx, fy, fz = (np.zeros(n) for _ in range(3))
        got = C.c_int64()
        pd = C.POINTER(C.c_double)
        self._check(self.lib.nbg_get_forces(self.ctx, fx.ctypes.data_as(pd), fy.ctypes.data_as(pd),
                                            fz.ctypes.data_as(pd), n, C.byref(got)))
        return fx, fy, fz

    def energy(self):
        ke, pe = C.c_double(), C.c_double()
        mom = (C.c_double * 3)()
        self._check(self.lib.nbg_energy(self.ctx, C.byref(ke), C.byref(pe), mom))
        return ke.value, pe.value, (mom[0], mom[1], mom[2])
