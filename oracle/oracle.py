"""Python binding of the CPU oracle (oracle/libnbg_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker or the timed CPU restatement of
the reference.  The product never imports it.
"""
import ctypes as C
import os

import numpy as np

from nbodygo_gb300 import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbg_oracle.so")
# the same restatement with the platform libm's transcendentals in the elastic
# collision instead of nbg_math.h (bounds the effect of that substitution)
LIBM_LIB_PATH = os.path.join(HERE, "libnbg_oracle_libm.so")
_LIBS = {}


def load(libm=False):
    if libm in _LIBS:
        return _LIBS[libm]
    path = LIBM_LIB_PATH if libm else LIB_PATH
    if not os.path.exists(path):
        from nbodygo_gb300 import build as _b
        _b.build_oracle()
    lib = C.CDLL(path)
    P = C.c_void_p
    pd = C.POINTER(C.c_double)
    sig = {
        "nbo_create": (P, [C.c_uint64]),
        "nbo_destroy": (None, [P]),
        "nbo_set_bodies": (C.c_int, [P, C.POINTER(A.NbgSoa), C.c_int64]),
        "nbo_count": (C.c_int64, [P]),
        "nbo_set_barnes_hut": (None, [P, C.c_int]),
        "nbo_get_state": (C.c_int, [P, C.POINTER(A.NbgSoa), C.c_int64]),
        "nbo_set_next_id": (None, [P, C.c_int64]),
        "nbo_get_next_id": (C.c_int64, [P]),
        "nbo_set_cycle": (None, [P, C.c_uint64]),
        "nbo_add_bodies": (C.c_int, [P, C.POINTER(A.NbgSoa), C.c_int64, C.POINTER(C.c_int64)]),
        "nbo_remove_bodies": (C.c_int64, [P, C.c_int64]),
        "nbo_apply_edit": (C.c_int32, [P, C.POINTER(A.NbgEdit)]),
        "nbo_step": (C.c_int, [P, C.c_double, C.c_double, C.c_int, C.c_int]),
        "nbo_phase_compute": (None, [P, C.c_int]),
        "nbo_phase_process_mods": (None, [P]),
        "nbo_phase_update": (None, [P, C.c_double, C.c_double]),
        "nbo_phase_cycle": (None, [P, C.c_double]),
        "nbo_enqueue_event": (C.c_int, [P, C.c_int, C.c_int64, C.c_int64]),
        "nbo_last_events": (C.c_int64, [P, C.c_void_p, C.c_int64]),
        "nbo_last_info": (None, [P, C.POINTER(A.NbgStepInfo)]),
        "nbo_forces": (C.c_int, [P, pd, pd, pd, C.c_int]),
        "nbo_forces_subset": (C.c_int, [P, C.POINTER(C.c_int64), C.c_int64, pd, pd, pd]),
        "nbo_math_eval": (C.c_double, [C.c_int, C.c_double, C.c_double]),
        "nbo_frag_point": (None, [C.c_uint64, C.c_int64, C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_double, pd]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[libm] = lib
    return lib


class OracleSim:
    """Same surface as nbodygo_gb300.api.Simulation, on the CPU restatement."""

    def __init__(self, seed=0x6E626F6479676F31, threads=1, libm=False):
        self.lib = load(libm)
        self.s = self.lib.nbo_create(int(seed) & (2 ** 64 - 1))
        self.threads = threads

    def close(self):
        if self.s:
            self.lib.nbo_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bodies(self, bodies):
        n = len(bodies["x"])
        soa, keep = A.soa_from_arrays(bodies)
        rc = self.lib.nbo_set_bodies(self.s, C.byref(soa), n)
        assert rc == 0
        del keep

    def set_barnes_hut(self, on=True):
        """Forces from the reference's octree (cmd/body/octree.go) instead of the direct sum."""
        self.lib.nbo_set_barnes_hut(self.s, 1 if on else 0)

    def count(self):
        return self.lib.nbo_count(self.s)

    def state(self):
        n = self.count()
        out = A.empty_state(n)
        soa, keep = A.soa_from_arrays(out)
        self.lib.nbo_get_state(self.s, C.byref(soa), n)
        del keep
        return out

    def set_next_id(self, v):
        self.lib.nbo_set_next_id(self.s, int(v))

    def next_id(self):
        return self.lib.nbo_get_next_id(self.s)

    def set_cycle(self, c):
        self.lib.nbo_set_cycle(self.s, int(c))

    def add_bodies(self, bodies):
        n = len(bodies["x"])
        soa, keep = A.soa_from_arrays(bodies)
        ids = np.zeros(max(n, 1), dtype=np.int64)
        self.lib.nbo_add_bodies(self.s, C.byref(soa), n, ids.ctypes.data_as(C.POINTER(C.c_int64)))
        return ids[:n]

    def remove_bodies(self, count):
        return self.lib.nbo_remove_bodies(self.s, int(count))

    def apply_edits(self, edits):
        arr = A.edit_array(edits)
        return np.array([self.lib.nbo_apply_edit(self.s, C.byref(arr[k])) for k in range(len(edits))],
                        dtype=np.int32)

    def step(self, dt, R=1.0, nsteps=1, threads=None):
        self.lib.nbo_step(self.s, float(dt), float(R), int(nsteps), int(threads or self.threads))
        info = A.NbgStepInfo()
        self.lib.nbo_last_info(self.s, C.byref(info))
        return {f: getattr(info, f) for f, _ in A.NbgStepInfo._fields_}

    def events(self):
        n = self.lib.nbo_last_events(self.s, None, 0)
        out = np.zeros(n, dtype=A.EVENT_DTYPE)
        self.lib.nbo_last_events(self.s, out.ctypes.data_as(C.c_void_p), n)
        return out

    def forces(self, threads=None):
        n = self.count()
        fx, fy, fz = (np.zeros(n) for _ in range(3))
        pd = C.POINTER(C.c_double)
        self.lib.nbo_forces(self.s, fx.ctypes.data_as(pd), fy.ctypes.data_as(pd), fz.ctypes.data_as(pd),
                            int(threads or self.threads))
        return fx, fy, fz

    def forces_subset(self, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        fx, fy, fz = (np.zeros(len(idx)) for _ in range(3))
        pd = C.POINTER(C.c_double)
        rc = self.lib.nbo_forces_subset(self.s, idx.ctypes.data_as(C.POINTER(C.c_int64)), len(idx),
                                        fx.ctypes.data_as(pd), fy.ctypes.data_as(pd), fz.ctypes.data_as(pd))
        assert rc == 0
        return fx, fy, fz

    # phases, for tests mirroring the reference's unit tests
    def compute(self, threads=None):
        self.lib.nbo_phase_compute(self.s, int(threads or self.threads))

    def process_mods(self):
        self.lib.nbo_phase_process_mods(self.s)

    def update(self, dt, R):
        self.lib.nbo_phase_update(self.s, float(dt), float(R))

    def cycle(self, R):
        self.lib.nbo_phase_cycle(self.s, float(R))

    def enqueue_event(self, ev_type, i, j):
        assert self.lib.nbo_enqueue_event(self.s, int(ev_type), int(i), int(j)) == 0


def math_eval(which, a, b=0.0):
    """The shared FP64 functions of nbg_math.h (0 sin .. 7 Go's math.Min)."""
    return load().nbo_math_eval(int(which), float(a), float(b))


def frag_point(seed, parent_id, cycle, cnt, center, radius):
    out = (C.c_double * 3)()
    load().nbo_frag_point(int(seed) & (2 ** 64 - 1), int(parent_id), int(cycle), int(cnt), float(center[0]),
                          float(center[1]), float(center[2]), float(radius), out)
    return out[0], out[1], out[2]
