"""ctypes declarations of include/nbgpu.h (the C ABI of libnbgpu.so).

The structures mirror the header field for field; `soa_from_arrays` builds an
nbg_soa that points into numpy arrays.  Shared by the product binding
(nbodygo_gb300.api) and by the oracle binding used in the tests.
"""
import ctypes as C

import numpy as np

NBG_OK = 0
NBG_E_CUDA = 1
NBG_E_ARG = 2
NBG_E_OVERFLOW = 3
NBG_E_TIMEOUT = 4
NBG_E_NAN = 5
NBG_E_STATE = 6
NBG_E_CANCELLED = 7

NONE, SUBSUME, ELASTIC, FRAGMENT = 0, 1, 2, 3

F_EXISTS = 0x01
F_IS_SUN = 0x02
F_PINNED = 0x04
F_TELEMETRY = 0x08
F_FRAGMENTING = 0x10
F_COLLIDED = 0x20

PRECISION_FP64 = 0
PRECISION_MIXED = 1

EV_COLLISION = 0
EV_SUBSUME = 1

M_X, M_Y, M_Z, M_VX, M_VY, M_VZ = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20
M_MASS, M_RADIUS, M_FRAG_FACTOR, M_FRAG_STEP = 0x40, 0x80, 0x100, 0x200
M_COLLISION, M_TELEMETRY, M_EXISTS = 0x400, 0x800, 0x1000

OPT_SPLIT = 1
OPT_GRAPH = 2
OPT_EV_CAP = 3
OPT_FRAG_CAP = 4
OPT_NEAR_PPM = 5
OPT_GRAPH_CYCLES = 6
OPT_MIX_SHAPE = 7
OPT_BARNES_HUT = 8
OPT_BH_SHAPE = 9
OPT_SORT_INTERVAL = 10
OPT_STEP_DEADLINE_MS = 12
OPT_EVENT_SORT = 13
OPT_TEST_WAIT_STALL = 14
OPT_TEST_FAIL_GROWTH = 15
OPT_P64_SPLIT_MAX = 11
MIX_SHAPES = 19
MIX_SYM = 15  # shapes 15 and 16: the symmetric kernel

_pd = C.POINTER(C.c_double)
_pi64 = C.POINTER(C.c_int64)
_pi32 = C.POINTER(C.c_int32)
_pu32 = C.POINTER(C.c_uint32)

# (field, ctypes pointer type, numpy dtype, required-on-input)
SOA_FIELDS = [
    ("id", _pi64, np.int64, False),
    ("x", _pd, np.float64, True),
    ("y", _pd, np.float64, True),
    ("z", _pd, np.float64, True),
    ("vx", _pd, np.float64, True),
    ("vy", _pd, np.float64, True),
    ("vz", _pd, np.float64, True),
    ("radius", _pd, np.float64, True),
    ("mass", _pd, np.float64, True),
    ("frag_factor", _pd, np.float64, False),
    ("frag_step", _pd, np.float64, False),
    ("collision", _pi32, np.int32, False),
    ("flags", _pu32, np.uint32, False),
    ("r", _pd, np.float64, False),
    ("fx", _pd, np.float64, False),
    ("fy", _pd, np.float64, False),
    ("fz", _pd, np.float64, False),
    ("frag_radius", _pd, np.float64, False),
    ("frag_new_radius", _pd, np.float64, False),
    ("frag_mass", _pd, np.float64, False),
    ("frag_fragments", _pi64, np.int64, False),
    ("frag_cx", _pd, np.float64, False),
    ("frag_cy", _pd, np.float64, False),
    ("frag_cz", _pd, np.float64, False),
]
FIELD_DTYPES = {f: dt for f, _, dt, _ in SOA_FIELDS}


class NbgSoa(C.Structure):
    # every field points into a host array (typed in nbgpu.h); void pointers
    # here take the arrays' addresses as integers, with no ctypes cast per
    # field on every call
    _fields_ = [(f, C.c_void_p) for f, _, _, _ in SOA_FIELDS]


class NbgStepInfo(C.Structure):
    _fields_ = [(f, C.c_int64) for f in (
        "steps_done", "n_bodies", "interactions", "events", "fragments_emitted", "removed", "nan_removed",
        "next_id", "bh_terms")]


class NbgRenderable(C.Structure):
    _fields_ = [("id", C.c_int64), ("x", C.c_float), ("y", C.c_float), ("z", C.c_float),
                ("flags", C.c_uint32), ("radius", C.c_double)]


class NbgEvent(C.Structure):
    _fields_ = [("id1", C.c_int64), ("id2", C.c_int64), ("type", C.c_int32), ("pad", C.c_int32)]


class NbgEdit(C.Structure):
    _fields_ = [("id", C.c_int64), ("mask", C.c_uint32), ("collision", C.c_int32),
                ("x", C.c_double), ("y", C.c_double), ("z", C.c_double),
                ("vx", C.c_double), ("vy", C.c_double), ("vz", C.c_double),
                ("mass", C.c_double), ("radius", C.c_double),
                ("frag_factor", C.c_double), ("frag_step", C.c_double),
                ("telemetry", C.c_int32), ("exists", C.c_int32)]


class NbgTiming(C.Structure):
    _fields_ = [("pair_ms", C.c_double), ("other_ms", C.c_double),
                ("pair_launches", C.c_int64), ("kernel_launches", C.c_int64)]


RENDERABLE_DTYPE = np.dtype([("id", np.int64), ("x", np.float32), ("y", np.float32), ("z", np.float32),
                             ("flags", np.uint32), ("radius", np.float64)])
EVENT_DTYPE = np.dtype([("id1", np.int64), ("id2", np.int64), ("type", np.int32), ("pad", np.int32)])
RING_SLOT_DTYPE = np.dtype([("cycle", np.int64), ("count", np.int64), ("written", np.int64), ("pad", np.int64)])
assert RENDERABLE_DTYPE.itemsize == C.sizeof(NbgRenderable)
assert EVENT_DTYPE.itemsize == C.sizeof(NbgEvent)


def soa_from_arrays(arrays):
    """nbg_soa pointing into a dict of contiguous numpy arrays (missing keys -> NULL).

    Returns (soa, keepalive) - keep `keepalive` referenced while the soa is used.
    """
    soa = NbgSoa()
    keep = []
    for f, _, dt, _ in SOA_FIELDS:
        a = arrays.get(f)
        if a is None:
            continue
        if not (isinstance(a, np.ndarray) and a.dtype == dt and a.flags.c_contiguous):
            a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        setattr(soa, f, a.ctypes.data)
    return soa, keep


def empty_state(n):
    """dict of numpy arrays for every SoA field, sized n."""
    return {f: np.zeros(n, dtype=dt) for f, _, dt, _ in SOA_FIELDS}


def edit_array(edits):
    """ctypes array of NbgEdit from a list of dicts (keys: id, mask, and values)."""
    arr = (NbgEdit * max(1, len(edits)))()
    for k, e in enumerate(edits):
        for key, v in e.items():
            setattr(arr[k], key, v)
    return arr


def declare(lib):
    """Sets argtypes/restype of every nbg_* function of a loaded libnbgpu."""
    P = C.c_void_p
    sigs = {
        "nbg_create": (C.c_int, [C.c_int, C.c_int, C.c_int64, C.POINTER(P)]),
        "nbg_destroy": (None, [P]),
        "nbg_last_error": (C.c_char_p, [P]),
        "nbg_set_precision": (C.c_int, [P, C.c_int]),
        "nbg_get_precision": (C.c_int, [P, C.POINTER(C.c_int)]),
        "nbg_set_stream": (C.c_int, [P, C.c_void_p]),
        "nbg_set_seed": (C.c_int, [P, C.c_uint64]),
        "nbg_set_next_id": (C.c_int, [P, C.c_int64]),
        "nbg_get_next_id": (C.c_int, [P, _pi64]),
        "nbg_set_cycle": (C.c_int, [P, C.c_uint64]),
        "nbg_set_bodies": (C.c_int, [P, C.POINTER(NbgSoa), C.c_int64]),
        "nbg_count": (C.c_int, [P, _pi64]),
        "nbg_set_collections": (C.c_int, [P, C.c_int64, _pi64, C.POINTER(NbgSoa)]),
        "nbg_sim_counts": (C.c_int, [P, _pi64, C.c_int64, _pi64]),
        "nbg_get_state": (C.c_int, [P, C.POINTER(NbgSoa), C.c_int64, _pi64]),
        "nbg_add_bodies": (C.c_int, [P, C.POINTER(NbgSoa), C.c_int64, _pi64]),
        "nbg_apply_edits": (C.c_int, [P, C.POINTER(NbgEdit), C.c_int64, _pi32]),
        "nbg_remove_bodies": (C.c_int, [P, C.c_int64, _pi64]),
        "nbg_get_body": (C.c_int, [P, C.c_int64, C.POINTER(NbgSoa), _pi32]),
        "nbg_add_bodies_to": (C.c_int, [P, C.c_int64, C.POINTER(NbgSoa), C.c_int64, _pi64]),
        "nbg_apply_edits_in": (C.c_int, [P, C.c_int64, C.POINTER(NbgEdit), C.c_int64, _pi32]),
        "nbg_remove_bodies_from": (C.c_int, [P, C.c_int64, C.c_int64, _pi64]),
        "nbg_get_body_in": (C.c_int, [P, C.c_int64, C.c_int64, C.POINTER(NbgSoa), _pi32]),
        "nbg_save_state": (C.c_int, [P, C.c_void_p, C.c_int64, _pi64]),
        "nbg_load_state": (C.c_int, [P, C.c_void_p, C.c_int64]),
        "nbg_step": (C.c_int, [P, C.c_double, C.c_double, C.c_int, C.POINTER(NbgStepInfo)]),
        "nbg_cancel": (C.c_int, [P]),
        "nbg_force_pass": (C.c_int, [P]),
        "nbg_get_renderables": (C.c_int, [P, C.c_void_p, C.c_int64, _pi64]),
        "nbg_get_events": (C.c_int, [P, C.c_void_p, C.c_int64, _pi64]),
        "nbg_set_render_ring": (C.c_int, [P, C.c_void_p, C.c_int64, C.c_int]),
        "nbg_get_forces": (C.c_int, [P, _pd, _pd, _pd, C.c_int64, _pi64]),
        "nbg_energy": (C.c_int, [P, _pd, _pd, _pd]),
        "nbg_enable_timing": (C.c_int, [P, C.c_int]),
        "nbg_get_timing": (C.c_int, [P, C.POINTER(NbgTiming)]),
        "nbg_set_option": (C.c_int, [P, C.c_int, C.c_int64]),
        "nbg_probe_peaks": (C.c_int, [C.c_int, _pd, _pd, _pd]),
        "nbg_autotune": (C.c_int, [P, C.c_char_p, _pi32, _pd]),
        "nbg_forces_mixed_noalloc": (C.c_int, [C.c_void_p] * 6 + [C.c_int64] + [C.c_void_p] * 4),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return list(sigs)
