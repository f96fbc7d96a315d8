"""ctypes binding of libsbc_gb300.so (the C-ABI in include/sbc_gb300.h and the
drop-in streamingbc.h / stinger.h surface).

This is how the tests and the benchmark call the CUDA path: through the same
exported C symbols a reference-side caller would bind.  Loading fails loudly
when the library is missing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import weakref

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libsbc_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)
_vp = C.c_void_p


class SbcError(RuntimeError):
    pass


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("batches", C.c_int64),
                ("graphs_admitted", C.c_int64), ("graphs_waiting", C.c_int64), ("p50_us", C.c_double),
                ("p99_us", C.c_double), ("mean_us", C.c_double), ("max_us", C.c_double),
                ("throughput", C.c_double), ("mean_batch", C.c_double), ("bytes_admitted", C.c_int64),
                ("bytes_budget", C.c_int64)]


class ModelStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("train_samples", C.c_int64), ("val_samples", C.c_int64),
                ("steps", C.c_int64), ("epochs", C.c_int), ("train_ms", C.c_double), ("val_mae", C.c_double),
                ("val_rmse", C.c_double), ("val_mae_mean", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("inserted", "duplicates", "invalid", "roots_active", "case1", "case2",
                                          "vertices", "edges", "scanned")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Profile(C.Structure):
    _fields_ = [("static_ms", C.c_double), ("static_launches", C.c_int64),
                ("append_ms", C.c_double), ("append_launches", C.c_int64),
                ("classify_ms", C.c_double), ("classify_launches", C.c_int64),
                ("update_ms", C.c_double), ("update_launches", C.c_int64),
                ("batch_ms", C.c_double), ("batches", C.c_int64)]

    def as_dict(self) -> dict:
        return {n: (float(getattr(self, n)) if t is C.c_double else int(getattr(self, n))) for n, t in self._fields_}


def header_functions() -> list[str]:
    """Every function name declared in include/*.h."""
    names = []
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", text):
            name = m.group(1)
            if name in ("if", "while", "for", "sizeof", "return"):
                continue
            names.append(name)
    return sorted(set(names))


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (no build, no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SbcError(f"{path} is missing: build it with streamingbc_gb300.build.build()")
    lib = C.CDLL(path)
    sig = {
        "sbc_last_error": (C.c_char_p, []),
        "sbc_set_device": (C.c_int, [C.c_int]),
        "sbc_graph_create": (C.c_int, [C.POINTER(_vp), C.c_int64, _i64p, _i64p]),
        "sbc_graph_destroy": (C.c_int, [_vp]),
        "sbc_graph_num_vertices": (C.c_int, [_vp, _i64p]),
        "sbc_graph_degree": (C.c_int, [_vp, C.c_int64, _i64p]),
        "sbc_graph_insert_directed": (C.c_int, [_vp, C.c_int64, C.c_int64, C.POINTER(C.c_int)]),
        "sbc_graph_to_csr": (C.c_int, [_vp, _i64p, _i64p]),
        "sbc_graph_reserve": (C.c_int, [_vp, C.c_int64, _i64p, _i64p]),
        "sbc_graph_repacks": (C.c_int, [_vp, _i64p]),
        "sbc_forest_create": (C.c_int, [C.POINTER(_vp), _vp, C.c_int64, _i64p, C.c_int64]),
        "sbc_forest_create_ex": (C.c_int, [C.POINTER(_vp), _vp, C.c_int64, _i64p, C.c_int64, C.c_int]),
        "sbc_update_variant_count": (C.c_int, [C.POINTER(C.c_int)]),
        "sbc_update_variant_info": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_int)]),
        "sbc_forest_destroy": (C.c_int, [_vp]),
        "sbc_forest_info": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p]),
        "sbc_static_init": (C.c_int, [_vp]),
        "sbc_insert_batch": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.POINTER(BatchStats)]),
        "sbc_insert_batch_device": (C.c_int, [_vp, C.c_int64, _vp, _vp]),
        "sbc_set_graph_capture": (C.c_int, [_vp, C.c_int]),
        "sbc_forest_set_variant": (C.c_int, [_vp, C.c_int]),
        "sbc_forest_variant": (C.c_int, [_vp, C.POINTER(C.c_int)]),
        "sbc_forest_set_delete_mode": (C.c_int, [_vp, C.c_int]),
        "sbc_forest_autotune": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.c_int, C.POINTER(C.c_int), _f64p,
                                          C.c_int]),
        "sbc_cost_model_size": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "sbc_cost_log_start": (C.c_int, [_vp, C.c_int64]),
        "sbc_cost_log_stop": (C.c_int, [_vp, _i64p]),
        "sbc_cost_log_read": (C.c_int, [_vp, C.c_int64, C.c_int64, _f32p, _f32p]),
        "sbc_cost_model_train": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64,
                                           C.POINTER(ModelStats)]),
        "sbc_set_schedule": (C.c_int, [_vp, C.c_int]),
        "sbc_forest_compare_schedules": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.c_int, _f64p, _f64p]),
        "sbc_cost_model_params": (C.c_int, [_vp, _f32p, _f32p]),
        "sbc_cost_model_predict": (C.c_int, [_vp, C.c_int64, _f32p, _f32p]),
        "sbc_cost_model_grad": (C.c_int, [_vp, C.c_int64, _f32p, _f32p, _f32p, _f32p]),
        "sbc_get_level_hist": (C.c_int, [_vp, C.c_int64, C.c_int64, _i32p]),
        "sbc_get_roster": (C.c_int, [_vp, C.c_int64, C.c_int, _i32p, C.POINTER(C.c_int)]),
        "sbc_insert_batch_async": (C.c_int, [_vp, C.c_int64, _i64p, _i64p]),
        "sbc_delete_batch": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.POINTER(BatchStats)]),
        "sbc_update_deleted": (C.c_int, [_vp, C.c_int64, C.c_int64, C.POINTER(BatchStats)]),
        "sbc_graph_remove_directed": (C.c_int, [_vp, C.c_int64, C.c_int64, C.POINTER(C.c_int)]),
        "sbc_server_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int64, C.c_int]),
        "sbc_server_destroy": (C.c_int, [_vp]),
        "sbc_server_set_max_inflight": (C.c_int, [_vp, C.c_int]),
        "sbc_server_set_tuning": (C.c_int, [_vp, C.c_int, C.c_int64]),
        "sbc_server_add_graph": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.c_int64, _i64p, C.c_int,
                                           C.POINTER(C.c_int)]),
        "sbc_server_graph_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), _i64p, _i64p, _i64p]),
        "sbc_server_submit": (C.c_int, [_vp, C.c_int, C.c_int64, C.c_int64]),
        "sbc_server_play": (C.c_int, [_vp, C.c_int64, _i32p, _i64p, _i64p, _f64p]),
        "sbc_server_drain": (C.c_int, [_vp]),
        "sbc_server_error": (C.c_char_p, [_vp]),
        "sbc_server_release": (C.c_int, [_vp, C.c_int]),
        "sbc_server_evict": (C.c_int, [_vp, C.c_int]),
        "sbc_checkpoint_take": (C.c_int, [_vp, C.POINTER(_vp)]),
        "sbc_checkpoint_restore": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp)]),
        "sbc_checkpoint_save": (C.c_int, [_vp, C.c_char_p]),
        "sbc_checkpoint_load": (C.c_int, [C.c_char_p, C.POINTER(_vp)]),
        "sbc_checkpoint_info": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p]),
        "sbc_checkpoint_read": (C.c_int, [_vp, _i32p, _i64p, _f64p]),
        "sbc_checkpoint_free": (C.c_int, [_vp]),
        "sbc_forest_roots": (C.c_int, [_vp, _i64p]),
        "sbc_group_get_bc": (C.c_int, [_vp, _f64p]),
        "sbc_dimacs_read": (C.c_int, [C.c_char_p, _i64p, _i64p, C.POINTER(_i64p), C.POINTER(_i64p)]),
        "sbc_free": (None, [_vp]),
        "sbc_graph_create_dimacs": (C.c_int, [C.POINTER(_vp), C.c_char_p, _i64p, _i64p]),
        "sbc_server_read": (C.c_int, [_vp, C.c_int, _i32p, _i64p, _f64p]),
        "sbc_server_get_stats": (C.c_int, [_vp, C.POINTER(ServerStats), C.c_int]),
        "sbc_group_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.POINTER(_vp), C.c_int]),
        "sbc_group_destroy": (C.c_int, [_vp]),
        "sbc_group_info": (C.c_int, [_vp, C.POINTER(C.c_int), _i64p, _i64p, C.POINTER(C.c_int)]),
        "sbc_group_set_variant": (C.c_int, [_vp, C.c_int]),
        "sbc_group_insert_batch": (C.c_int, [_vp, _i64p, _i64p, _i64p, _f64p]),
        "sbc_group_autotune": (C.c_int, [_vp, _i64p, _i64p, _i64p, C.c_int, C.POINTER(C.c_int), _f64p, C.c_int]),
        "sbc_group_read_counters": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p, _i64p]),
        "sbc_update_inserted": (C.c_int, [_vp, C.c_int64, _i64p, _i64p, C.POINTER(BatchStats)]),
        "sbc_sync": (C.c_int, [_vp]),
        "sbc_read_counters": (C.c_int, [_vp, _i64p, _i64p, _i64p, _i64p, _i64p]),
        "sbc_get_bc": (C.c_int, [_vp, _f64p]),
        "sbc_get_dist": (C.c_int, [_vp, C.c_int64, C.c_int64, _i32p]),
        "sbc_get_sigma": (C.c_int, [_vp, C.c_int64, C.c_int64, _i64p]),
        "sbc_get_delta": (C.c_int, [_vp, C.c_int64, C.c_int64, _f64p]),
        "sbc_set_profiling": (C.c_int, [_vp, C.c_int]),
        "sbc_get_profile": (C.c_int, [_vp, C.POINTER(Profile)]),
        "sbc_reset_profile": (C.c_int, [_vp]),
        "sbc_timer_start": (C.c_int, [_vp]),
        "sbc_timer_stop": (C.c_int, [_vp, _f64p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int):
    if rc != 0:
        msg = _lib.sbc_last_error().decode() if _lib else ""
        raise SbcError(f"sbc error {rc}: {msg}")


def _a64(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.int64)


def p64(a: np.ndarray):
    return a.ctypes.data_as(_i64p)


class DeviceGraph:
    """sbc_graph: the device slack-CSR adjacency."""

    def __init__(self, nv: int, off, adj):
        self.lib = load()
        self._off = _a64(off)
        self._adj = _a64(adj)
        h = _vp()
        _check(self.lib.sbc_graph_create(C.byref(h), int(nv), p64(self._off), p64(self._adj)))
        self.h = h
        self.nv = int(nv)
        self._forests = weakref.WeakSet()

    @classmethod
    def from_dimacs(cls, path: str) -> "DeviceGraph":
        """A device graph from a DIMACS .graph file (parsed by all host
        threads, adjacency built on the device)."""
        lib = load()
        h = _vp()
        nv = C.c_int64(0)
        _check(lib.sbc_graph_create_dimacs(C.byref(h), os.fsencode(path), C.byref(nv), None))
        return cls._adopt(h, nv.value)

    @classmethod
    def _adopt(cls, h, nv: int) -> "DeviceGraph":
        self = cls.__new__(cls)
        self.lib = load()
        self.h = h
        self.nv = int(nv)
        self._forests = weakref.WeakSet()
        return self

    def remove_directed(self, u: int, v: int) -> int:
        """Remove u -> v: 1 removed, 0 absent, -1 invalid."""
        r = C.c_int(0)
        _check(self.lib.sbc_graph_remove_directed(self.h, int(u), int(v), C.byref(r)))
        return r.value

    def degree(self, v: int) -> int:
        d = C.c_int64()
        _check(self.lib.sbc_graph_degree(self.h, int(v), C.byref(d)))
        return d.value

    def insert_directed(self, a: int, b: int) -> int:
        r = C.c_int()
        _check(self.lib.sbc_graph_insert_directed(self.h, int(a), int(b), C.byref(r)))
        return r.value

    def reserve(self, pairs):
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        _check(self.lib.sbc_graph_reserve(self.h, u.size, p64(u), p64(v)))

    def repacks(self) -> int:
        c = C.c_int64()
        _check(self.lib.sbc_graph_repacks(self.h, C.byref(c)))
        return c.value

    def to_csr(self):
        off = np.zeros(self.nv + 1, dtype=np.int64)
        _check(self.lib.sbc_graph_to_csr(self.h, p64(off), None))
        adj = np.zeros(int(off[-1]), dtype=np.int64)
        _check(self.lib.sbc_graph_to_csr(self.h, p64(off), p64(adj)))
        return off, adj

    def close(self):
        for f in list(getattr(self, "_forests", ())):
            f.close()  # forests first: they use the graph's stream
        if getattr(self, "h", None):
            self.lib.sbc_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_dimacs(path: str):
    """Parse a DIMACS .graph file with the library's threaded parser (the
    reference's ParseDimacsGraph reading: vertex 0 isolated, line u = vertex
    u).  Returns (nv, off int64[nv+1], adj int64[ne]).  Needs no GPU."""
    lib = load()
    nv, ne = C.c_int64(0), C.c_int64(0)
    po, pa = _i64p(), _i64p()
    _check(lib.sbc_dimacs_read(os.fsencode(path), C.byref(nv), C.byref(ne), C.byref(po), C.byref(pa)))
    try:
        off = np.ctypeslib.as_array(po, shape=(nv.value + 1,)).copy()
        adj = np.ctypeslib.as_array(pa, shape=(max(ne.value, 1),))[:ne.value].copy()
    finally:
        lib.sbc_free(C.cast(po, _vp))
        lib.sbc_free(C.cast(pa, _vp))
    return nv.value, off, adj


class Checkpoint:
    """sbc_checkpoint: a forest's graph and per-root state in host memory."""

    def __init__(self, h):
        self.lib = load()
        self.h = h

    @classmethod
    def take(cls, forest: "DeviceForest") -> "Checkpoint":
        h = _vp()
        _check(load().sbc_checkpoint_take(forest.h, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str) -> "Checkpoint":
        h = _vp()
        _check(load().sbc_checkpoint_load(os.fsencode(path), C.byref(h)))
        return cls(h)

    def save(self, path: str):
        _check(self.lib.sbc_checkpoint_save(self.h, os.fsencode(path)))

    def info(self) -> dict:
        v = [C.c_int64() for _ in range(4)]
        _check(self.lib.sbc_checkpoint_info(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("nv", "nk", "ne", "bytes"), [x.value for x in v]))

    def read(self):
        """(dist [nk][nv] int32, sigma [nk][nv] int64, bc [nv] float64) as saved."""
        i = self.info()
        dist = np.zeros((i["nk"], i["nv"]), dtype=np.int32)
        sigma = np.zeros((i["nk"], i["nv"]), dtype=np.int64)
        bc = np.zeros(i["nv"], dtype=np.float64)
        _check(self.lib.sbc_checkpoint_read(self.h, dist.ctypes.data_as(_i32p), p64(sigma),
                                            bc.ctypes.data_as(_f64p)))
        return dist, sigma, bc

    def restore(self, variant: int = -1):
        """A new (DeviceGraph, DeviceForest) in the saved state, no static init."""
        g, f = _vp(), _vp()
        _check(self.lib.sbc_checkpoint_restore(self.h, int(variant), C.byref(g), C.byref(f)))
        dg = DeviceGraph._adopt(g, self.info()["nv"])
        nk = self.info()["nk"]
        roots = np.zeros(nk, dtype=np.int64)
        _check(self.lib.sbc_forest_roots(f, p64(roots)))
        return dg, DeviceForest._adopt(f, dg, roots)

    def close(self):
        if getattr(self, "h", None):
            self.lib.sbc_checkpoint_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceForest:
    """sbc_forest: per-root dist/sigma/delta and BC on the device."""

    @classmethod
    def _adopt(cls, h, graph: "DeviceGraph", roots) -> "DeviceForest":
        self = cls.__new__(cls)
        self.lib = load()
        self.graph = graph
        self.roots = _a64(roots)
        self.h = h
        self.nv = graph.nv
        self.nk = int(self.roots.size)
        graph._forests.add(self)
        self._groups = weakref.WeakSet()
        return self

    def __init__(self, graph: DeviceGraph, roots, workers: int = 0, variant: int = -1):
        self.lib = load()
        self.graph = graph
        self.roots = _a64(roots)
        h = _vp()
        _check(self.lib.sbc_forest_create_ex(C.byref(h), graph.h, self.roots.size, p64(self.roots), int(workers),
                                             int(variant)))
        self.h = h
        self.nv = graph.nv
        self.nk = int(self.roots.size)
        graph._forests.add(self)
        self._groups = weakref.WeakSet()

    def info(self) -> dict:
        v = [C.c_int64() for _ in range(4)]
        _check(self.lib.sbc_forest_info(self.h, *[C.byref(x) for x in v]))
        return {"nv": v[0].value, "nk": v[1].value, "workers": v[2].value, "bytes": v[3].value}

    def static_init(self, sync: bool = True):
        _check(self.lib.sbc_static_init(self.h))
        if sync:
            self.sync()

    def insert(self, pairs) -> dict:
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        st = BatchStats()
        _check(self.lib.sbc_insert_batch(self.h, u.size, p64(u), p64(v), C.byref(st)))
        return st.as_dict()

    def delete(self, pairs) -> dict:
        """Remove each edge (both directions) and update every root, one
        deletion at a time; stats: inserted = removed, duplicates = absent."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        st = BatchStats()
        _check(self.lib.sbc_delete_batch(self.h, u.size, p64(u), p64(v), C.byref(st)))
        return st.as_dict()

    DELETE_AUTO, DELETE_MOVE_DOWN, DELETE_RECOMPUTE = 0, 1, 2

    def set_delete_mode(self, mode: int) -> None:
        """How roots whose deeper endpoint loses its last parent are updated:
        moved down in place, recomputed after the call, or by graph size."""
        _check(self.lib.sbc_forest_set_delete_mode(self.h, int(mode)))

    def update_deleted(self, u: int, v: int) -> dict:
        """The update for a deletion whose edge was already removed from the graph."""
        st = BatchStats()
        _check(self.lib.sbc_update_deleted(self.h, int(u), int(v), C.byref(st)))
        return st.as_dict()

    def insert_async(self, pairs):
        """Queue a batch from host pairs without waiting (sync() waits)."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        _check(self.lib.sbc_insert_batch_async(self.h, u.size, p64(u), p64(v)))

    def insert_device(self, n: int, d_u: int, d_v: int):
        """Asynchronous batch from int32 device pointers (e.g. tensor.data_ptr())."""
        _check(self.lib.sbc_insert_batch_device(self.h, int(n), _vp(d_u), _vp(d_v)))

    def set_graph_capture(self, on: bool):
        _check(self.lib.sbc_set_graph_capture(self.h, 1 if on else 0))

    # ---- cost model ----
    SCHED_STATIC, SCHED_MODEL = 0, 1

    def cost_log_start(self, capacity: int):
        _check(self.lib.sbc_cost_log_start(self.h, int(capacity)))

    def cost_log_stop(self) -> int:
        n = C.c_int64(0)
        _check(self.lib.sbc_cost_log_stop(self.h, C.byref(n)))
        return n.value

    def cost_log_read(self, first: int, count: int):
        x = np.zeros((count, 8), dtype=np.float32)
        y = np.zeros(count, dtype=np.float32)
        _check(self.lib.sbc_cost_log_read(self.h, int(first), int(count), x.ctypes.data_as(_f32p),
                                          y.ctypes.data_as(_f32p)))
        return x, y

    def train_cost_model(self, epochs=8, batch=4096, lr=2e-3, val_frac=0.1, seed=1) -> dict:
        st = ModelStats()
        _check(self.lib.sbc_cost_model_train(self.h, int(epochs), int(batch), float(lr), float(val_frac), int(seed),
                                             C.byref(st)))
        return {k: getattr(st, k) for k, _ in ModelStats._fields_}

    def set_schedule(self, schedule: int):
        _check(self.lib.sbc_set_schedule(self.h, int(schedule)))

    def compare_schedules(self, pairs, reps: int = 1):
        """Insert `pairs` after timing its update under the static and the
        model schedule on copies of the state; returns (ms_static, ms_model)."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        a, b = C.c_double(0), C.c_double(0)
        _check(self.lib.sbc_forest_compare_schedules(self.h, len(u), p64(u), p64(v), int(reps), C.byref(a),
                                                     C.byref(b)))
        return a.value, b.value

    def model_params(self, new=None) -> np.ndarray:
        n = C.c_int(0)
        _check(self.lib.sbc_cost_model_size(C.byref(n), None))
        out = np.zeros(n.value, dtype=np.float32)
        src = None
        if new is not None:
            src = np.ascontiguousarray(new, dtype=np.float32)
            assert src.size == n.value
        _check(self.lib.sbc_cost_model_params(self.h, out.ctypes.data_as(_f32p),
                                              src.ctypes.data_as(_f32p) if src is not None else None))
        return out

    def model_predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 8)
        out = np.zeros(len(x), dtype=np.float32)
        _check(self.lib.sbc_cost_model_predict(self.h, len(x), x.ctypes.data_as(_f32p), out.ctypes.data_as(_f32p)))
        return out

    def model_grad(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 8)
        y = np.ascontiguousarray(y, dtype=np.float32)
        n = C.c_int(0)
        _check(self.lib.sbc_cost_model_size(C.byref(n), None))
        g = np.zeros(n.value - 16, dtype=np.float32)
        pred = np.zeros(len(x), dtype=np.float32)
        _check(self.lib.sbc_cost_model_grad(self.h, len(x), x.ctypes.data_as(_f32p), y.ctypes.data_as(_f32p),
                                            g.ctypes.data_as(_f32p), pred.ctypes.data_as(_f32p)))
        return g, pred

    def roster(self, r: int, level: int):
        """Members listed for level `level` of root row r, or None if untracked."""
        out = np.zeros(256, dtype=np.int32)
        n = C.c_int(0)
        _check(self.lib.sbc_get_roster(self.h, int(r), int(level), out.ctypes.data_as(_i32p), C.byref(n)))
        return None if n.value < 0 else out[:n.value].copy()

    def level_hist(self) -> np.ndarray:
        out = np.zeros((self.nk, 64), dtype=np.int32)
        _check(self.lib.sbc_get_level_hist(self.h, 0, self.nk, out.ctypes.data_as(_i32p)))
        return out

    @property
    def variant(self) -> int:
        v = C.c_int(0)
        _check(self.lib.sbc_forest_variant(self.h, C.byref(v)))
        return v.value

    def set_variant(self, variant: int):
        """Re-size the worker scratch for update launch shape `variant`."""
        _check(self.lib.sbc_forest_set_variant(self.h, int(variant)))

    def autotune(self, pairs, reps: int = 2):
        """Insert the batch `pairs` after timing its update under every launch
        shape that fits (on copies of the state); the fastest shape is kept.
        Returns (chosen shape, per-shape ms with -1 for skipped shapes)."""
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        n = C.c_int(0)
        _check(self.lib.sbc_update_variant_count(C.byref(n)))
        ms = np.full(n.value, -1.0)
        chosen = C.c_int(-1)
        _check(self.lib.sbc_forest_autotune(self.h, len(u), p64(u), p64(v), int(reps), C.byref(chosen),
                                            ms.ctypes.data_as(_f64p),
                                            n.value))
        return chosen.value, ms

    def update_inserted(self, pairs) -> dict:
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        st = BatchStats()
        _check(self.lib.sbc_update_inserted(self.h, u.size, p64(u), p64(v), C.byref(st)))
        return st.as_dict()

    def sync(self):
        _check(self.lib.sbc_sync(self.h))

    def counters(self) -> dict:
        v = [C.c_int64() for _ in range(5)]
        _check(self.lib.sbc_read_counters(self.h, *[C.byref(x) for x in v]))
        return {"vertices": v[0].value, "edges": v[1].value, "case1": v[2].value, "case2": v[3].value,
                "scanned": v[4].value}

    def bc(self) -> np.ndarray:
        out = np.zeros(self.nv, dtype=np.float64)
        _check(self.lib.sbc_get_bc(self.h, out.ctypes.data_as(_f64p)))
        return out

    def dist(self, r0: int = 0, nr: int | None = None) -> np.ndarray:
        nr = self.nk - r0 if nr is None else nr
        out = np.zeros((nr, self.nv), dtype=np.int32)
        _check(self.lib.sbc_get_dist(self.h, r0, nr, out.ctypes.data_as(_i32p)))
        return out

    def sigma(self, r0: int = 0, nr: int | None = None) -> np.ndarray:
        nr = self.nk - r0 if nr is None else nr
        out = np.zeros((nr, self.nv), dtype=np.int64)
        _check(self.lib.sbc_get_sigma(self.h, r0, nr, p64(out)))
        return out

    def delta(self, r0: int = 0, nr: int | None = None) -> np.ndarray:
        nr = self.nk - r0 if nr is None else nr
        out = np.zeros((nr, self.nv), dtype=np.float64)
        _check(self.lib.sbc_get_delta(self.h, r0, nr, out.ctypes.data_as(_f64p)))
        return out

    def level64(self, r0: int = 0, nr: int | None = None) -> np.ndarray:
        """dist widened to the reference convention (INT64_MAX = unreachable)."""
        d = self.dist(r0, nr).astype(np.int64)
        d[d == np.iinfo(np.int32).max] = np.iinfo(np.int64).max
        return d

    def set_profiling(self, on: bool):
        _check(self.lib.sbc_set_profiling(self.h, 1 if on else 0))

    def profile(self) -> dict:
        p = Profile()
        _check(self.lib.sbc_get_profile(self.h, C.byref(p)))
        return p.as_dict()

    def reset_profile(self):
        _check(self.lib.sbc_reset_profile(self.h))

    def timer_start(self):
        _check(self.lib.sbc_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_double()
        _check(self.lib.sbc_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def close(self):
        for grp in list(getattr(self, "_groups", ())):
            grp.close()  # a live group holds this forest
        if getattr(self, "h", None):
            self.lib.sbc_forest_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceGroup:
    """sbc_group: up to 64 forests over different graphs, updated by one
    append, one classify and one persistent update launch per batch."""

    def __init__(self, forests, variant: int = -1):
        self.lib = load()
        self.forests = list(forests)
        arr = (_vp * len(self.forests))(*[f.h for f in self.forests])
        h = _vp()
        _check(self.lib.sbc_group_create(C.byref(h), len(self.forests), arr, int(variant)))
        self.h = h
        for f in self.forests:
            f._groups.add(self)

    @staticmethod
    def _flatten(batches):
        parts = [np.asarray(b, dtype=np.int64).reshape(-1, 2) for b in batches]
        counts = np.array([len(p) for p in parts], dtype=np.int64)
        cat = np.concatenate(parts) if len(parts) else np.zeros((0, 2), np.int64)
        return counts, np.ascontiguousarray(cat[:, 0]), np.ascontiguousarray(cat[:, 1])

    def insert(self, batches) -> float:
        """Apply batches[i] (pairs) to forests[i], all in one launch sequence;
        returns the device time of that sequence in ms."""
        counts, u, v = self._flatten(batches)
        if len(counts) != len(self.forests):
            raise ValueError("one batch per member forest")
        ms = C.c_double(0.0)
        _check(self.lib.sbc_group_insert_batch(self.h, p64(counts), p64(u), p64(v), C.byref(ms)))
        return ms.value

    def autotune(self, batches, reps: int = 2):
        counts, u, v = self._flatten(batches)
        if len(counts) != len(self.forests):
            raise ValueError("one batch per member forest")
        n = C.c_int(0)
        _check(self.lib.sbc_update_variant_count(C.byref(n)))
        ms = np.full(n.value, -1.0)
        chosen = C.c_int(-1)
        _check(self.lib.sbc_group_autotune(self.h, p64(counts), p64(u), p64(v), int(reps), C.byref(chosen),
                                           ms.ctypes.data_as(_f64p), n.value))
        return chosen.value, ms

    def bc(self) -> list:
        """Every member's BC vector (one wait for all of them)."""
        sizes = [f.nv for f in self.forests]
        out = np.zeros(int(sum(sizes)), dtype=np.float64)
        _check(self.lib.sbc_group_get_bc(self.h, out.ctypes.data_as(_f64p)))
        return np.split(out, np.cumsum(sizes)[:-1])

    def set_variant(self, variant: int):
        _check(self.lib.sbc_group_set_variant(self.h, int(variant)))

    def info(self) -> dict:
        n, var = C.c_int(0), C.c_int(0)
        w, b = C.c_int64(0), C.c_int64(0)
        _check(self.lib.sbc_group_info(self.h, C.byref(n), C.byref(w), C.byref(b), C.byref(var)))
        return {"forests": n.value, "workers": w.value, "bytes": b.value, "variant": var.value}

    def counters(self) -> dict:
        v = [C.c_int64() for _ in range(5)]
        _check(self.lib.sbc_group_read_counters(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("vertices", "edges", "case1", "case2", "scanned"), [x.value for x in v]))

    def close(self):
        if getattr(self, "h", None):
            self.lib.sbc_group_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceServer:
    """sbc_server: graphs resident on one device, insertion requests batched
    per graph as they arrive (admission by HBM footprint)."""

    def __init__(self, budget_bytes: int, max_batch: int = 256, device: int = 0, max_inflight: int = 0,
                 autotune: bool = False, train_insertions: int = 0):
        self.lib = load()
        h = _vp()
        _check(self.lib.sbc_server_create(C.byref(h), int(device), int(budget_bytes), int(max_batch)))
        self.h = h
        self._shape = {}
        if max_inflight:
            self._rc(self.lib.sbc_server_set_max_inflight(self.h, int(max_inflight)))
        if autotune or train_insertions:
            self._rc(self.lib.sbc_server_set_tuning(self.h, 1 if autotune else 0, int(train_insertions)))

    def _rc(self, rc: int):
        if rc != 0:
            msg = self.lib.sbc_server_error(self.h).decode() or (_lib.sbc_last_error().decode() if _lib else "")
            raise SbcError(f"sbc server error {rc}: {msg}")

    def add_graph(self, g, roots, variant: int = -1) -> int:
        off, adj, roots = _a64(g.off), _a64(g.adj), _a64(roots)
        gid = C.c_int(-1)
        self._rc(self.lib.sbc_server_add_graph(self.h, int(g.nv), p64(off), p64(adj), roots.size, p64(roots),
                                               int(variant), C.byref(gid)))
        self._shape[gid.value] = (int(g.nv), int(roots.size))
        return gid.value

    def graph_info(self, gid: int) -> dict:
        st = C.c_int(0)
        fp, done, nb = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        self._rc(self.lib.sbc_server_graph_info(self.h, int(gid), C.byref(st), C.byref(fp), C.byref(done),
                                                C.byref(nb)))
        return {"state": ("waiting", "admitted", "released", "evicted")[st.value], "footprint": fp.value,
                "completed": done.value, "batches": nb.value}

    def submit(self, gid: int, u: int, v: int):
        self._rc(self.lib.sbc_server_submit(self.h, int(gid), int(u), int(v)))

    def play(self, gids, pairs, t_offsets):
        """Submit request i at t_offsets[i] seconds after the call (native
        timing loop); returns when all are submitted."""
        gids = np.ascontiguousarray(gids, dtype=np.int32)
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        u = np.ascontiguousarray(pairs[:, 0])
        v = np.ascontiguousarray(pairs[:, 1])
        t = np.ascontiguousarray(t_offsets, dtype=np.float64)
        self._rc(self.lib.sbc_server_play(self.h, len(gids), gids.ctypes.data_as(_i32p), p64(u), p64(v),
                                          t.ctypes.data_as(_f64p)))

    def drain(self):
        self._rc(self.lib.sbc_server_drain(self.h))

    def release(self, gid: int):
        self._rc(self.lib.sbc_server_release(self.h, int(gid)))

    def evict(self, gid: int):
        """Checkpoint graph gid into host memory and free its device memory
        once no batch of it is on the device; it is restored when it fits."""
        self._rc(self.lib.sbc_server_evict(self.h, int(gid)))

    def read(self, gid: int):
        nv, nk = self._shape[gid]
        dist = np.zeros((nk, nv), dtype=np.int32)
        sigma = np.zeros((nk, nv), dtype=np.int64)
        bc = np.zeros(nv, dtype=np.float64)
        self._rc(self.lib.sbc_server_read(self.h, int(gid), dist.ctypes.data_as(_i32p), sigma.ctypes.data_as(_i64p),
                                          bc.ctypes.data_as(_f64p)))
        return dist, sigma, bc

    def stats(self, reset: bool = False) -> dict:
        st = ServerStats()
        self._rc(self.lib.sbc_server_get_stats(self.h, C.byref(st), 1 if reset else 0))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.sbc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

