"""ctypes front end of the parity oracle -- TEST INFRASTRUCTURE ONLY.

``PortOracle`` wraps liboracle.so, the C restatement of the reference's COARSE
CPU path (sbc_oracle.c).  ``RefOracle`` wraps oracle/_ref/libsbcref.so, the
unmodified reference sources driven by ref_harness.c; it only exists where the
reference tree was available to compile it.  Only tests, the smoke check and
the benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsbcref.so")

_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)


def reference_src() -> str:
    """Directory of the reference's C sources: $SBC_REFERENCE_SRC when set,
    else the Makefile's overridable REF default."""
    env = os.environ.get("SBC_REFERENCE_SRC")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


def reference_available() -> bool:
    src = reference_src()
    return bool(src) and os.path.isfile(os.path.join(src, "streamingbc.c"))


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference harness when ``ref``, from
    reference_src())."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={reference_src()}"], check=True)


def _p64(a: np.ndarray):
    return a.ctypes.data_as(_i64p)


_port = None


def _port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build()
        lib = C.CDLL(PORT_SO)
        lib.orc_graph_new.restype = C.c_void_p
        lib.orc_graph_new.argtypes = [C.c_int64, _i64p, _i64p]
        lib.orc_graph_free.argtypes = [C.c_void_p]
        lib.orc_graph_insert.restype = C.c_int
        lib.orc_graph_insert.argtypes = [C.c_void_p, C.c_int64, C.c_int64]
        lib.orc_graph_remove.restype = C.c_int
        lib.orc_graph_remove.argtypes = [C.c_void_p, C.c_int64, C.c_int64]
        lib.orc_graph_degree.restype = C.c_int64
        lib.orc_graph_degree.argtypes = [C.c_void_p, C.c_int64]
        lib.orc_forest_new.restype = C.c_void_p
        lib.orc_forest_new.argtypes = [C.c_int64, C.c_int64, _i64p, C.c_int64]
        lib.orc_forest_free.argtypes = [C.c_void_p]
        for name in ("orc_forest_level", "orc_forest_sigma"):
            getattr(lib, name).restype = _i64p
            getattr(lib, name).argtypes = [C.c_void_p]
        for name in ("orc_forest_delta", "orc_forest_bc"):
            getattr(lib, name).restype = _f64p
            getattr(lib, name).argtypes = [C.c_void_p]
        lib.orc_forest_counters.argtypes = [C.c_void_p, _i64p]
        lib.orc_static.argtypes = [C.c_void_p, C.c_void_p]
        lib.orc_insert.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
        lib.orc_classify.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(C.c_int8)]
        lib.orc_insert_timed.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, _f64p, _f64p]
        lib.orc_static_timed.restype = C.c_double
        lib.orc_static_timed.argtypes = [C.c_void_p, C.c_void_p]
        lib.orc_set_threads.argtypes = [C.c_void_p, C.c_int64]
        _port = lib
    return _port


INF = np.iinfo(np.int64).max


class PortOracle:
    """C restatement of the reference hot path over one graph and root set."""

    def __init__(self, nv, off, adj, roots, nthreads: int | None = None):
        self.lib = _port_lib()
        self.nv = int(nv)
        self.roots = np.ascontiguousarray(roots, dtype=np.int64)
        self.nk = self.roots.size
        off = np.ascontiguousarray(off, dtype=np.int64)
        adj = np.ascontiguousarray(adj, dtype=np.int64)
        nt = nthreads or os.cpu_count() or 1
        self.nt = nt
        self.g = self.lib.orc_graph_new(self.nv, _p64(off), _p64(adj))
        self.f = self.lib.orc_forest_new(self.nv, self.nk, _p64(self.roots), nt)
        if not self.g or not self.f:
            raise MemoryError("oracle allocation failed")

    def close(self):
        if self.f:
            self.lib.orc_forest_free(self.f)
            self.f = None
        if self.g:
            self.lib.orc_graph_free(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def static(self):
        self.lib.orc_static(self.f, self.g)

    def set_threads(self, n: int) -> None:
        """Threads of the following calls (1 .. nthreads): the reference's NT."""
        self.lib.orc_set_threads(self.f, int(n))

    def insert(self, u: int, v: int) -> None:
        """Insert (u,v) into the graph (both directions), then update every root."""
        self.lib.orc_graph_insert(self.g, int(u), int(v))
        self.lib.orc_graph_insert(self.g, int(v), int(u))
        self.lib.orc_insert(self.f, self.g, int(u), int(v))

    def delete(self, u: int, v: int) -> bool:
        """Remove (u,v) from the graph (both directions) and recompute every
        root from scratch: the state after a deletion, by definition.  (The
        reference's own deleteEdgeStreamingBC, src/streamingbc.c:258-416,
        disagrees with this recomputation -- see tests/test_oracle.py -- so
        deletions are checked against the recomputation.)  Returns whether
        the edge was present."""
        a = self.lib.orc_graph_remove(self.g, int(u), int(v))
        self.lib.orc_graph_remove(self.g, int(v), int(u))
        if a:
            self.lib.orc_static(self.f, self.g)
        return bool(a)

    def static_timed(self) -> float:
        return self.lib.orc_static_timed(self.f, self.g)

    def insert_timed(self, u: int, v: int) -> tuple[float, float]:
        """Like insert(); returns (seconds in the per-root updates, seconds in
        the BC reduce).  The graph insertion itself is not timed, as in
        updateEdgeNEW (src/sbcMain_utils.c:568-571)."""
        self.lib.orc_graph_insert(self.g, int(u), int(v))
        self.lib.orc_graph_insert(self.g, int(v), int(u))
        a = C.c_double()
        b = C.c_double()
        self.lib.orc_insert_timed(self.f, self.g, int(u), int(v), C.byref(a), C.byref(b))
        return a.value, b.value

    def classify(self, u: int, v: int) -> np.ndarray:
        out = np.zeros(self.nk, dtype=np.int8)
        self.lib.orc_classify(self.f, int(u), int(v), out.ctypes.data_as(C.POINTER(C.c_int8)))
        return out

    def counters(self) -> dict:
        c = np.zeros(4, dtype=np.int64)
        self.lib.orc_forest_counters(self.f, _p64(c))
        return {"vertices": int(c[0]), "edges": int(c[1]), "case1": int(c[2]), "case2": int(c[3])}

    def _view(self, fn, dtype, count):
        p = fn(self.f)
        return np.ctypeslib.as_array(p, shape=(count,)).view(dtype)

    def level(self) -> np.ndarray:
        return self._view(self.lib.orc_forest_level, np.int64, self.nk * self.nv).reshape(self.nk, self.nv).copy()

    def sigma(self) -> np.ndarray:
        return self._view(self.lib.orc_forest_sigma, np.int64, self.nk * self.nv).reshape(self.nk, self.nv).copy()

    def delta(self) -> np.ndarray:
        return self._view(self.lib.orc_forest_delta, np.float64, self.nk * self.nv).reshape(self.nk, self.nv).copy()

    def bc(self) -> np.ndarray:
        return self._view(self.lib.orc_forest_bc, np.float64, self.nv).copy()


_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_SO)
        lib.ref_init.restype = C.c_int
        lib.ref_init.argtypes = [C.c_int64, _i64p, _i64p, C.c_int64, _i64p, C.c_int64]
        lib.ref_static.restype = C.c_double
        lib.ref_insert.restype = C.c_double
        lib.ref_insert.argtypes = [C.c_int64, C.c_int64]
        lib.ref_delete.restype = C.c_double
        lib.ref_delete.argtypes = [C.c_int64, C.c_int64]
        lib.ref_counters.argtypes = [_i64p]
        lib.ref_dump.argtypes = [_i64p, _i64p, _f64p, _f64p]
        _ref = lib
    return _ref


class RefOracle:
    """The unmodified reference (COARSE + BALANCE) behind ref_harness.c.

    The reference keeps its graph in a process-global STINGER pool, so only one
    instance may exist at a time; ``close`` must be called before the next."""

    def __init__(self, nv, off, adj, roots, nthreads: int = 1):
        self.lib = _ref_lib()
        self.nv = int(nv)
        self.roots = np.ascontiguousarray(roots, dtype=np.int64)
        self.nk = self.roots.size
        off = np.ascontiguousarray(off, dtype=np.int64)
        adj = np.ascontiguousarray(adj, dtype=np.int64)
        self.lib.ref_init(self.nv, _p64(off), _p64(adj), self.nk, _p64(self.roots), int(nthreads))
        self.open = True

    def static(self) -> float:
        return self.lib.ref_static()

    def insert(self, u: int, v: int) -> float:
        return self.lib.ref_insert(int(u), int(v))

    def delete(self, u: int, v: int) -> float:
        """Remove (u,v) from the graph (both directions), then update every root."""
        return self.lib.ref_delete(int(u), int(v))

    def counters(self) -> dict:
        c = np.zeros(4, dtype=np.int64)
        self.lib.ref_counters(_p64(c))
        return {"vertices": int(c[0]), "edges": int(c[1]), "case1": int(c[2]), "case2": int(c[3])}

    def dump(self):
        lv = np.zeros(self.nk * self.nv, dtype=np.int64)
        sg = np.zeros(self.nk * self.nv, dtype=np.int64)
        dl = np.zeros(self.nk * self.nv, dtype=np.float64)
        bc = np.zeros(self.nv, dtype=np.float64)
        self.lib.ref_dump(_p64(lv), _p64(sg), dl.ctypes.data_as(_f64p), bc.ctypes.data_as(_f64p))
        shape = (self.nk, self.nv)
        return lv.reshape(shape), sg.reshape(shape), dl.reshape(shape), bc

    def close(self):
        if self.open:
            self.lib.ref_free()
            self.open = False


def compare(lv_a, sg_a, bc_a, lv_b, sg_b, bc_b, rtol=1e-9):
    """Parity rule: levels equal everywhere (INF included), sigma equal on
    reachable vertices, |bc_a-bc_b| <= rtol*max(|bc_b|,1).  Returns a dict of
    mismatch counts and the worst BC error."""
    lv_a = np.asarray(lv_a)
    lv_b = np.asarray(lv_b)
    reach = lv_b != INF
    bad_lv = int(np.count_nonzero(lv_a != lv_b))
    bad_sg = int(np.count_nonzero((np.asarray(sg_a) != np.asarray(sg_b)) & reach))
    err = np.abs(np.asarray(bc_a) - np.asarray(bc_b)) / np.maximum(np.abs(bc_b), 1.0)
    return {"level": bad_lv, "sigma": bad_sg, "bc": int(np.count_nonzero(err > rtol)),
            "bc_maxerr": float(err.max()) if err.size else 0.0}
