"""The static init entry point that allocates nothing (sbc_static_init_noalloc).

Some callers cannot allocate device memory themselves or let a library do it:
code that runs inside another runtime which owns the device's memory pool, or
a process whose device memory is reserved up front.  For them the library has
one entry point whose scratch is a fixed array compiled into the library; the
caller passes the graph and the output arrays in its own device memory.

This file is collected last so that, if it fails, a run that stops at the
first failure has already run every other test.  It calls the entry point
through the C-ABI twice in a row, on two different graphs (so stale contents of
the shared array from the first call would show in the second), and checks each
result against the ordinary entry point (sbc_static_init on an sbc_forest):
dist and sigma bit-exact, delta and BC within the 1e-9 relative tolerance of
the other parity tests.  Sizes above the stated maximum must be rejected.
"""
import ctypes as C

import numpy as np
import pytest

from _util import INF32, assert_bc, bc_err
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu

MAX_VERTICES = 262144  # SBC_NOALLOC_MAX_VERTICES in include/sbc_gb300.h


def _entry(lib):
    fn = lib.sbc_static_init_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p]
    lib.sbc_noalloc_last_error.restype = C.c_char_p
    return fn


def _run_noalloc(lib, g, roots, stream=None, adj=None):
    """Outputs of one call (rc 0 asserted); `stream` a torch.cuda.Stream or None."""
    rc, out = _call_noalloc(lib, g, roots, stream=stream, adj=adj)
    assert rc == 0, lib.sbc_noalloc_last_error().decode()
    return out


def _call_noalloc(lib, g, roots, stream=None, adj=None):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda")
    k, n = len(roots), g.nv
    off = torch.tensor(g.off, dtype=torch.int64, device=dev)
    col = torch.tensor(g.adj if adj is None else adj, dtype=torch.int32, device=dev)
    rt = torch.tensor(roots, dtype=torch.int64, device=dev)
    # outputs start as garbage: every entry must be written by the call
    dist = torch.full((k, n), -7, dtype=torch.int32, device=dev)
    sigma = torch.full((k, n), -7, dtype=torch.int64, device=dev)
    delta = torch.full((k, n), float("nan"), dtype=torch.float64, device=dev)
    bc = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    handle = None if stream is None else stream.cuda_stream
    rc = _entry(lib)(n, off.data_ptr(), col.data_ptr(), k, rt.data_ptr(), dist.data_ptr(), sigma.data_ptr(),
                     delta.data_ptr(), bc.data_ptr(), handle)
    torch.cuda.synchronize()
    return rc, (dist.cpu().numpy(), sigma.cpu().numpy(), delta.cpu().numpy(), bc.cpu().numpy())


def _run_existing(g, roots):
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    out = f.dist(), f.sigma(), f.delta(), f.bc()
    f.close()
    dg.close()
    return out


def _check(got, want):
    d, s, dl, bc = got
    d0, s0, dl0, bc0 = want
    assert np.array_equal(d, d0), "dist differs from sbc_static_init"
    reach = d0 != INF32
    assert np.array_equal(s[reach], s0[reach]), "sigma differs from sbc_static_init"
    assert bc_err(dl, dl0) <= 1e-9, "delta differs from sbc_static_init"
    assert_bc(bc, bc0, "bc vs sbc_static_init")


def test_noalloc_static_init_matches_existing_entry_point_twice(sbc_lib):
    g1 = G.er(3000, 12000, seed=41)
    r1 = G.pick_roots(g1.nv, 48, seed=41)
    g2 = G.rmat(12, 8, seed=42)            # different size and shape, isolated vertices
    r2 = G.pick_roots(g2.nv, 100, seed=42)
    _check(_run_noalloc(sbc_lib, g1, r1), _run_existing(g1, r1))
    _check(_run_noalloc(sbc_lib, g2, r2), _run_existing(g2, r2))


def test_noalloc_rejects_sizes_beyond_its_maximum(sbc_lib):
    fn = _entry(sbc_lib)
    one = C.c_int64(0)
    p = C.cast(C.pointer(one), C.c_void_p)
    rc = fn(MAX_VERTICES + 1, p, p, 1, p, p, p, p, p, None)
    assert rc == -1
    assert b"SBC_NOALLOC_MAX_VERTICES" in sbc_lib.sbc_noalloc_last_error()
    rc = fn(100000, p, p, 100, p, p, p, p, p, None)  # 1e7 cells > SBC_NOALLOC_MAX_CELLS
    assert rc == -1
    assert b"SBC_NOALLOC_MAX_CELLS" in sbc_lib.sbc_noalloc_last_error()


def test_noalloc_on_a_caller_stream_with_fewer_roots_than_worker_slots(sbc_lib):
    """Work queued on a stream the caller created, and nk (3) below the
    array's worker slots, so fewer CTAs run than slots exist."""
    torch = pytest.importorskip("torch")
    g = G.er(500, 2000, seed=43)
    r = G.pick_roots(g.nv, 3, seed=43)
    st = torch.cuda.Stream()
    _check(_run_noalloc(sbc_lib, g, r, stream=st), _run_existing(g, r))
    _check(_run_noalloc(sbc_lib, g, r, stream=st), _run_existing(g, r))


def test_noalloc_rejects_ids_outside_the_graph(sbc_lib):
    """A root or a neighbour id outside [0, nv) is caught on the device
    before the init runs: the call returns SBC_ERR_ARG and writes nothing,
    and the next valid call is unaffected."""
    g = G.er(400, 1600, seed=44)
    r = G.pick_roots(g.nv, 6, seed=44)
    bad_roots = np.array(r, dtype=np.int64)
    bad_roots[2] = g.nv + 5
    rc, (d, s, dl, bc) = _call_noalloc(sbc_lib, g, bad_roots)
    assert rc == -1
    assert b"root outside" in sbc_lib.sbc_noalloc_last_error()
    assert (d == -7).all() and (s == -7).all() and np.isnan(bc).all()
    bad_adj = np.array(g.adj, dtype=np.int32)
    bad_adj[len(bad_adj) // 2] = g.nv
    rc, (d, s, dl, bc) = _call_noalloc(sbc_lib, g, r, adj=bad_adj)
    assert rc == -1
    assert b"neighbour id outside" in sbc_lib.sbc_noalloc_last_error()
    assert (d == -7).all() and np.isnan(bc).all()
    _check(_run_noalloc(sbc_lib, g, r), _run_existing(g, r))
