"""Forest checkpoint files on the host (no GPU): a file written by hand in the
documented layout (40-byte header "SBCCKPT1", version 1, nv, nk, ne; then
off, adj (int32), roots, bc, dist, sigma, delta) loads, reports its sizes and
returns its state; truncated, foreign or inconsistent files are refused."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from streamingbc_gb300 import native


def _file(nv=5, nk=2, *, magic=b"SBCCKPT1", version=1, off=None, adj=None, roots=None, cut=0):
    rng = np.random.default_rng(3)
    off = np.array([0, 2, 4, 6, 8, 8], dtype=np.int64) if off is None else np.asarray(off, dtype=np.int64)
    adj = np.array([1, 2, 0, 3, 0, 3, 1, 2], dtype=np.int32) if adj is None else np.asarray(adj, dtype=np.int32)
    roots = np.array([0, 3], dtype=np.int64) if roots is None else np.asarray(roots, dtype=np.int64)
    bc = rng.random(nv)
    dist = rng.integers(0, 4, size=(nk, nv)).astype(np.int32)
    sigma = rng.integers(1, 9, size=(nk, nv)).astype(np.int64)
    delta = rng.random((nk, nv))
    head = magic + struct.pack("<IIqqq", version, 0, nv, nk, len(adj))
    raw = head + b"".join(a.tobytes() for a in (off, adj, roots, bc, dist, sigma, delta))
    return raw[:len(raw) - cut], (bc, dist, sigma)


def test_hand_written_file_loads(sbc_lib, tmp_path):
    raw, (bc, dist, sigma) = _file()
    assert len(raw) >= 40 and raw[:8] == b"SBCCKPT1"
    p = tmp_path / "f.sbc"
    p.write_bytes(raw)
    ck = native.Checkpoint.load(str(p))
    info = ck.info()
    assert (info["nv"], info["nk"], info["ne"]) == (5, 2, 8)
    assert info["bytes"] == 6 * 8 + 8 * 4 + 2 * 8 + 5 * 8 + 10 * 4 + 10 * 8 + 10 * 8
    d, s, b = ck.read()
    np.testing.assert_array_equal(d, dist)
    np.testing.assert_array_equal(s, sigma)
    np.testing.assert_array_equal(b, bc)
    ck.save(str(tmp_path / "g.sbc"))  # written back byte for byte
    assert (tmp_path / "g.sbc").read_bytes() == raw
    ck.close()


@pytest.mark.parametrize("kw", [
    {"magic": b"NOTACKPT"},
    {"version": 2},
    {"cut": 1},                                  # truncated
    {"off": [0, 2, 4, 6, 8, 9]},                 # off[nv] != ne
    {"off": [0, 3, 2, 6, 8, 8]},                 # offsets not monotone
    {"adj": [1, 2, 0, 3, 0, 3, 1, 7]},           # neighbour id out of range
    {"roots": [0, 5]},                           # root out of range
])
def test_bad_files_are_refused(sbc_lib, tmp_path, kw):
    raw, _ = _file(**kw)
    p = tmp_path / "bad.sbc"
    p.write_bytes(raw)
    with pytest.raises(native.SbcError):
        native.Checkpoint.load(str(p))
