"""DIMACS ingestion (host side, no GPU): the library's threaded parser reads
files the way the reference's ParseDimacsGraph does (src/sbcMain_utils.c:
382-422) -- header "NV NE", line u = vertex u's neighbours, ids as they
stand, vertex 0 isolated, a line's reading stops at its first non-integer
token -- checked against a plain line-by-line reading of the same rules, on
the golden graphs written back as DIMACS, on edge cases, and on a file large
enough to be split over all host threads."""
from __future__ import annotations

import numpy as np
import pytest

from _util import load_golden
from streamingbc_gb300 import native


def plain_read(text: str):
    """Line-by-line statement of the reading (the checker)."""
    lines = text.split("\n")
    head = lines[0].split()
    nv = int(head[0]) + 1
    body = lines[1:]
    if body and body[-1] == "":
        body = body[:-1]  # a final newline ends the last line; it is not a line
    off = [0, 0]
    adj = []
    for line in body:
        for tok in line.split():
            try:
                adj.append(int(tok))
            except ValueError:
                break
        off.append(len(adj))
    while len(off) < nv + 1:
        off.append(len(adj))
    return nv, np.array(off, dtype=np.int64), np.array(adj, dtype=np.int64)


def to_dimacs(nv0: int, off, adj, ne_header=None) -> str:
    """A 0-based CSR as DIMACS text (1-based ids, one line per vertex)."""
    rows = [" ".join(str(int(x) + 1) for x in adj[off[u]:off[u + 1]]) for u in range(nv0)]
    ne = ne_header if ne_header is not None else len(adj) // 2
    return f"{nv0} {ne} 0\n" + "\n".join(rows) + "\n"


def _parse(tmp_path, text, name="g.graph"):
    p = tmp_path / name
    p.write_text(text)
    return native.read_dimacs(str(p))


@pytest.mark.parametrize("case", ["karate", "dolphins", "er200sparse"])
def test_golden_graphs_round_trip(sbc_lib, tmp_path, case):
    z = load_golden(case)
    text = to_dimacs(int(z["nv"]), z["off"], z["adj"])
    nv, off, adj = _parse(tmp_path, text)
    pnv, poff, padj = plain_read(text)
    assert nv == pnv == int(z["nv"]) + 1
    np.testing.assert_array_equal(off, poff)
    np.testing.assert_array_equal(adj, padj)
    # vertex u + 1 holds golden vertex u's neighbours, shifted by one
    np.testing.assert_array_equal(off[1:], z["off"])
    np.testing.assert_array_equal(adj, z["adj"] + 1)


@pytest.mark.parametrize("text", [
    "3 2\n2\n1 3\n2\n",                 # plain
    "3 2\n2\n1 3\n2",                   # no final newline
    "3 2 0\r\n2\r\n1 3\r\n2\r\n",       # CRLF
    "5 2\n2\n1\n",                      # missing trailing lines: empty lists
    "3 2\n2 x 3\n1 3\n\n",              # a non-integer token ends the line's list
    "4 3\n\n  3   4 \n2\n2\n",          # blank line = isolated vertex; spacing
    "2 1\n2 % comment\n1\n",            # text after the list is ignored
])
def test_edge_cases_match_the_reading(sbc_lib, tmp_path, text):
    nv, off, adj = _parse(tmp_path, text)
    pnv, poff, padj = plain_read(text)
    assert nv == pnv
    np.testing.assert_array_equal(off, poff)
    np.testing.assert_array_equal(adj, padj)


@pytest.mark.parametrize("text", [
    "",                        # no header
    "x y\n1\n",                # no numeric header
    "2 1\n2\n1\n1\n",          # more lines than NV
    "2 1\n3\n1\n",             # id beyond NV
    "2 1\n-1\n1\n",            # negative id
])
def test_bad_files_are_refused(sbc_lib, tmp_path, text):
    with pytest.raises(native.SbcError):
        _parse(tmp_path, text)


def test_missing_file_is_refused(sbc_lib, tmp_path):
    with pytest.raises(native.SbcError):
        native.read_dimacs(str(tmp_path / "missing.graph"))


def test_large_file_split_over_threads(sbc_lib, tmp_path):
    """A ~6 MB file (parsed in parts by all host threads) equals the plain reading."""
    rng = np.random.default_rng(7)
    n = 60000
    deg = rng.integers(0, 30, size=n)
    rows = [" ".join(str(x) for x in rng.integers(1, n + 1, size=d)) for d in deg]
    text = f"{n} {int(deg.sum()) // 2}\n" + "\n".join(rows) + "\n"
    assert len(text) > (1 << 20)
    nv, off, adj = _parse(tmp_path, text)
    pnv, poff, padj = plain_read(text)
    assert nv == pnv
    np.testing.assert_array_equal(off, poff)
    np.testing.assert_array_equal(adj, padj)
