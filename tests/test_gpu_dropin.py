"""The drop-in boundary used the way the reference's callers use it: a plain C
program (tests/c/drop_in_driver.c) compiled with gcc against
include/streamingbc.h, linked to libsbc_gb300.so, driving the GPU through the
reference's own entry points.  Its BC after every insertion and its final
levels/sigmas are compared with the golden vectors of the unmodified
reference."""
import os
import subprocess

import numpy as np
import pytest

from _util import BC_RTOL, assert_levels, assert_sigma, bc_err, load_golden
from streamingbc_gb300 import native

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory, sbc_lib):
    d = tmp_path_factory.mktemp("dropin")
    exe = d / "drop_in_driver"
    libdir = os.path.dirname(native.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "c", "drop_in_driver.c"), "-o", str(exe), "-L", libdir,
                        "-lsbc_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_compiles(driver):
    assert os.path.exists(driver)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["karate", "er200sparse", "rmat9"])
def test_reference_style_c_caller_matches_reference(driver, tmp_path, case, port_lib):
    z = load_golden(case)
    nv = int(z["nv"])
    # deletions after the insertions: three original edges
    src = np.repeat(np.arange(nv), np.diff(z["off"]))
    orig = [(int(a), int(b)) for a, b in zip(src, z["adj"]) if a < b]
    dels = [orig[i] for i in (0, len(orig) // 2, len(orig) - 1)]
    inp = tmp_path / "in.txt"
    with open(inp, "w") as fh:
        fh.write(f"{nv} {z['adj'].size} {z['roots'].size} {len(z['ins'])}\n")
        fh.write(" ".join(map(str, z["off"].tolist())) + "\n")
        fh.write(" ".join(map(str, z["adj"].tolist())) + "\n")
        fh.write(" ".join(map(str, z["roots"].tolist())) + "\n")
        for u, v in z["ins"].tolist():
            fh.write(f"{u} {v}\n")
        fh.write(f"{len(dels)}\n")
        for u, v in dels:
            fh.write(f"{u} {v}\n")
        fh.write("1\n")  # then delete vertex 1 with all its edges
        # then re-insert vertex 1 with every other former neighbour, a vertex
        # it never had as a neighbour, a repeated entry and a self-loop (the
        # last two are skipped)
        src0 = list(dict.fromkeys([int(y) for y in z["adj"][z["off"][1]:z["off"][2]]]))
        back = src0[::2]
        far = next(y for y in range(nv - 1, -1, -1) if y != 1 and y not in src0)
        vins = back + [far, back[0], 1]
        fh.write(f"1 {len(vins)} " + " ".join(map(str, vins)) + "\n")
    outp = tmp_path / "out.txt"
    r = subprocess.run([str(driver), str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    bc, lv, sg = {}, {}, {}
    deg0 = vdeg = ivdeg = None
    for line in open(outp):
        p = line.split()
        if p[0] == "bc":
            bc[int(p[1])] = np.array(p[2:], dtype=np.float64)
        elif p[0] == "lv":
            lv[int(p[1])] = np.array(p[2:], dtype=np.int64)
        elif p[0] == "sg":
            sg[int(p[1])] = np.array(p[2:], dtype=np.int64)
        elif p[0] == "degree0":
            deg0 = int(p[1])
        elif p[0] == "dbc":
            bc[("del", int(p[1]))] = np.array(p[2:], dtype=np.float64)
        elif p[0] == "vbc":
            bc["vertex"] = np.array(p[2:], dtype=np.float64)
        elif p[0] == "vdeg":
            vdeg = (int(p[1]), int(p[2]))
        elif p[0] == "ivbc":
            bc["ivertex"] = np.array(p[2:], dtype=np.float64)
        elif p[0] == "ivlv":
            lv[("iv", int(p[1]))] = np.array(p[2:], dtype=np.int64)
        elif p[0] == "ivsg":
            sg[("iv", int(p[1]))] = np.array(p[2:], dtype=np.int64)
        elif p[0] == "ivdeg":
            ivdeg = int(p[1])
    assert bc_err(bc[-1], z["bc0"]) <= BC_RTOL
    for i in range(len(z["ins"])):
        assert bc_err(bc[i], z["bc_trace"][i]) <= BC_RTOL, f"bc after insertion {i}"
    k = z["roots"].size
    assert_levels(np.stack([lv[r] for r in range(k)]), z["level1"])
    assert_sigma(np.stack([sg[r] for r in range(k)]), z["sigma1"], z["level1"])
    added = sum(1 for u, v in z["ins"].tolist() if 0 in (u, v))
    assert deg0 == int(z["off"][1] - z["off"][0]) + added
    # deletions: BC after each equals a recompute of the modified graph
    o = port_lib.PortOracle(nv, z["off"], z["adj"], z["roots"])
    o.static()
    for u, v in z["ins"].tolist():
        o.insert(int(u), int(v))
    for i, (u, v) in enumerate(dels):
        assert o.delete(u, v)
        assert bc_err(bc[("del", i)], o.bc()) <= BC_RTOL, f"bc after deletion {i}"
    # vertex 1: all its edges, then BC of the graph without them
    nb = [int(y) for y in z["adj"][z["off"][1]:z["off"][2]]]
    nb += [v if u == 1 else u for u, v in z["ins"].tolist() if 1 in (u, v)]
    nb = [y for y in dict.fromkeys(nb) if (min(1, y), max(1, y)) not in set(dels)]
    for y in nb:
        o.delete(1, y)
    assert vdeg == (len(nb), 0)
    assert bc_err(bc["vertex"], o.bc()) <= BC_RTOL
    # vertex 1 re-inserted: its new edges one at a time in the oracle
    new = list(dict.fromkeys(y for y in back + [far] if y != 1))
    for y in new:
        o.insert(1, y)
    assert ivdeg == len(new)
    assert bc_err(bc["ivertex"], o.bc()) <= BC_RTOL
    assert_levels(np.stack([lv[("iv", r)] for r in range(k)]), o.level())
    assert_sigma(np.stack([sg[("iv", r)] for r in range(k)]), o.sigma(), o.level())
    o.close()


@pytest.fixture(scope="module")
def dimacs_driver(tmp_path_factory, sbc_lib):
    d = tmp_path_factory.mktemp("dimacs")
    exe = d / "dimacs_driver"
    libdir = os.path.dirname(native.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "c", "dimacs_driver.c"), "-o", str(exe), "-L", libdir,
                        "-lsbc_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dimacs_driver_compiles(dimacs_driver):
    assert os.path.exists(dimacs_driver)


@pytest.mark.gpu
def test_reference_driver_flow_from_a_dimacs_file(dimacs_driver, tmp_path):
    """karate written as a DIMACS file and run through the reference driver's
    flow (ParseDimacsGraph, PickRoots with NK = NV: exact BC, static init,
    insertions): BC after static init and after every insertion equals the
    reference's golden vectors (the file's vertex u + 1 is golden vertex u;
    vertex 0, the unused slot, stays at 0)."""
    from test_ingest import to_dimacs
    z = load_golden("karate")
    n0 = int(z["nv"])
    graph = tmp_path / "karate.graph"
    graph.write_text(to_dimacs(n0, z["off"], z["adj"], ne_header=78))
    ins = z["ins"][:16]
    insf = tmp_path / "ins.txt"
    insf.write_text(f"{len(ins)}\n" + "".join(f"{u + 1} {v + 1}\n" for u, v in ins.tolist()))
    outp = tmp_path / "out.txt"
    r = subprocess.run([str(dimacs_driver), str(graph), "0", str(insf), str(outp)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    lines = outp.read_text().split("\n")
    assert lines[0] == f"nv {n0 + 1} ne 156"
    bc = {}
    for line in lines[1:]:
        if line.startswith("bc "):
            p = line.split()
            bc[int(p[1])] = np.array([float(x) for x in p[2:]])
    assert bc[-1][0] == 0.0
    assert bc_err(bc[-1][1:], z["bc0"]) <= BC_RTOL
    for i in range(len(ins)):
        assert bc[i][0] == 0.0
        assert bc_err(bc[i][1:], z["bc_trace"][i]) <= BC_RTOL, i
