"""CPU tests of the drop-in boundary: the C-ABI library builds for sm_103a,
loads, and exports every function that include/*.h declares.  No compute call
is made (there may be no GPU)."""
import ctypes
import os
import subprocess

from streamingbc_gb300 import native


def test_every_declared_symbol_is_exported(sbc_lib):
    names = native.header_functions()
    assert len(names) >= 50
    for n in names:
        assert hasattr(sbc_lib, n), f"{n} declared in include/*.h but not exported"


def test_reference_surface_is_declared():
    # The reference's src/streamingbc.h:38-64 entry points keep their names.
    names = set(native.header_functions())
    for n in ("streamingBCCreateForestExact", "streamingBCCreateForestApproximate", "streamingBCDeleteForestExact",
              "streamingBCDeleteForestApproximate", "streamingBCCreateAuxilary", "streamingBCDeleteAuxilary",
              "streamingBCInitStaticExact", "streamingBCInitStaticApproximate", "insertEdgeStreamingBC",
              "deleteEdgeStreamingBC", "insertVertexStreamingBC", "deleteVertexStreamingBC",
              "stinger_new", "stinger_set_initial_edges", "stinger_insert_edge", "stinger_outdegree",
              "stinger_free", "CreateStingerFromCSR", "PickRoots"):
        assert n in names, n


def test_error_message_without_device_is_clean(sbc_lib):
    # Asking for a graph on a machine without a GPU must fail with a status, not abort.
    h = ctypes.c_void_p()
    off = (ctypes.c_int64 * 2)(0, 0)
    rc = sbc_lib.sbc_graph_create(ctypes.byref(h), 1, off, off)
    if rc == 0:
        sbc_lib.sbc_graph_destroy(h)
    else:
        assert rc < 0
        assert sbc_lib.sbc_last_error()


def test_headers_compile_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "streamingbc.h"\nint main(void){ bcForest f; (void)f; return 0; }\n')
    inc = os.path.join(os.path.dirname(native.LIB_PATH), "..", "include")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", inc, "-c", str(src), "-o", str(tmp_path / "t.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
