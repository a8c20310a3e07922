"""The C-ABI library loads and exports every function include/midsx_gpu.h declares, and the
ctypes mirror of the structures has the C layout (checked against offsetof/sizeof computed
by the C compiler).  No device calls: runs without a GPU."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from midsx_gb300 import build, native as N

ROOT = build.ROOT
HEADER = os.path.join(ROOT, "include", "midsx_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(midsx_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = N.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_core_library_exports_api_symbols():
    path = build.LIB_CORE
    if not os.path.exists(path):
        pytest.skip("C++ API library not built")
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", path], capture_output=True, text=True).stdout
    for sym in ("runSimulation", "ComputationalDomain::", "InteractionData::", "PhotonSource::",
                "PhysicsEngine::", "AACuboidVolumeTally::", "DiscSurfaceTally::", "RectangularSurfaceTally::"):
        assert sym in out, sym


STRUCTS = {
    "midsx_lin_table": N.LinTable, "midsx_spline_table": N.SplineTable, "midsx_rita_table": N.RitaTable,
    "midsx_material_table": N.MaterialTable, "midsx_table_blob": N.TableBlob,
    "midsx_geometry_spec": N.GeometrySpec, "midsx_source_spec": N.SourceSpec,
    "midsx_tally_spec": N.TallySpec, "midsx_run_config": N.RunConfig, "midsx_run_stats": N.RunStats,
    "midsx_batch_job": N.BatchJob, "midsx_server_config": N.ServerConfig, "midsx_request": N.Request,
    "midsx_request_info": N.RequestInfo, "midsx_server_stats": N.ServerStats, "midsx_grid_spec": N.GridSpec,
}


def test_ctypes_layout_matches_c_compiler():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "midsx_gpu.h"', "int main(void){"]
    for cname, py in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(src, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = dict(line.split() for line in out.strip().splitlines())
    for cname, py in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)


def test_status_strings_and_errors_without_gpu():
    lib = N.load()
    assert lib.midsx_status_string(N.TABLE_RANGE) == b"energy outside tables"
    # invalid arguments are rejected on the host before any device call
    assert lib.midsx_gpu_tables_create(None, None) == N.INVALID_ARG
    assert lib.midsx_gpu_run(None, None, None, None, None, None) == N.INVALID_ARG
