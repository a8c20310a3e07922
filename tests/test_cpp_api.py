"""The MIDSX C++ API (include/MIDSX/Core.h, lib/libmidsx_core.so): reference-style programs
in midsx_gb300/examples built against it.

* scene loading (JSON + NIfTI-1, written here) and material tables, on the CPU;
* the half-value-layer program (the form of the reference's
  cpp_simulations/half_value_layer/hvl_30keV.cpp) on the GPU, against the reference's own
  committed HVL results.
"""
import gzip
import math
import os
import struct
import subprocess

import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import build

LIB = build.LIBDIR


def exe(name):
    p = os.path.join(LIB, "midsx_example_" + name)
    assert os.path.exists(p), p
    return p


def write_nifti(path, ids, spacing_mm):
    """NIfTI-1 single file, uint8, x fastest; ids shaped (nz, ny, nx)."""
    nz, ny, nx = ids.shape
    hdr = bytearray(348)
    struct.pack_into("<i", hdr, 0, 348)
    struct.pack_into("<8h", hdr, 40, 3, nx, ny, nz, 1, 1, 1, 1)
    struct.pack_into("<hh", hdr, 70, 2, 8)
    struct.pack_into("<8f", hdr, 76, 1.0, spacing_mm[0], spacing_mm[1], spacing_mm[2], 0, 0, 0, 0)
    struct.pack_into("<f", hdr, 108, 352.0)
    struct.pack_into("<f", hdr, 112, 1.0)
    hdr[123] = 2 | 8  # mm, s
    hdr[344:348] = b"n+1\x00"
    data = bytes(hdr) + b"\x00" * 4 + ids.astype(np.uint8).tobytes()
    if path.endswith(".gz"):
        with gzip.open(path, "wb") as f:
            f.write(data)
    else:
        with open(path, "wb") as f:
            f.write(data)


def write_scene(tmp_path, ids, spacing_mm, origin, dim_space, background="Air, Dry (near sea level)", gz=False):
    nii = tmp_path / ("grid.nii.gz" if gz else "grid.nii")
    write_nifti(str(nii), ids, spacing_mm)
    js = tmp_path / "scene.json"
    js.write_text('{"dim_space": [%g, %g, %g], "background_material_name": "%s", '
                  '"voxel_grids": [{"file_path": "%s", "origin": [%g, %g, %g]}]}'
                  % (*dim_space, background, nii.name, *origin))
    return str(js)


def parse(out):
    d = {}
    for line in out.splitlines():
        parts = line.split()
        if parts:
            d.setdefault(parts[0], []).append(parts[1:])
    return d


def test_scene_json_and_nifti_load_through_cpp_api(tmp_path):
    ids = np.full((3, 2, 4), 61, np.uint8)
    ids[0, 0, 0] = 48
    js = write_scene(tmp_path, ids, (1.0, 2.0, 0.5), (1, 2, 3), (10, 10, 20))
    r = subprocess.run([exe("scene_info"), js, "60000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = parse(r.stdout)
    assert [float(x) for x in d["dim_space"][0]] == [10, 10, 20]
    assert d["background"][0] == ["Air,", "Dry", "(near", "sea", "level)"]
    g = d["grid"][0]
    assert g[2:5] == ["4", "2", "3"]
    assert [float(x) for x in g[6:9]] == pytest.approx([0.1, 0.2, 0.05])
    assert [float(x) for x in g[10:13]] == [1, 2, 3]
    assert sorted(int(m[0]) for m in d["material"]) == [48, 61]
    assert int(d["first_voxel_material"][0][0]) == 48
    # table values agree with the Python binding of the same C ABI
    blob = M.TableBlob([3, 48, 61], e_max=150e3)
    mus = {int(m[0]): float(m[-3]) for m in d["mu"]}
    for i, mid in enumerate([3, 48, 61]):
        assert mus[mid] == pytest.approx(blob.eval(i, "total", np.array([60e3]))[0], rel=1e-12)


def test_gz_scene_loads_when_zlib_present(tmp_path):
    if not build._have_zlib():
        pytest.skip("built without zlib")
    ids = np.full((2, 2, 2), 61, np.uint8)
    js = write_scene(tmp_path, ids, (1.0, 1.0, 1.0), (0, 0, 0), (5, 5, 5), gz=True)
    r = subprocess.run([exe("scene_info"), js], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_api_errors_are_exceptions(tmp_path):
    js = tmp_path / "bad.json"
    js.write_text('{"dim_space": [1, 1, 1], "background_material_name": "Unobtainium", "voxel_grids": []}')
    r = subprocess.run([exe("scene_info"), str(js)], capture_output=True, text=True)
    assert r.returncode == 1 and "unknown material name" in r.stderr


def run_hvl(args):
    r = subprocess.run([exe("hvl")] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return {k: float(v[0][0]) for k, v in parse(r.stdout).items()}


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["30keV", "100keV"])
def test_cpp_hvl_program_reproduces_reference(golden, case, tmp_path):
    """The reference-style C++ program (runSimulation, DiscSurfaceTally, PhysicsEngine,
    ComputationalDomain) on the GPU reproduces the reference's own AK_hvl / AK_0 and
    AK_qvl / AK_0 (mono-energetic: ratios of primary counts)."""
    e = float(case.replace("keV", "")) * 1e3
    n = 2_000_000
    c = golden["cases"][case]
    air = run_hvl(["-", e, n])
    assert air["area"] == pytest.approx(math.pi)
    for kind in ("hvl", "qvl"):
        s = c["slab_" + kind]
        if kind == "hvl":
            r = run_hvl(["-", e, n, s["dims"][2], s["spacing_cm"][2]])
        else:  # the same slab read from a scene JSON + NIfTI file
            ids = np.full((s["dims"][2], 1, 1), 61, np.uint8)
            js = write_scene(tmp_path, ids, [10 * x for x in s["spacing_cm"]], (0, 0, 10), (4, 4, 100))
            r = run_hvl([js, e, n])
        ratio = r["primary_photons"] / air["primary_photons"]
        ref = c["AK_" + kind]["mean"] / c["AK_0"]["mean"]
        pa, pb = r["primary_photons"] / n, air["primary_photons"] / n
        sig = ratio * math.sqrt((1 - pa) / (n * pa) + (1 - pb) / (n * pb))
        assert abs(ratio - ref) < 4 * math.hypot(sig, 1e-4), (kind, ratio, ref)
        assert r["primary_energy"] == pytest.approx(e * r["primary_photons"], rel=1e-9)
