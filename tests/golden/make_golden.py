"""Generate tests/golden/hvl_reference.json from the MIDSX reference checkout.

The reference's own committed results for its half-value-layer simulations
(cpp_simulations/half_value_layer/data/Al_*_AK_*.txt, 10 repeat runs of 1e6 photons each,
written by generate_hvl_data.sh with hvl_*.cpp) are the only numeric outputs of the
reference transport for a scene that can be rebuilt here.  This script collects:

* the mean and standard error of each air-kerma series,
* the geometry of the aluminium slabs read from the NIfTI headers of
  data/voxels/al_{hvl,qvl}_*.nii.gz (dims, voxel size in cm, material id),
* the scene of hvl.json and hvl_*.cpp (domain, slab origin, disc tally, source),
* the photon spectra data/source_distributions/*.csv (keV, weight),
* the air mass energy-absorption coefficients of the TG-195 sheet
  data/reference_set/04-Case 1 Air Mass Energy Absorption Coefficients.xlsx
  (the reference's own table came from its missing database).

Usage: python make_golden.py [REFERENCE_ROOT]
"""
import gzip
import json
import os
import re
import struct
import sys
import zipfile

HERE = os.path.dirname(os.path.abspath(__file__))


def nifti_header(path):
    with gzip.open(path) as f:
        h = f.read(348)
    dims = struct.unpack("<8h", h[40:56])[1:4]
    pix = struct.unpack("<8f", h[76:108])[1:4]
    unit = h[123] & 0x07  # NIfTI xyz units: 1 m, 2 mm, 3 um
    scale = {1: 100.0, 2: 0.1, 3: 1e-4}.get(unit, 0.1)
    return [int(d) for d in dims], [float(p) * scale for p in pix]


def nifti_first_value(path):
    with gzip.open(path) as f:
        b = f.read(352 + 16)
    off = int(struct.unpack("<f", gzip.open(path).read(348)[108:112])[0])
    with gzip.open(path) as f:
        f.read(off)
        return f.read(1)[0]


def read_xlsx_column_pairs(path):
    z = zipfile.ZipFile(path)
    sheet = z.read("xl/worksheets/sheet1.xml").decode()
    out = []
    for row in re.findall(r"<row[^>]*>(.*?)</row>", sheet):
        cells = dict((ref, val) for ref, attr, val in
                     re.findall(r'<c r="([A-Z]+)\d+"([^>]*)>(?:<f>[^<]*</f>)?<v>([^<]*)</v>', row)
                     if 't="s"' not in attr)
        if "A" in cells and "B" in cells:
            out.append([float(cells["A"]), float(cells["B"])])
    return out


def main(ref):
    hvl = os.path.join(ref, "cpp_simulations/half_value_layer")
    out = {"source": "MIDSX cpp_simulations/half_value_layer (hvl.json, hvl_*.cpp, data/*.txt)",
           "scene": {"domain": [4, 4, 100], "background_id": 3, "slab_origin": [0, 0, 10],
                     "disc_tally": {"center": [2, 2, 100], "normal": [0, 0, 1], "radius": 1.0},
                     "source": {"position": [2, 2, 0], "disc_center": [2, 2, 10], "disc_normal": [0, 0, 1],
                                "disc_radius": 0.1}},
           "cases": {}}
    for case in ("30keV", "100keV", "30kVp", "100kVp"):
        c = {}
        for kind in ("0", "hvl", "qvl"):
            vals = [float(v) for v in open(os.path.join(hvl, "data", "Al_%s_AK_%s.txt" % (case, kind))).read().split()]
            n = len(vals)
            mean = sum(vals) / n
            var = sum((v - mean) ** 2 for v in vals) / (n - 1)
            c["AK_" + kind] = {"mean": mean, "stderr": (var / n) ** 0.5, "runs": n}
            if kind != "0":
                p = os.path.join(ref, "data/voxels", "al_%s_%s.nii.gz" % (kind, case))
                dims, spacing = nifti_header(p)
                c["slab_" + kind] = {"dims": dims, "spacing_cm": spacing, "material_id": nifti_first_value(p)}
        out["cases"][case] = c
    spectra = {}
    for name in ("RQRM3_MO_MO_30kVp", "RQR8_W_AL_100kVp", "RQR9_W_AL_120kVp"):
        rows = [[float(x) for x in line.split(",")] for line in
                open(os.path.join(ref, "data/source_distributions", name + "_E_spectrum.csv")) if line.strip()]
        spectra[name] = rows
    out["spectra"] = spectra
    out["spectrum_of_case"] = {"30kVp": "RQRM3_MO_MO_30kVp", "100kVp": "RQR8_W_AL_100kVp"}
    out["air_mu_en"] = read_xlsx_column_pairs(
        os.path.join(ref, "data/reference_set/04-Case 1 Air Mass Energy Absorption Coefficients.xlsx"))
    with open(os.path.join(HERE, "hvl_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "hvl_reference.json"))


if __name__ == "__main__":
    # the reference checkout: the first argument, else the MIDSX_REFERENCE_ROOT environment variable
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MIDSX_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s <reference checkout> (or set MIDSX_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
