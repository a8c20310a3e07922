"""Regenerate the photon-interaction data files shipped in this directory.

The MIDSX reference reads its cross sections, form factors, scattering functions and
material compositions from an SQLite database (`include/MIDSX/Core/interaction_data.h:20-22`,
`src/MIDSX/Core/material_data.cpp:145-152`, `src/MIDSX/Core/material_properties.cpp:25-75`).
That database was produced from two sources which the reference repository carries:

* the EPDL97 ENDF-6 element files `data/data_sources/EPDL/NNN.txt`, converted table by
  table in `utility_scripts/sql_database_generator.ipynb` (cells 9, 21-31): MF23/MT502
  coherent, MF23/MT504 incoherent, MF23/MT522 photoionisation cross sections (barn vs eV),
  MF27/MT502 coherent form factors and MF27/MT504 incoherent scattering functions
  (vs momentum transfer x = sin(theta/2)/lambda in 1/Angstrom).  The (x, y) pairs are
  stored unchanged; interpolation laws in the files are ignored, as in the reference.
* material compositions and densities (`utility_scripts/case_5_materials_to_sql.ipynb`,
  `sql_material_generator.ipynb`).  The web-scraped NIST part is not in the reference
  checkout; the AAPM TG-195 sheets `data/reference_set/01-Material Definitions.xlsx` and
  `02-Case 5 Material Definitions.xlsx` are, and supply the compositions used here.

Material IDs follow the reference's numbering where its own phantoms pin it:
3 = "Air, Dry (near sea level)", 48 + Z = pure element named by its symbol (Al = 61,
Pb = 130 in `data/voxels/*.nii.gz`), 150 + voxel value = TG-195 Case 5 materials
("<name> - C5").  Other TG-195 materials get IDs from 170 upward.

Usage:  python make_data.py [REFERENCE_ROOT]
Writes `epdl_photon.bin`, `materials.txt` and `elements.txt` next to this script.
"""
import os
import re
import struct
import sys
import zipfile

HERE = os.path.dirname(os.path.abspath(__file__))

# (MF, MT) of the five tables the transport path reads, in file order.
EPDL_TABLES = [(23, 502), (23, 504), (23, 522), (27, 502), (27, 504)]

# Standard atomic weights (g/mol, IUPAC) of the elements the catalogue uses.  The reference
# took `Elements.Mass` from the `periodictable` package (sql_database_generator.ipynb cell 16).
ATOMIC_WEIGHT = {
    1: 1.00794, 6: 12.0107, 7: 14.0067, 8: 15.9994, 11: 22.98977, 12: 24.305,
    13: 26.981538, 15: 30.973761, 16: 32.065, 17: 35.453, 18: 39.948, 19: 39.0983,
    20: 40.078, 42: 95.94, 53: 126.90447, 74: 183.84, 82: 207.2,
}
SYMBOL = {1: "H", 6: "C", 7: "N", 8: "O", 11: "Na", 12: "Mg", 13: "Al", 15: "P", 16: "S",
          17: "Cl", 18: "Ar", 19: "K", 20: "Ca", 42: "Mo", 53: "I", 74: "W", 82: "Pb"}
SYMBOL_TO_Z = {v: k for k, v in SYMBOL.items()}

# Pure-element materials: symbol -> density (g/cm3).  Al, Mo and W densities are the
# TG-195 values; lead is 11.35 g/cm3.
ELEMENT_MATERIALS = {"Al": 2.699, "Mo": 10.22, "W": 19.3, "Pb": 11.35}

# TG-195 sheet-1 material name -> (catalogue name, catalogue id)
SHEET1_NAMES = {
    "Air": ("Air, Dry (near sea level)", 3),
    "Water": ("Water, Liquid", 48),
    "Breast Adipose": ("Breast Adipose", 170),
    "Breast Glandular": ("Breast Glandular", 171),
    "Breast Skin": ("Breast Skin", 172),
    "PMMA": ("PMMA", 173),
    "Soft Tissue": ("Soft Tissue", 174),
}


def endf_float(field):
    s = field.strip()
    if not s:
        return 0.0
    if "e" not in s.lower():
        # Fortran short form: mantissa followed by a signed exponent, e.g. 1.2345-6
        m = re.match(r"^([+-]?[0-9.]+)([+-][0-9]+)$", s)
        if m:
            return float(m.group(1) + "e" + m.group(2))
    return float(s)


def endf_sections(path):
    secs = {}
    awr = None
    with open(path) as f:
        for line in f:
            if len(line) < 75:
                continue
            try:
                mf = int(line[70:72])
                mt = int(line[72:75])
            except ValueError:
                continue
            secs.setdefault((mf, mt), []).append(line)
            if awr is None and mf == 1 and mt == 451:
                awr = endf_float(line[11:22])
    return secs, awr


def endf_tab1(lines):
    """Parse HEAD + TAB1 of one MF/MT section into (x, y) lists."""
    cont = lines[1]
    nr = int(cont[44:55])
    npts = int(cont[55:66])
    n_interp_lines = (2 * nr + 5) // 6
    vals = []
    for line in lines[2 + n_interp_lines:]:
        for i in range(6):
            field = line[11 * i:11 * i + 11]
            if field.strip():
                vals.append(endf_float(field))
        if len(vals) >= 2 * npts:
            break
    vals = vals[:2 * npts]
    if len(vals) != 2 * npts:
        raise ValueError("short TAB1 record")
    return vals[0::2], vals[1::2]


def read_xlsx_rows(path):
    z = zipfile.ZipFile(path)
    strings = re.findall(r"<t[^>]*>([^<]*)</t>", z.read("xl/sharedStrings.xml").decode())
    sheet = z.read("xl/worksheets/sheet1.xml").decode()
    rows = []
    for row in re.findall(r"<row[^>]*>(.*?)</row>", sheet):
        cells = {}
        for ref, attr, val in re.findall(
                r'<c r="([A-Z]+)\d+"([^>]*)>(?:<f>[^<]*</f>)?<v>([^<]*)</v>', row):
            cells[ref] = strings[int(val)] if 't="s"' in attr else val
        rows.append(cells)
    return rows


def parse_material_sheet(path, first_element_col):
    rows = read_xlsx_rows(path)
    z_row = next(r for r in rows if first_element_col in r and r[first_element_col].isdigit())
    cols = [c for c in sorted(z_row, key=lambda c: (len(c), c)) if z_row[c].isdigit()]
    out = []
    for r in rows:
        yield_row = r
        if not any(c in r for c in cols):
            continue
        if r is z_row or not _is_number(r.get(cols[0], "")):
            continue
        out.append(yield_row)
    return out, {c: int(z_row[c]) for c in cols}


def _is_number(s):
    try:
        float(s)
        return True
    except ValueError:
        return False


def build_materials(ref_root):
    mats = []  # (id, name, density, [(Z, w)])
    rows, zcols = parse_material_sheet(
        os.path.join(ref_root, "data/reference_set/01-Material Definitions.xlsx"), "C")
    for r in rows:
        name = r.get("A")
        if name not in SHEET1_NAMES:
            continue
        cname, cid = SHEET1_NAMES[name]
        comp = [(zcols[c], float(r[c]) / 100.0) for c in zcols if float(r.get(c, "0")) != 0.0]
        mats.append((cid, cname, float(r["B"]), comp))
    rows, zcols = parse_material_sheet(
        os.path.join(ref_root, "data/reference_set/02-Case 5 Material Definitions.xlsx"), "D")
    for r in rows:
        if "B" not in r or not _is_number(r.get("A", "")):
            continue
        comp = [(zcols[c], float(r[c]) / 100.0) for c in zcols if float(r.get(c, "0")) != 0.0]
        mats.append((150 + int(float(r["A"])), r["B"] + " - C5", float(r["C"]), comp))
    for sym, dens in ELEMENT_MATERIALS.items():
        mats.append((48 + SYMBOL_TO_Z[sym], sym, dens, [(SYMBOL_TO_Z[sym], 1.0)]))
    mats.sort()
    ids = [m[0] for m in mats]
    assert len(ids) == len(set(ids)), "duplicate material id"
    return mats


def main(ref_root):
    mats = build_materials(ref_root)
    zs = sorted({z for m in mats for z, _ in m[3]})
    missing = [z for z in zs if z not in ATOMIC_WEIGHT]
    assert not missing, missing
    with open(os.path.join(HERE, "materials.txt"), "w") as f:
        f.write("# id|name|density g/cm3|Z:weight fraction,...  (generated by make_data.py)\n")
        for mid, name, dens, comp in mats:
            f.write("%d|%s|%r|%s\n" % (mid, name, dens, ",".join("%d:%r" % c for c in comp)))
    with open(os.path.join(HERE, "elements.txt"), "w") as f:
        f.write("# Z|symbol|atomic weight g/mol  (generated by make_data.py)\n")
        for z in zs:
            f.write("%d|%s|%r\n" % (z, SYMBOL[z], ATOMIC_WEIGHT[z]))
    blob = bytearray(b"MIDSXEPD")
    blob += struct.pack("<II", 1, len(zs))
    total = 0
    for z in zs:
        secs, awr = endf_sections(os.path.join(ref_root, "data/data_sources/EPDL/%03d.txt" % z))
        blob += struct.pack("<Id", z, awr)
        for key in EPDL_TABLES:
            x, y = endf_tab1(secs[key])
            total += len(x)
            blob += struct.pack("<I", len(x))
            blob += struct.pack("<%dd" % len(x), *x)
            blob += struct.pack("<%dd" % len(y), *y)
    with open(os.path.join(HERE, "epdl_photon.bin"), "wb") as f:
        f.write(bytes(blob))
    print("materials: %d, elements: %d, table points: %d, bytes: %d"
          % (len(mats), len(zs), total, len(blob)))


if __name__ == "__main__":
    # the reference checkout: the first argument, else the MIDSX_REFERENCE_ROOT environment variable
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MIDSX_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s <reference checkout> (or set MIDSX_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
