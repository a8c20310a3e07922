"""The reference's SQLite interaction database (midsx.db) to and from the data files here.

The MIDSX reference reads everything it knows about materials and photon interactions from
an SQLite file, `data/data_sources/EPDL/midsx.db` (include/MIDSX/Core/interaction_data.h:20-22),
through queries of the form (material_data.cpp:147, material_properties.cpp:25-62,
material_helpers.h:113-119):

    SELECT Energy, <column> FROM <table> WHERE ElementID = <Z>
    SELECT MaterialCompositions.ElementID, MaterialCompositions.WeightFraction FROM Materials
        INNER JOIN MaterialCompositions ON Materials.MaterialID = MaterialCompositions.MaterialID
        WHERE Materials.Name = '<name>'
    SELECT AtomicNumber, Mass | Density | MassNumber FROM Elements WHERE ID IN (...)
    SELECT Density FROM Materials WHERE Name = '<name>'
    SELECT Name FROM Materials WHERE MaterialID = <id> / SELECT MaterialID ... WHERE Name = ...

The file itself is not in the reference checkout (only its interaction-table schema,
data/data_sources/EPDL/midsx.sql).  This module is the pipeline between that format and the
files the GPU build reads (epdl_photon.bin, materials.txt, elements.txt):

* ``export``: writes a midsx.db with the reference's schema - Elements, Materials,
  MaterialCompositions and the five interaction tables the transport reads
  (CoherentScatteringCrossSections, IncoherentScatteringCrossSections,
  TotalPhotoIonizationCrossSections in barn vs eV; CoherentScatteringFormFactors,
  IncoherentScatteringFunctions vs momentum transfer) - so that the reference's own queries
  run on the data this build uses;
* ``import``: reads a midsx.db of that schema (the reference's, where a user has one) into
  the three files, so the GPU path runs on exactly the reference's data.

    python midsx_db.py export OUT.db [DATA_DIR]
    python midsx_db.py import IN.db OUT_DIR
"""
import os
import sqlite3
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# (table, value column) of the EPDL tables in epdl_photon.bin order: MF23/MT502, MT504,
# MT522 cross sections, MF27/MT502 form factors, MF27/MT504 scattering functions.
INTERACTION_TABLES = [
    ("CoherentScatteringCrossSections", "CrossSection"),
    ("IncoherentScatteringCrossSections", "CrossSection"),
    ("TotalPhotoIonizationCrossSections", "CrossSection"),
    ("CoherentScatteringFormFactors", "FormFactor"),
    ("IncoherentScatteringFunctions", "ScatteringFunction"),
]

NEUTRON_MASS_U = 1.00866491595  # ENDF AWR = atomic mass / neutron mass

SCHEMA = [
    'CREATE TABLE IF NOT EXISTS "Elements" ("ID" BIGINT, "Symbol" TEXT, "AtomicNumber" BIGINT, "Mass" FLOAT, '
    '"Density" TEXT, "MassNumber" BIGINT, "AtomicWeightRatio" FLOAT)',
    'CREATE TABLE IF NOT EXISTS "Materials" ("MaterialID" BIGINT, "Name" TEXT, "Density" FLOAT)',
    'CREATE TABLE IF NOT EXISTS "MaterialCompositions" ("MaterialID" BIGINT, "ElementID" BIGINT, '
    '"WeightFraction" FLOAT)',
] + [
    'CREATE TABLE IF NOT EXISTS "%s" ("index" BIGINT, "ElementID" BIGINT, "Energy" FLOAT, "%s" FLOAT)' % (t, c)
    for t, c in INTERACTION_TABLES
] + ['CREATE INDEX IF NOT EXISTS "ix_%s_index" ON "%s" ("index")' % (t, t) for t, _ in INTERACTION_TABLES]


def read_files(data_dir=HERE):
    """(elements, materials, tables): elements [(Z, symbol, weight)], materials
    [(id, name, density, [(Z, fraction)])], tables {Z: (awr, [(x, y)] * 5)}."""
    elements = []
    with open(os.path.join(data_dir, "elements.txt")) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            z, sym, w = line.strip().split("|")
            elements.append((int(z), sym, float(w)))
    materials = []
    with open(os.path.join(data_dir, "materials.txt")) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            mid, name, dens, comp = line.rstrip("\n").split("|")
            frac = [(int(a), float(b)) for a, b in (c.split(":") for c in comp.split(","))]
            materials.append((int(mid), name, float(dens), frac))
    tables = {}
    with open(os.path.join(data_dir, "epdl_photon.bin"), "rb") as f:
        b = f.read()
    if b[:8] != b"MIDSXEPD":
        raise ValueError("not an epdl_photon.bin file")
    _, n = struct.unpack_from("<II", b, 8)
    off = 16
    for _ in range(n):
        z, awr = struct.unpack_from("<Id", b, off)
        off += 12
        tabs = []
        for _ in INTERACTION_TABLES:
            (m,) = struct.unpack_from("<I", b, off)
            off += 4
            x = struct.unpack_from("<%dd" % m, b, off)
            off += 8 * m
            y = struct.unpack_from("<%dd" % m, b, off)
            off += 8 * m
            tabs.append((list(x), list(y)))
        tables[z] = (awr, tabs)
    return elements, materials, tables


def write_files(out_dir, elements, materials, tables):
    """The three data files from (elements, materials, tables) as read_files returns them."""
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "materials.txt"), "w") as f:
        f.write("# id|name|density g/cm3|Z:weight fraction,...  (generated by midsx_db.py)\n")
        for mid, name, dens, comp in sorted(materials):
            f.write("%d|%s|%r|%s\n" % (mid, name, dens, ",".join("%d:%r" % c for c in comp)))
    with open(os.path.join(out_dir, "elements.txt"), "w") as f:
        f.write("# Z|symbol|atomic weight g/mol  (generated by midsx_db.py)\n")
        for z, sym, w in sorted(elements):
            f.write("%d|%s|%r\n" % (z, sym, w))
    blob = bytearray(b"MIDSXEPD") + struct.pack("<II", 1, len(tables))
    for z in sorted(tables):
        awr, tabs = tables[z]
        blob += struct.pack("<Id", z, awr)
        for x, y in tabs:
            blob += struct.pack("<I", len(x)) + struct.pack("<%dd" % len(x), *x) + struct.pack("<%dd" % len(y), *y)
    with open(os.path.join(out_dir, "epdl_photon.bin"), "wb") as f:
        f.write(bytes(blob))


def export_db(db_path, data_dir=HERE):
    """Writes a midsx.db (the reference's schema) holding the data files of data_dir."""
    elements, materials, tables = read_files(data_dir)
    if os.path.exists(db_path):
        os.remove(db_path)
    con = sqlite3.connect(db_path)
    try:
        for stmt in SCHEMA:
            con.execute(stmt)
        for z, sym, w in elements:
            con.execute('INSERT INTO "Elements" VALUES (?, ?, ?, ?, ?, ?, ?)',
                        (z, sym, z, w, None, int(round(w)), tables[z][0] if z in tables else w / NEUTRON_MASS_U))
        for mid, name, dens, comp in materials:
            con.execute('INSERT INTO "Materials" VALUES (?, ?, ?)', (mid, name, dens))
            for z, frac in comp:
                con.execute('INSERT INTO "MaterialCompositions" VALUES (?, ?, ?)', (mid, z, frac))
        for k, (table, column) in enumerate(INTERACTION_TABLES):
            index = 0
            rows = []
            for z in sorted(tables):
                x, y = tables[z][1][k]
                for xi, yi in zip(x, y):
                    rows.append((index, z, xi, yi))
                    index += 1
            con.executemany('INSERT INTO "%s" VALUES (?, ?, ?, ?)' % table, rows)
        con.commit()
    finally:
        con.close()


def import_db(db_path, out_dir):
    """Reads a midsx.db of the reference's schema and writes the three data files: every
    element with interaction tables, every material whose elements all have them.  Rows of
    an element's table keep the database's order by "index" (the reference reads them in
    the order the query returns, which for its files is that order)."""
    con = sqlite3.connect("file:%s?mode=ro" % db_path, uri=True)
    try:
        cols = [r[1] for r in con.execute('PRAGMA table_info("Elements")')]
        has_awr = "AtomicWeightRatio" in cols
        q = 'SELECT ID, Symbol, Mass%s FROM "Elements"' % (", AtomicWeightRatio" if has_awr else "")
        el = {int(r[0]): (r[1], float(r[2]), (float(r[3]) if has_awr and r[3] is not None else None))
              for r in con.execute(q)}
        tables = {}
        for z in sorted(el):
            tabs = []
            for table, column in INTERACTION_TABLES:
                rows = con.execute('SELECT Energy, "%s" FROM "%s" WHERE ElementID = ? ORDER BY "index"'
                                   % (column, table), (z,)).fetchall()
                tabs.append(([float(r[0]) for r in rows], [float(r[1]) for r in rows]))
            if all(len(x) > 1 for x, _ in tabs):
                awr = el[z][2] if el[z][2] is not None else el[z][1] / NEUTRON_MASS_U
                tables[z] = (awr, tabs)
        materials = []
        for mid, name, dens in con.execute('SELECT MaterialID, Name, Density FROM "Materials" ORDER BY MaterialID'):
            comp = [(int(r[0]), float(r[1])) for r in con.execute(
                'SELECT ElementID, WeightFraction FROM "MaterialCompositions" WHERE MaterialID = ? ORDER BY rowid',
                (mid,))]
            if comp and all(z in tables for z, _ in comp):
                materials.append((int(mid), name, float(dens), comp))
    finally:
        con.close()
    used = sorted({z for m in materials for z, _ in m[3]})
    elements = [(z, el[z][0], el[z][1]) for z in used]
    write_files(out_dir, elements, materials, {z: tables[z] for z in used})
    return len(elements), len(materials)


if __name__ == "__main__":
    if len(sys.argv) >= 3 and sys.argv[1] == "export":
        export_db(sys.argv[2], sys.argv[3] if len(sys.argv) > 3 else HERE)
    elif len(sys.argv) == 4 and sys.argv[1] == "import":
        print("elements %d, materials %d" % import_db(sys.argv[2], sys.argv[3]))
    else:
        sys.exit(__doc__)
