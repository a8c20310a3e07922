"""The interaction database pipeline (midsx_gb300/data/midsx_db.py): the data files of this
build written as a midsx.db with the reference's schema, the reference's own queries run on
it, and a database of that schema read back into data files that build the same tables."""
import importlib.util
import os

import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(os.path.dirname(HERE), "midsx_gb300", "data")


def load_module():
    spec = importlib.util.spec_from_file_location("midsx_db", os.path.join(DATA, "midsx_db.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def db(tmp_path_factory):
    mod = load_module()
    path = str(tmp_path_factory.mktemp("db") / "midsx.db")
    mod.export_db(path, DATA)
    return mod, path


def body(path):
    with open(path) as f:
        return [line for line in f if not line.startswith("#")]


def test_round_trip_gives_the_same_files(db, tmp_path):
    mod, path = db
    n_el, n_mat = mod.import_db(path, str(tmp_path))
    assert n_el == len(body(os.path.join(DATA, "elements.txt")))
    assert n_mat == len(body(os.path.join(DATA, "materials.txt")))
    for name in ("elements.txt", "materials.txt"):
        assert body(os.path.join(DATA, name)) == body(str(tmp_path / name)), name
    with open(os.path.join(DATA, "epdl_photon.bin"), "rb") as a, open(str(tmp_path / "epdl_photon.bin"), "rb") as b:
        assert a.read() == b.read()


def test_reference_queries_on_the_exported_database(db):
    """The queries of material_properties.cpp:25-62, material_helpers.h:113-119 and
    material_data.cpp:147, as the reference writes them, on the exported file."""
    import sqlite3
    mod, path = db
    con = sqlite3.connect(path)
    name = "Water, Liquid"
    rows = con.execute("SELECT MaterialCompositions.ElementID, MaterialCompositions.WeightFraction "
                       "FROM Materials "
                       "INNER JOIN MaterialCompositions ON Materials.MaterialID = MaterialCompositions.MaterialID "
                       "WHERE Materials.Name = '" + name + "';").fetchall()
    comp = dict(rows)
    assert set(comp) == {1, 8} and sum(comp.values()) == pytest.approx(1.0)
    assert con.execute("SELECT Density FROM Materials WHERE Name = '" + name + "';").fetchone()[0] == 1.0
    assert con.execute("SELECT MaterialID FROM Materials WHERE Name = 'Air, Dry (near sea level)';").fetchone()[0] == 3
    assert con.execute("SELECT Name FROM Materials WHERE MaterialID = 130;").fetchone()[0] == "Pb"
    for column in ("Mass", "MassNumber"):
        out = dict(con.execute("SELECT AtomicNumber, " + column + " FROM Elements WHERE ID IN (1,8);").fetchall())
        assert set(out) == {1, 8}
    assert dict(con.execute("SELECT AtomicNumber, MassNumber FROM Elements WHERE ID IN (8,82);").fetchall()) == \
        {8: 16, 82: 207}
    _, _, tables = mod.read_files(DATA)
    for k, (table, column) in enumerate(mod.INTERACTION_TABLES):
        rows = con.execute("SELECT Energy, " + column + " FROM " + table + " WHERE ElementID = " + str(82)).fetchall()
        x, y = tables[82][1][k]
        assert [r[0] for r in rows] == x and [r[1] for r in rows] == y, table
    con.close()


def test_tables_from_an_imported_database_equal_the_shipped_ones(db, tmp_path):
    """A data directory read back from the database builds bit-identical tables."""
    mod, path = db
    mod.import_db(path, str(tmp_path))
    mats = [scenes.AIR, scenes.WATER, scenes.CORTICAL_BONE, scenes.LEAD]
    a = M.TableBlob(mats, e_max=150e3)
    b = M.TableBlob(mats, e_max=150e3, data_dir=str(tmp_path))
    e = np.geomspace(1e3, 150e3, 997)
    for m in range(len(mats)):
        for which in ("total", "photo", "coherent", "incoherent"):
            np.testing.assert_array_equal(a.eval(m, which, e), b.eval(m, which, e))
    assert a.blob.n_data == b.blob.n_data and a.blob.n_idata == b.blob.n_idata
    np.testing.assert_array_equal(a.array(0, a.blob.n_data), b.array(0, b.blob.n_data))


def test_import_keeps_only_materials_with_tables(tmp_path):
    """A database whose material lists an element without interaction tables: the material is
    left out, the others come through."""
    import sqlite3
    mod = load_module()
    path = str(tmp_path / "partial.db")
    mod.export_db(path, DATA)
    con = sqlite3.connect(path)
    con.execute('INSERT INTO "Materials" VALUES (999, ?, 1.0)', ("Unobtainium",))
    con.execute('INSERT INTO "MaterialCompositions" VALUES (999, 99, 1.0)')
    con.commit()
    con.close()
    out = tmp_path / "out"
    _, n_mat = mod.import_db(path, str(out))
    assert n_mat == len(body(os.path.join(DATA, "materials.txt")))
    assert all("Unobtainium" not in line for line in body(str(out / "materials.txt")))
