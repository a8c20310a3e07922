"""Table sets of many materials: the twenty materials of the TG-195 Case 5 voxel volume
(ids 150-169), which the reference's CT example (cpp_simulations/CT_w_voxelized_solid) runs
in one domain.  The per-photon attenuation caches in shared memory grow with the material
count; launches whose default block would not fit take a smaller one.  FP64 histories equal
the oracle's on the same Philox streams, the schedulers and the batched launch give the
same results, and the macro-cell masks carry all twenty materials."""
import os

import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import native as N
from midsx_gb300 import scenes

CASE5 = list(range(150, 170))  # "Air - C5" (150) ... "Cortical Bone - C5" (169)


def case5_scene(n_histories=50_000, edge=24, seed=3):
    """edge^3 voxels at 2 mm in 2^3-voxel blocks of random Case 5 materials, with an air
    margin, in a 10 cm air box; 80 kVp cone beam from the box's face, dose and an exit
    detector."""
    rng = np.random.default_rng(seed)
    blocks = rng.choice(CASE5, size=(edge // 2,) * 3)
    ids = np.repeat(np.repeat(np.repeat(blocks, 2, 0), 2, 1), 2, 2).astype(np.uint8)
    ids[:, :, :2] = 150
    h = 0.2
    ext = edge * h
    origin = (5.0 - ext / 2, 5.0 - ext / 2, 2.0)
    spectrum = scenes.kramers_spectrum(80.0)
    source = dict(position=(5.0, 5.0, 0.0), direction=("disc", (5.0, 5.0, 2.0), (0, 0, 1), 2.0),
                  spectrum=spectrum)
    specs = [dict(kind="binned", corner=(origin[0], origin[1], 2.0 + ext), edge1=(ext, 0, 0), edge2=(0, ext, 0),
                  nu=8, nv=8)]
    return scenes.Scene("case5_materials", CASE5, (10.0, 10.0, 10.0), (h, h, h), origin, ids, 150, source, specs,
                        N.DOSE_FULL, n_histories, 100e3)


def test_blob_takes_twenty_materials_and_refuses_too_many():
    blob = M.TableBlob(CASE5, e_max=100e3)
    assert blob.blob.n_materials == 20
    assert [blob.blob.mat[m].id for m in range(20)] == CASE5
    with pytest.raises(N.MidsxError) as e:
        M.TableBlob((CASE5 * 2)[:N.MAX_MATERIALS + 1], e_max=100e3)
    assert e.value.status == N.INVALID_ARG


@pytest.fixture(scope="module")
def case5():
    sc = case5_scene()
    return sc, sc.build()


@pytest.mark.gpu
def test_fp64_histories_equal_oracle_with_twenty_materials(case5):
    sc, (tables, ph, src, tl) = case5
    n = 40_000
    g = M.trace_deposits(tables, ph, src, n, seed=8, precision="fp64")
    o = oracle.run(oracle.tables_like(tables), n=n, seed=8, history=True, dose=False, **sc.oracle_kwargs())["history_deposit"]
    same = np.abs(g - o) <= 1e-9 * np.maximum(1.0, np.abs(o))
    assert same.mean() > 0.999, same.mean()
    assert g.sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_schedulers_and_batch_agree_with_twenty_materials(case5, precision):
    """Pool and lane-parking launches, and a two-job batch whose default block shrinks to fit
    the caches of twenty materials, give the same tallies (bit for bit in the mixed form)."""
    sc, (tables, ph, src, _) = case5

    def single(scheduler, seed):
        tl = M.Tallies(ph, sc.specs, sc.dose_mode)
        M.run(tables, ph, src, tl, sc.n_histories, seed=seed, precision=precision, scheduler=scheduler)
        return tl

    def check(a, b):
        da, db = a.dose(), b.dose()
        sa, sb = a.stats(), b.stats()
        assert sa["histories"] == sb["histories"] == sc.n_histories
        assert sa["steps"] == sb["steps"] and sa["voxel_fetches"] == sb["voxel_fetches"]
        for k in ("sum", "sumsq", "count"):
            if precision == "mixed":
                np.testing.assert_array_equal(da[k], db[k])
            else:
                np.testing.assert_allclose(da[k], db[k], rtol=1e-9, atol=1e-9)

    pool, lanes = single("pool", 4), single("lanes", 4)
    check(pool, lanes)
    assert pool.stats()["photo"] > 0 and pool.dose()["count"].sum() > 0
    jobs = [M.Tallies(ph, sc.specs, sc.dose_mode) for _ in range(2)]
    batch = M.Batch(tables, [(ph, src, tl, 4 + j, 0, sc.n_histories) for j, tl in enumerate(jobs)])
    batch.run(precision, scheduler="pool")
    check(jobs[0], pool)
    check(jobs[1], single("pool", 5))


@pytest.mark.gpu
def test_whole_catalogue_in_one_table_set():
    """All 31 materials of the data files in one table set: a batch's default block shrinks
    until the FP64 caches of its photon slots fit (256 threads would need 512 slots x 31
    materials x 2 x 8 B = 254 KB) and equals the single run; asking for 256 threads is an
    error, not a failed launch."""
    path = os.path.join(os.path.dirname(M.__file__), "data", "materials.txt")
    catalogue = [int(line.split("|")[0]) for line in open(path) if line.strip() and not line.startswith("#")]
    assert len(catalogue) == 31 and set(CASE5) <= set(catalogue)
    sc = case5_scene(n_histories=20_000)
    tables = M.Tables(catalogue, e_max=100e3)
    ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    src = M.Source(**sc.source)
    tl = M.Tallies(ph, sc.specs, sc.dose_mode)
    M.run(tables, ph, src, tl, sc.n_histories, seed=6, precision="fp64")
    jobs = [M.Tallies(ph, sc.specs, sc.dose_mode)]
    batch = M.Batch(tables, [(ph, src, jobs[0], 6, 0, sc.n_histories)])
    batch.run("fp64")
    a, b = jobs[0].dose(), tl.dose()
    np.testing.assert_allclose(a["sum"], b["sum"], rtol=1e-9, atol=1e-9)
    assert jobs[0].stats()["steps"] == tl.stats()["steps"] > 0
    jobs[0].reset()
    with pytest.raises(N.MidsxError) as e:
        batch.run("fp64", scheduler="pool", block=256)
    assert e.value.status == N.INVALID_ARG
    assert jobs[0].stats()["histories"] == 0


@pytest.mark.gpu
def test_macro_cells_with_twenty_materials(case5):
    """Macro-cell tracking with masks over twenty materials: energy balance, and totals within
    statistics of the reference tracking."""
    sc, (tables, ph, src, _) = case5
    n = 400_000
    out = {}
    for mode in ("reference", "macro_cell"):
        tl = M.Tallies(ph, sc.specs, sc.dose_mode)
        M.run(tables, ph, src, tl, n, seed=12, precision="mixed", tracking=mode)
        st = tl.stats()
        bal = st["deposited_grid"] + st["deposited_background"] + st["escaped_energy"]
        assert bal == pytest.approx(st["source_energy"], rel=1e-6)
        out[mode] = (st, tl.dose())
    (sr, dr), (sm, dm) = out["reference"], out["macro_cell"]
    assert sm["steps"] < sr["steps"]
    # two independent estimates of the grid deposit (relative standard error ~0.3 %)
    assert sm["deposited_grid"] == pytest.approx(sr["deposited_grid"], rel=0.015)
    assert dm["sum"].sum() == pytest.approx(dr["sum"].sum(), rel=0.015)
