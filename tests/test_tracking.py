"""MIDSX_TRACK_BACKGROUND_FAST: flights that start in the background use the background
material's own attenuation as the majorant (exact there) and stop at the first grid face.
MIDSX_TRACK_MACRO_CELL adds local majorants inside the grids: one optical depth is spent cell
by cell (8^3-voxel cells, each with the largest attenuation among its own materials).
Unbiased but with a different use of the random numbers than the reference's global-majorant
Woodcock tracking, so the checks are statistical: per-voxel dose z-scores, totals and
detector tallies against the reference algorithm (same kernel) and against the oracle run
with the reference's own generator; energy balance exact; far fewer steps."""
import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu


def zscores(s1, q1, s2, q2, frac=0.01):
    s1, q1, s2, q2 = (np.ravel(a) for a in (s1, q1, s2, q2))
    sel = (s1 + s2) > frac * max(s1.max(), s2.max())
    return (s1[sel] - s2[sel]) / np.sqrt(q1[sel] + q2[sel])


def run(tables, ph, src, specs, n, seed, precision, tracking, dose_mode=N.DOSE_FULL):
    tl = M.Tallies(ph, specs, dose_mode)
    M.run(tables, ph, src, tl, n, seed=seed, precision=precision, tracking=tracking)
    return tl


FAST = ["background_fast", "macro_cell"]


@pytest.mark.parametrize("tracking", FAST)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fast_equals_reference_water_cube(precision, tracking):
    sc = scenes.water_cube(n_histories=1, n=50, bins=20)
    tables, ph, src, _ = sc.build()
    n = 400_000
    a = run(tables, ph, src, sc.specs, n, 3, precision, "reference")
    b = run(tables, ph, src, sc.specs, n, 4, precision, tracking)
    sa, sb = a.stats(), b.stats()
    assert sb["histories"] == n
    assert sb["steps"] < sa["steps"], (sa["steps"], sb["steps"])
    bal = sb["deposited_grid"] + sb["deposited_background"] + sb["escaped_energy"]
    assert bal == pytest.approx(sb["source_energy"], rel=1e-6)
    da, db = a.dose(), b.dose()
    qa, qb = da["sumsq"].sum(), db["sumsq"].sum()
    assert abs(da["sum"].sum() - db["sum"].sum()) / np.sqrt(qa + qb) < 4
    z = zscores(da["sum"], da["sumsq"], db["sum"], db["sumsq"])
    assert z.size > 100 and np.mean(np.abs(z) > 3) < 0.01
    assert np.mean(z * z) < 1 + 4 * np.sqrt(2 / z.size)
    ea, ca = a.binned(0)
    eb, cb = b.binned(0)
    ta, tb = ea.sum(axis=2).ravel(), eb.sum(axis=2).ravel()
    na, nb = ca.sum(axis=2).ravel(), cb.sum(axis=2).ravel()
    sel = (na + nb) > 200
    zb = (ta[sel] - tb[sel]) / np.sqrt(ta[sel] ** 2 / np.maximum(na[sel], 1) + tb[sel] ** 2 / np.maximum(nb[sel], 1))
    assert np.mean(np.abs(zb) > 4) < 0.01


@pytest.mark.parametrize("tracking", FAST)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fast_cone_beam_crop_against_oracle(precision, tracking):
    """Heterogeneous phantom 50 cm from a cone-beam source (most of a history's reference
    steps are delta steps in that air gap)."""
    sc = scenes.cone_beam_dose(n_histories=1, shape=(32, 64, 64), spacing=0.1, seed=2)
    tables, ph, src, _ = sc.build()
    n = 300_000
    tl = run(tables, ph, src, [], n, 31, precision, tracking)
    st, d = tl.stats(), tl.dose()
    o = oracle.run(oracle.tables_like(tables), n=n, seed=32, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["steps"] < 0.35 * so["steps"], (st["steps"], so["steps"])
    q = d["sumsq"].sum() + o["dose"]["sumsq"].sum()
    assert abs(st["deposited_grid"] - so["deposited_grid"]) / np.sqrt(q) < 4
    esc_rel = abs(st["escaped_energy"] - so["escaped_energy"]) / so["escaped_energy"]
    assert esc_rel < 0.005
    z = zscores(d["sum"], d["sumsq"], o["dose"]["sum"], o["dose"]["sumsq"])
    assert np.mean(np.abs(z) > 3) < 0.015, np.mean(np.abs(z) > 3)


@pytest.mark.parametrize("tracking", FAST)
def test_fast_multi_grid_against_oracle(tracking):
    from test_grids import MATERIALS, three_grid_scene
    domain, grids, source = three_grid_scene()
    tables = M.Tables(MATERIALS, e_max=100e3)
    ph = M.Phantom.from_grids(tables, domain, scenes.AIR, grids)
    src = M.Source(**source)
    n = 300_000
    tl = run(tables, ph, src, [], n, 7, "mixed", tracking)
    d, st = tl.dose(), tl.stats()
    o = oracle.run(oracle.tables_like(tables), domain, None, None, None, scenes.AIR, source, n=n, seed=8, rng=oracle.RNG_MT19937,
                   grids=grids)
    for k in range(3):
        gs, os_ = d["sum"][k].sum(), o["dose"]["sum"][k].sum()
        zt = (gs - os_) / np.sqrt(d["sumsq"][k].sum() + o["dose"]["sumsq"][k].sum())
        assert abs(zt) < 4, (k, zt)
    assert st["steps"] < o["stats"]["steps"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_macro_cells_radiography_with_lead(precision):
    """The radiography layout with lead spheres inside the phantom (the global majorant is
    lead's everywhere): macro cells take the steps per history down by more than an order of
    magnitude while the detector image, the dose and the escaped energy agree with the
    reference algorithm."""
    sc = scenes.radiography(1, shape=(48, 64, 64), spacing=0.1, seed=11, det_bins=16, det_pitch=0.6, sid=40.0,
                            lead_spheres=6)
    tables, ph, src, _ = sc.build()
    n = 200_000
    specs = sc.specs
    a = run(tables, ph, src, specs, n, 5, precision, "reference", N.DOSE_FULL)
    b = run(tables, ph, src, specs, n, 6, precision, "macro_cell", N.DOSE_FULL)
    sa, sb = a.stats(), b.stats()
    assert sb["steps"] * 10 < sa["steps"], (sa["steps"] / n, sb["steps"] / n)
    bal = sb["deposited_grid"] + sb["deposited_background"] + sb["escaped_energy"]
    assert bal == pytest.approx(sb["source_energy"], rel=1e-6)
    da, db = a.dose(), b.dose()
    q = da["sumsq"].sum() + db["sumsq"].sum()
    assert abs(da["sum"].sum() - db["sum"].sum()) / np.sqrt(q) < 4
    z = zscores(da["sum"], da["sumsq"], db["sum"], db["sumsq"])
    assert z.size > 100 and np.mean(np.abs(z) > 3) < 0.015
    ea, ca = a.binned(0)
    eb, cb = b.binned(0)
    for cls in (0, 1, 2, 3):
        na, nb = ca[..., cls].sum(), cb[..., cls].sum()
        assert abs(na - nb) < 4 * np.sqrt(na + nb) + 1, (cls, na, nb)
    ta, tb = ea.sum(axis=2).ravel(), eb.sum(axis=2).ravel()
    ka, kb = ca.sum(axis=2).ravel(), cb.sum(axis=2).ravel()
    sel = (ka + kb) > 200
    zb = (ta[sel] - tb[sel]) / np.sqrt(ta[sel] ** 2 / ka[sel] + tb[sel] ** 2 / kb[sel])
    # tot^2 / count understates a bin's variance when its energies spread (scatter), so a
    # 4-sigma bin is not rare enough to forbid among a few dozen: one is allowed, or 1 %
    assert np.sum(np.abs(zb) > 4) <= max(1, int(0.01 * zb.size)), (zb.size, np.sort(np.abs(zb))[-3:])


def test_macro_cells_overlapping_grids():
    """A later grid that overlaps an earlier one (the earlier grid owns the overlap): the
    later grid's cells there take every material, so a lead block of the first grid inside a
    water slab of the second is still met with a valid majorant - totals and per-grid dose
    against the reference algorithm."""
    lead = np.full((10, 10, 10), scenes.LEAD, np.uint8)
    water = np.full((40, 40, 40), scenes.WATER, np.uint8)
    grids = [(lead, (0.05, 0.05, 0.05), (4.75, 4.75, 4.75)), (water, (0.25, 0.25, 0.25), (0.0, 0.0, 0.0))]
    tables = M.Tables([scenes.AIR, scenes.WATER, scenes.LEAD], e_max=100e3)
    ph = M.Phantom.from_grids(tables, (10, 10, 10), scenes.AIR, grids)
    src = M.Source(position=(5, 5, 0), direction=("disc", (5, 5, 10), (0, 0, 1), 1.0), energy=60e3)
    n = 300_000
    out = {}
    for t, seed in (("reference", 1), ("macro_cell", 2)):
        tl = M.Tallies(ph, [], N.DOSE_FULL)
        M.run(tables, ph, src, tl, n, seed=seed, precision="mixed", tracking=t)
        out[t] = (tl.dose(), tl.stats())
    (da, sa), (db, sb) = out["reference"], out["macro_cell"]
    assert sb["steps"] < sa["steps"]
    for k in range(2):
        zt = (da["sum"][k].sum() - db["sum"][k].sum()) / np.sqrt(da["sumsq"][k].sum() + db["sumsq"][k].sum())
        assert da["sum"][k].sum() > 0 and abs(zt) < 4, (k, zt)
    assert abs(sa["escaped_energy"] - sb["escaped_energy"]) / sa["escaped_energy"] < 0.005


@pytest.mark.parametrize("tracking", FAST)
def test_fast_needs_the_pool(tracking):
    sc = scenes.water_cube(n_histories=1, n=4, bins=2)
    tables, ph, src, tl = sc.build()
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, scheduler="lanes", tracking=tracking)
    assert e.value.status == N.INVALID_ARG
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, tracking=5)
    assert e.value.status == N.INVALID_ARG


def test_macro_cell_edges():
    """Any cell edge gives the same physics: edges of 1 (a majorant per voxel), 4 and 32
    voxels against the reference algorithm on the lead radiography crop; invalid edges are
    refused."""
    sc = scenes.radiography(1, shape=(32, 48, 48), spacing=0.1, seed=12, det_bins=8, det_pitch=0.8, sid=30.0,
                            lead_spheres=4)
    tables, ph, src, _ = sc.build()
    n = 200_000
    ref = run(tables, ph, src, sc.specs, n, 1, "mixed", "reference", N.DOSE_FULL)
    dr, sr = ref.dose(), ref.stats()
    steps = {}
    for edge, seed in ((1, 2), (4, 3), (32, 4)):
        ph.macro_cells(edge)
        tl = run(tables, ph, src, sc.specs, n, seed, "mixed", "macro_cell", N.DOSE_FULL)
        d, st = tl.dose(), tl.stats()
        steps[edge] = st["steps"] / n
        zt = (d["sum"].sum() - dr["sum"].sum()) / np.sqrt(d["sumsq"].sum() + dr["sumsq"].sum())
        assert abs(zt) < 4, (edge, zt)
        assert abs(st["escaped_energy"] - sr["escaped_energy"]) / sr["escaped_energy"] < 0.005, edge
        ea, ca = ref.binned(0)
        eb, cb = tl.binned(0)
        na, nb = ca[..., 0].sum(), cb[..., 0].sum()
        assert abs(na - nb) < 4 * np.sqrt(na + nb), (edge, na, nb)
    # a majorant per voxel is exact: every tentative collision in the grid is real
    assert steps[1] < steps[32]
    for bad in (0, 3, 128, -8):
        with pytest.raises(N.MidsxError) as e:
            ph.macro_cells(bad)
        assert e.value.status == N.INVALID_ARG
