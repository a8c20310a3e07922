"""MIDSX_TRACK_BACKGROUND_FAST: flights that start in the background use the background
material's own attenuation as the majorant (exact there) and stop at the first grid face.
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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fast_equals_reference_water_cube(precision):
    sc = scenes.water_cube(n_histories=1, n=50, bins=20)
    tables, ph, src, _ = sc.build()
    n = 400_000
    a = run(tables, ph, src, sc.specs, n, 3, precision, "reference")
    b = run(tables, ph, src, sc.specs, n, 4, precision, "background_fast")
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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fast_cone_beam_crop_against_oracle(precision):
    """Heterogeneous phantom 50 cm from a cone-beam source (most of a history's reference
    steps are delta steps in that air gap)."""
    sc = scenes.cone_beam_dose(n_histories=1, shape=(32, 64, 64), spacing=0.1, seed=2)
    tables, ph, src, _ = sc.build()
    n = 300_000
    tl = run(tables, ph, src, [], n, 31, precision, "background_fast")
    st, d = tl.stats(), tl.dose()
    o = oracle.run(tables.host, n=n, seed=32, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["steps"] < 0.35 * so["steps"], (st["steps"], so["steps"])
    q = d["sumsq"].sum() + o["dose"]["sumsq"].sum()
    assert abs(st["deposited_grid"] - so["deposited_grid"]) / np.sqrt(q) < 4
    esc_rel = abs(st["escaped_energy"] - so["escaped_energy"]) / so["escaped_energy"]
    assert esc_rel < 0.005
    z = zscores(d["sum"], d["sumsq"], o["dose"]["sum"], o["dose"]["sumsq"])
    assert np.mean(np.abs(z) > 3) < 0.015, np.mean(np.abs(z) > 3)


def test_fast_multi_grid_against_oracle():
    from test_grids import MATERIALS, three_grid_scene
    domain, grids, source = three_grid_scene()
    tables = M.Tables(MATERIALS, e_max=100e3)
    ph = M.Phantom.from_grids(tables, domain, scenes.AIR, grids)
    src = M.Source(**source)
    n = 300_000
    tl = run(tables, ph, src, [], n, 7, "mixed", "background_fast")
    d, st = tl.dose(), tl.stats()
    o = oracle.run(tables.host, domain, None, None, None, scenes.AIR, source, n=n, seed=8, rng=oracle.RNG_MT19937,
                   grids=grids)
    for k in range(3):
        gs, os_ = d["sum"][k].sum(), o["dose"]["sum"][k].sum()
        zt = (gs - os_) / np.sqrt(d["sumsq"][k].sum() + o["dose"]["sumsq"][k].sum())
        assert abs(zt) < 4, (k, zt)
    assert st["steps"] < o["stats"]["steps"]


def test_fast_needs_the_pool():
    sc = scenes.water_cube(n_histories=1, n=4, bins=2)
    tables, ph, src, tl = sc.build()
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, scheduler="lanes", tracking="background_fast")
    assert e.value.status == N.INVALID_ARG
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, tracking=5)
    assert e.value.status == N.INVALID_ARG
