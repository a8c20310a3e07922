"""The two warp schedulers of the transport kernel (MIDSX_SCHED_LANES: each lane parks its
history on an event; MIDSX_SCHED_POOL: each warp keeps 64 photons in shared memory and runs
events 32 at a time) change only the order of work.  Every history keeps its Philox stream,
so the mixed form's integer tallies and the run statistics must be identical, and the FP64
form's tallies equal to rounding order (relative 1e-9), for single and batched launches, any
regroup threshold and block size, and runs with fewer histories than a warp holds."""
import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu

EXACT_STATS = ("histories", "steps", "voxel_fetches", "photo", "coherent", "incoherent", "compton_trials",
               "tally_words", "step_cap_hits", "edge_clamps")


@pytest.fixture(scope="module")
def scene():
    """A 32^3 ellipsoid phantom with lead, a polyenergetic cone beam, a full dose tally, a
    binned detector, a disc and a cuboid tally: every code path of the collision event."""
    sc = scenes.radiography(1, shape=(32, 32, 32), spacing=0.1, seed=11, det_bins=16, det_pitch=0.4, sid=30.0,
                            kvp=90.0, lead_spheres=3)
    sc.specs = sc.specs + [dict(kind="disc", center=(sc.domain[0] / 2, sc.domain[1] / 2, 29.0), normal=(0, 0, 1),
                                radius=3.0),
                           dict(kind="cuboid", min=sc.origin, max=tuple(o + 3.2 for o in sc.origin))]
    sc.dose_mode = N.DOSE_FULL
    tables = M.Tables(sc.materials, e_max=150e3)
    ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    src = M.Source(**sc.source)
    return sc, tables, ph, src


def run(scene, n, precision, scheduler, seed=3, first=0, **kw):
    sc, tables, ph, src = scene
    tl = M.Tallies(ph, sc.specs, sc.dose_mode)
    M.run(tables, ph, src, tl, n, seed=seed, first=first, precision=precision, scheduler=scheduler, **kw)
    out = {"stats": tl.stats(), "dose": tl.dose(), "binned": tl.binned(0), "disc": tl.scalar(1),
           "cuboid": tl.scalar(2)}
    tl.close()
    return out


def same(a, b, exact):
    for k in EXACT_STATS:
        assert a["stats"][k] == b["stats"][k], k
    pairs = [(a["dose"][k], b["dose"][k]) for k in ("sum", "sumsq", "count")]
    pairs += list(zip(a["binned"], b["binned"])) + [(a["disc"], b["disc"]), (a["cuboid"], b["cuboid"])]
    for x, y in pairs:
        if exact:
            np.testing.assert_array_equal(x, y)
        else:
            np.testing.assert_allclose(x, y, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_pool_equals_lanes(scene, precision):
    a = run(scene, 60_000, precision, "lanes")
    b = run(scene, 60_000, precision, "pool")
    assert a["stats"]["histories"] == 60_000 and a["stats"]["photo"] > 0 and a["stats"]["coherent"] > 0
    same(a, b, exact=(precision == "mixed"))


@pytest.mark.parametrize("kw", [dict(regroup=1), dict(regroup=7), dict(regroup=20), dict(block=32),
                                dict(block=64, per_sm=1)])
def test_pool_launch_shapes(scene, kw):
    a = run(scene, 20_000, "mixed", "lanes", seed=5, first=123)
    b = run(scene, 20_000, "mixed", "pool", seed=5, first=123, **kw)
    same(a, b, exact=True)


@pytest.mark.parametrize("n", [1, 5, 63, 64, 65, 300])
def test_pool_few_histories(scene, n):
    same(run(scene, n, "mixed", "lanes", seed=9), run(scene, n, "mixed", "pool", seed=9), exact=True)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_zero_histories_leave_the_tallies_empty(scene, precision):
    """A run of no histories launches nothing: statistics, dose, detector and scalar tallies
    stay zero under both schedulers."""
    for scheduler in ("lanes", "pool"):
        out = run(scene, 0, precision, scheduler)
        assert all(out["stats"][k] == 0 for k in EXACT_STATS)
        for k in ("sum", "sumsq", "count"):
            assert not np.any(out["dose"][k]), k
        for arr in list(out["binned"]) + [out["disc"], out["cuboid"]]:
            assert not np.any(np.asarray(arr, dtype=float))


def test_pool_batched_equals_lanes():
    jobs = scenes.batch_jobs(n_jobs=5, seed=4, edge_range=(12, 40), hist_range=(3e3, 4e4), spacing=0.2)
    tables = M.Tables(jobs[0].materials, e_max=150e3)

    def go(scheduler):
        objs = []
        for sc in jobs:
            ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
            objs.append((ph, M.Source(**sc.source), M.Tallies(ph, sc.specs, sc.dose_mode)))
        b = M.Batch(tables, [(ph, src, tl, 2 + j, 10 * j, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs))])
        b.run("mixed", scheduler=scheduler)
        b.run("mixed", scheduler=scheduler)  # second epoch
        return [(tl.dose(), tl.stats()) for _, _, tl in objs]

    for (da, sa), (db, sb) in zip(go("lanes"), go("pool")):
        for k in ("sum", "sumsq", "count"):
            np.testing.assert_array_equal(da[k], db[k])
        for k in EXACT_STATS:
            assert sa[k] == sb[k], k


def test_bad_scheduler_and_block_rejected(scene):
    sc, tables, ph, src = scene
    tl = M.Tallies(ph, sc.specs, sc.dose_mode)
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, scheduler=7)
    assert e.value.status == N.INVALID_ARG
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, tl, 10, seed=1, scheduler="pool", block=256)
    assert e.value.status == N.INVALID_ARG


def test_pool_aggregates_shared_records():
    """A 2x2x2-voxel water phantom under a pencil beam: most collisions of a warp deposit into
    the same few dose records and cross the same detector bins and scalar tallies, so the
    warp-aggregated atomics sum large peer groups; the integer totals must still equal those
    of one atomic per lane."""
    ids = np.full((2, 2, 2), scenes.WATER, dtype=np.uint8)
    tables = M.Tables([scenes.AIR, scenes.WATER], e_max=100e3)
    ph = M.Phantom(tables, (20, 20, 20), (5, 5, 5), (5, 5, 5), ids, scenes.AIR)
    src = M.Source(position=(10, 10, 0), direction=("beam", (10, 10, 20)), energy=60e3)
    specs = [dict(kind="binned", corner=(5, 5, 19), edge1=(10, 0, 0), edge2=(0, 10, 0), nu=2, nv=2),
             dict(kind="disc", center=(10, 10, 18), normal=(0, 0, 1), radius=8.0),
             dict(kind="cuboid", min=(5, 5, 5), max=(15, 15, 15))]
    out = {}
    for sched in ("lanes", "pool"):
        tl = M.Tallies(ph, specs, N.DOSE_FULL)
        M.run(tables, ph, src, tl, 50_000, seed=21, precision="mixed", scheduler=sched)
        out[sched] = (tl.dose(), tl.binned(0), tl.scalar(1), tl.scalar(2), tl.stats())
    a, b = out["lanes"], out["pool"]
    for k in ("sum", "sumsq", "count"):
        np.testing.assert_array_equal(a[0][k], b[0][k])
    for x, y in zip(a[1], b[1]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[3], b[3])
    for k in EXACT_STATS:
        assert a[4][k] == b[4][k], k
    assert a[0]["count"].sum() > 1000 and a[2][0] > 0
