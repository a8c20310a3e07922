"""Batched launches: several simulations with different phantoms, sources, seeds and history
counts in one persistent launch (midsx_gpu_batch_*), CUDA-graph capture and replay, and the
launch-shape autotuner.  Each job's results must equal those of running that job alone on
the same Philox streams: bit for bit in the mixed form (integer tallies), to rounding in FP64.
"""
import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    jobs = scenes.batch_jobs(n_jobs=4, seed=7, edge_range=(16, 40), hist_range=(2e4, 2e5), spacing=0.2)
    tables = M.Tables(jobs[0].materials, e_max=150e3)
    return tables, jobs


def make(tables, sc):
    ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    src = M.Source(**sc.source)
    tl = M.Tallies(ph, sc.specs, sc.dose_mode)
    return ph, src, tl


def results(tl):
    d = tl.dose()
    st = tl.stats()
    return d["sum"].copy(), d["sumsq"].copy(), d["count"].copy(), st


def test_batch_jobs_equal_single_runs(setup):
    tables, jobs = setup
    objs = [make(tables, sc) for sc in jobs]
    batch = M.Batch(tables, [(ph, src, tl, 100 + j, 1000 * j, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs))])
    batch.run("mixed")
    for j, sc in enumerate(jobs):
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, sc.n_histories, seed=100 + j, first=1000 * j, precision="mixed")
        a = results(objs[j][2])
        b = results(tl)
        for x, y in zip(a[:3], b[:3]):
            np.testing.assert_array_equal(x, y)
        for k in ("histories", "steps", "voxel_fetches", "photo", "coherent", "incoherent", "deposited_grid",
                  "escaped_energy", "source_energy"):
            assert a[3][k] == b[3][k], (j, k)
        assert a[3]["histories"] == sc.n_histories


@pytest.mark.parametrize("scheduler", ["lanes", "pool"])
def test_batch_with_empty_jobs(setup, scheduler):
    """Jobs of no histories, first, between and after the others, take no history ids: the
    other jobs equal their single runs, the empty jobs' tallies stay zero, and a batch of
    empty jobs only runs nothing."""
    tables, jobs = setup
    plan = [(jobs[0], 0), (jobs[0], jobs[0].n_histories), (jobs[1], 0), (jobs[1], jobs[1].n_histories),
            (jobs[1], 0)]
    objs = [make(tables, sc) for sc, _ in plan]
    batch = M.Batch(tables, [(ph, src, tl, 40 + j, 0, n)
                             for j, ((sc, n), (ph, src, tl)) in enumerate(zip(plan, objs))])
    batch.run("mixed", scheduler=scheduler)
    for j, (sc, n) in enumerate(plan):
        a = results(objs[j][2])
        assert a[3]["histories"] == n
        if n == 0:
            assert a[3]["steps"] == 0 and not any(np.any(x) for x in a[:3])
            continue
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, n, seed=40 + j, precision="mixed", scheduler=scheduler)
        b = results(tl)
        for x, y in zip(a[:3], b[:3]):
            np.testing.assert_array_equal(x, y)
        assert a[3]["steps"] == b[3]["steps"]
    empty = [make(tables, jobs[2]) for _ in range(2)]
    nothing = M.Batch(tables, [(ph, src, tl, 1, 0, 0) for ph, src, tl in empty])
    nothing.run("mixed", scheduler=scheduler)
    for _, _, tl in empty:
        st = tl.stats()
        assert st["histories"] == 0 and st["steps"] == 0


def test_batch_fp64_equals_single_runs(setup):
    tables, jobs = setup
    objs = [make(tables, sc) for sc in jobs[:2]]
    batch = M.Batch(tables, [(ph, src, tl, 5, 0, sc.n_histories) for sc, (ph, src, tl) in zip(jobs[:2], objs)])
    batch.run("fp64")
    for j, sc in enumerate(jobs[:2]):
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, sc.n_histories, seed=5, precision="fp64")
        a, b = results(objs[j][2]), results(tl)
        np.testing.assert_allclose(a[0], b[0], rtol=1e-9, atol=1e-6)
        np.testing.assert_array_equal(a[2], b[2])
        assert a[3]["steps"] == b[3]["steps"]


def test_graph_replays_advance_epochs(setup):
    """Two graph replays equal two batch runs and equal single runs over [first, first + 2n)."""
    tables, jobs = setup
    sub = jobs[:3]
    stream = M.Stream()
    A = [make(tables, sc) for sc in sub]
    B = [make(tables, sc) for sc in sub]
    ba = M.Batch(tables, [(ph, src, tl, 9, 0, sc.n_histories) for sc, (ph, src, tl) in zip(sub, A)])
    bb = M.Batch(tables, [(ph, src, tl, 9, 0, sc.n_histories) for sc, (ph, src, tl) in zip(sub, B)])
    ba.capture(stream.handle, "mixed", regroup=20)
    ba.replay(stream.handle)
    ba.replay(stream.handle)
    stream.synchronize()
    bb.run("mixed", stream.handle, regroup=12)
    bb.run("mixed", stream.handle)
    stream.synchronize()
    for j, sc in enumerate(sub):
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, 2 * sc.n_histories, seed=9, precision="mixed")
        a, b, c = results(A[j][2]), results(B[j][2]), results(tl)
        for x, y, z in zip(a[:3], b[:3], c[:3]):
            np.testing.assert_array_equal(x, y)
            np.testing.assert_array_equal(x, z)
        assert a[3]["histories"] == 2 * sc.n_histories


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_large_jobs_in_launches_of_their_own_equal_single_runs(setup, precision):
    """With the own-launch threshold between the jobs' sizes, the large jobs run single-job
    launches inside the batch run and its captured graph: two replays still equal single
    runs over [first, first + 2n) (history ids from the batch's epoch), job by job."""
    tables, jobs = setup
    sizes = sorted(sc.n_histories for sc in jobs)
    threshold = sizes[len(sizes) // 2]
    assert sizes[0] < threshold <= sizes[-1]
    stream = M.Stream()
    objs = [make(tables, sc) for sc in jobs]
    batch = M.Batch(tables, [(ph, src, tl, 60 + j, 500 * j, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs))])
    batch.set_own_launch(threshold)
    batch.capture(stream.handle, precision)
    batch.replay(stream.handle)
    batch.replay(stream.handle)
    stream.synchronize()
    for j, sc in enumerate(jobs):
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, 2 * sc.n_histories, seed=60 + j, first=500 * j, precision=precision)
        a, b = results(objs[j][2]), results(tl)
        if precision == "mixed":
            for x, y in zip(a[:3], b[:3]):
                np.testing.assert_array_equal(x, y)
        else:
            np.testing.assert_allclose(a[0], b[0], rtol=1e-9, atol=1e-6)
            np.testing.assert_array_equal(a[2], b[2])
        assert a[3]["histories"] == b[3]["histories"] == 2 * sc.n_histories
        assert a[3]["steps"] == b[3]["steps"]
    # every job in launches of its own, then none
    for t in (1, 2**64 - 1):
        objs2 = [make(tables, sc) for sc in jobs[:2]]
        b2 = M.Batch(tables, [(ph, src, tl, 60 + j, 500 * j, sc.n_histories)
                              for j, (sc, (ph, src, tl)) in enumerate(zip(jobs[:2], objs2))])
        b2.set_own_launch(t)
        b2.run(precision)
        for j, sc in enumerate(jobs[:2]):
            ph, src, tl = make(tables, sc)
            M.run(tables, ph, src, tl, sc.n_histories, seed=60 + j, first=500 * j, precision=precision)
            assert results(objs2[j][2])[3]["steps"] == results(tl)[3]["steps"]
        b2.close()
    batch.close()
    stream.close()


def test_autotune_picks_a_shape_and_resets_tallies(setup):
    tables, jobs = setup
    objs = [make(tables, sc) for sc in jobs]
    batch = M.Batch(tables, [(ph, src, tl, 1, 0, sc.n_histories) for sc, (ph, src, tl) in zip(jobs, objs)])
    launch, rate = batch.autotune("mixed", trial=200_000)
    assert rate > 0
    if launch["scheduler"] == N.SCHED_POOL:
        assert launch["block"] in (64, 128, 256) and 24 <= launch["regroup"] <= 32
    else:
        assert launch["scheduler"] == N.SCHED_LANES
        assert launch["block"] in (128, 256) and 12 <= launch["regroup"] <= 28 and launch["chunk"] in (1, 4)
    for ph, src, tl in objs:
        assert tl.dose()["sum"].sum() == 0 and tl.stats()["histories"] == 0
    batch.run("mixed", **launch)
    assert sum(tl.stats()["histories"] for _, _, tl in objs) == batch.histories


def test_batch_rejects_mismatched_tables(setup):
    tables, jobs = setup
    other = M.Tables(jobs[0].materials, e_max=150e3)
    ph, src, tl = make(other, jobs[0])
    with pytest.raises(N.MidsxError) as e:
        M.Batch(tables, [(ph, src, tl, 1, 0, 10)])
    assert e.value.status == N.INVALID_ARG


@pytest.mark.parametrize("tracking", ["background_fast", "macro_cell"])
def test_batch_opt_in_tracking_equals_single_runs(setup, tracking):
    """The opt-in tracking modes in batched launches (per-job geometry and macro cells from
    the job records): each job equals its single run with the same mode, bit for bit."""
    tables, jobs = setup
    objs = [make(tables, sc) for sc in jobs]
    batch = M.Batch(tables, [(ph, src, tl, 40 + j, 0, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs, objs))])
    batch.run("mixed", tracking=tracking)
    for j, sc in enumerate(jobs):
        ph, src, tl = make(tables, sc)
        M.run(tables, ph, src, tl, sc.n_histories, seed=40 + j, precision="mixed", tracking=tracking)
        a, b = results(objs[j][2]), results(tl)
        for x, y in zip(a[:3], b[:3]):
            np.testing.assert_array_equal(x, y)
        assert a[3]["steps"] == b[3]["steps"] and a[3]["histories"] == sc.n_histories


def test_batch_with_spectrum_tallies_equals_single_runs(setup):
    """Jobs whose tallies keep incident-energy spectra run on the lane-parking kernel in a
    batch as alone (the photon pool is refused for them); each equals its single run."""
    tables, jobs = setup
    objs = []
    specs = []
    for sc in jobs[:2]:
        ext = [n * h for n, h in zip(sc.ids.shape[::-1], sc.spacing)]
        z = sc.origin[2] + ext[2]
        spec = dict(kind="rect", corner=(sc.origin[0], sc.origin[1], z), edge1=(ext[0], 0, 0), edge2=(0, ext[1], 0),
                    spectrum=(0.0, 2000.0, 80))
        specs.append(spec)
        ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
        objs.append((ph, M.Source(**sc.source), M.Tallies(ph, [spec], sc.dose_mode)))
    batch = M.Batch(tables, [(ph, src, tl, 70 + j, 0, sc.n_histories)
                             for j, (sc, (ph, src, tl)) in enumerate(zip(jobs[:2], objs))])
    with pytest.raises(N.MidsxError):
        batch.run("mixed", scheduler="pool")
    batch.run("mixed")
    for j, sc in enumerate(jobs[:2]):
        ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
        tl = M.Tallies(ph, [specs[j]], sc.dose_mode)
        M.run(tables, ph, M.Source(**sc.source), tl, sc.n_histories, seed=70 + j, precision="mixed")
        a, b = objs[j][2].spectrum(0), tl.spectrum(0)
        assert a[0].sum() > 0
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        np.testing.assert_array_equal(objs[j][2].dose()["sum"], tl.dose()["sum"])
