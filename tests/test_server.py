"""Request server (midsx_server_*): continuous batching of requests that arrive while others
run, admission by HBM footprint with phantom eviction and re-upload, failures isolated to
their request.  Every request's results must equal those of running it alone with
midsx_gpu_run on the same Philox streams: bit for bit in the mixed form (integer tallies),
to rounding in FP64 (relative 1e-9)."""
import threading
import time

import numpy as np
import pytest

import midsx_gb300 as M
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    """Two dose classes on tables without lead, radiography on tables with lead; the server's
    default tables are the dose tables, radiography phantoms register their own."""
    tmpl = scenes.serving_templates(pool=2, seed=3, small_edge=16, medium_edge=24, radio_shape=(16, 32, 32),
                                    radio_bins=32, radio_lead=2)
    flat = [sc for v in tmpl.values() for sc in v]
    by_set = {}
    for sc in flat:
        key = tuple(sc.materials)
        if key not in by_set:
            by_set[key] = M.Tables(list(key), e_max=150e3)
    tabs = [by_set[tuple(sc.materials)] for sc in flat]
    assert len(by_set) == 2
    sources = [M.Source(**sc.source) for sc in flat]
    return tabs, flat, sources


def alone(tables, sc, src, n, seed, first, precision, tracking="reference"):
    ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    tl = M.Tallies(ph, sc.specs, sc.dose_mode)
    M.run(tables, ph, src, tl, n, seed=seed, first=first, precision=precision, tracking=tracking)
    return read(tl, sc)


def read(tl, sc):
    out = {"stats": tl.stats()}
    if sc.dose_mode:
        out.update({"dose_" + k: v for k, v in tl.dose().items()})
    for i, spec in enumerate(sc.specs):
        if spec["kind"] == "binned":
            out["binned%d" % i] = tl.binned(i)
        else:
            out["scalar%d" % i] = tl.scalar(i)
    return out


def same(a, b, exact):
    for k in a:
        if k == "stats":
            for f in ("histories", "steps", "voxel_fetches", "photo", "coherent", "incoherent"):
                assert a[k][f] == b[k][f], f
            continue
        x = a[k] if isinstance(a[k], tuple) else (a[k],)
        y = b[k] if isinstance(b[k], tuple) else (b[k],)
        for u, v in zip(x, y):
            if exact:
                np.testing.assert_array_equal(u, v, err_msg=k)
            else:
                np.testing.assert_allclose(u, v, rtol=1e-9, atol=1e-9, err_msg=k)


def register(server, flat, tabs):
    return [server.add_phantom(sc.domain, sc.spacing, sc.origin, sc.ids, sc.background,
                               tables=None if t is server.tables else t) for sc, t in zip(flat, tabs)]


def test_results_same_alone_and_in_the_mix(env):
    tabs, flat, sources = env
    srv = M.Server(tabs[0], launch_histories=40_000, in_flight=2)
    pids = register(srv, flat, tabs)
    rng = np.random.default_rng(5)
    plan = []
    for i in range(14):
        j = int(rng.integers(0, len(flat)))
        n = int(rng.choice([7_000, 25_000, 90_000]))
        prec = "fp64" if i % 5 == 4 else "mixed"
        plan.append((j, n, 1000 + i, int(rng.integers(0, 1 << 20)), prec))
    ids = [None] * len(plan)

    def client():  # arrivals spread over the first launches
        for k, (j, n, seed, first, prec) in enumerate(plan):
            ids[k] = srv.submit(pids[j], sources[j], n, seed, first, prec, flat[j].specs, flat[j].dose_mode)
            time.sleep(0.002)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    infos = [srv.wait(r, timeout=300) for r in ids]
    st = srv.stats()
    assert st["completed"] == len(plan) and st["failed"] == 0
    # requests shared launches: more request-launch pairs than launches
    assert sum(i["launches"] for i in infos) > st["launches"]
    assert st["max_active_seen"] > 1
    for k, (j, n, seed, first, prec) in enumerate(plan):
        info = infos[k]
        assert info["histories_done"] == n and info["t_submit"] <= info["t_admit"] <= info["t_done"]
        got = read(srv.tallies(ids[k]), flat[j])
        ref = alone(tabs[j], flat[j], sources[j], n, seed, first, prec)
        same(got, ref, exact=(prec == "mixed"))
        srv.release(ids[k])
    st = srv.stats()
    assert st["bytes_in_use"] == st["resident_phantom_bytes"]
    srv.close()


def test_macro_cell_tracking_in_the_mix(env):
    """A server launching with MIDSX_TRACK_MACRO_CELL: the requests' phantoms get their
    macro cells when packed, and every request equals its single run with that tracking."""
    tabs, flat, sources = env
    srv = M.Server(tabs[0], launch_histories=30_000, in_flight=2, tracking="macro_cell")
    pids = register(srv, flat, tabs)
    plan = [(j % len(flat), 20_000 + 5_000 * j, 300 + j, 17 * j) for j in range(6)]
    ids = [srv.submit(pids[j], sources[j], n, seed, first, "mixed", flat[j].specs, flat[j].dose_mode)
           for j, n, seed, first in plan]
    for k, (j, n, seed, first) in enumerate(plan):
        srv.wait(ids[k], timeout=300)
        got = read(srv.tallies(ids[k]), flat[j])
        same(got, alone(tabs[j], flat[j], sources[j], n, seed, first, "mixed", "macro_cell"), exact=True)
        srv.release(ids[k])
    assert srv.stats()["failed"] == 0
    srv.close()


def test_admission_by_footprint_evicts_and_reuploads(env):
    """Statistics-only requests (tallies of a few hundred bytes) on a budget that holds about
    two phantoms: admissions wait for memory, idle phantoms are evicted and uploaded again,
    and the trajectories (step, voxel-fetch and interaction counts, integer energy sums) are
    those of the request run alone."""
    tabs, flat, sources = env
    budget = 2 * max(sc.ids.size for sc in flat) + 4096
    srv = M.Server(tabs[0], budget_bytes=budget, launch_histories=30_000)
    pids = register(srv, flat, tabs)
    order = [0, 2, 4, 1, 3, 5, 0, 4]
    ids = [srv.submit(pids[j], sources[j], 20_000, 77 + k, 0, "mixed", (), N.DOSE_OFF)
           for k, j in enumerate(order)]
    for r in ids:
        srv.wait(r, timeout=300)
    st = srv.stats()
    assert st["peak_bytes_in_use"] <= budget
    assert st["phantom_evictions"] > 0 and st["phantom_uploads"] > len(set(order))
    for k, (r, j) in enumerate(zip(ids, order)):
        got = srv.tallies(r).stats()
        ph = M.Phantom(tabs[j], flat[j].domain, flat[j].spacing, flat[j].origin, flat[j].ids, flat[j].background)
        tl = M.Tallies(ph, (), N.DOSE_OFF)
        M.run(tabs[j], ph, sources[j], tl, 20_000, seed=77 + k, precision="mixed")
        ref = tl.stats()
        for f in ("histories", "steps", "voxel_fetches", "photo", "coherent", "incoherent", "deposited_grid",
                  "escaped_energy"):
            assert got[f] == ref[f], (k, f)
        srv.release(r)
    srv.close()


def test_failed_request_is_isolated(env):
    tabs, flat, sources = env
    tables = tabs[0]
    srv = M.Server(tables, launch_histories=20_000)
    pids = register(srv, flat[:1], tabs[:1])
    sc = flat[0]
    hot = M.Source(position=sc.source["position"], direction=sc.source["direction"], energy=300e3)
    bad = srv.submit(pids[0], hot, 5_000, 1, 0, "mixed", sc.specs, sc.dose_mode)
    good = srv.submit(pids[0], sources[0], 15_000, 2, 0, "mixed", sc.specs, sc.dose_mode)
    with pytest.raises(N.MidsxError) as e:
        srv.wait(bad, timeout=120)
    assert e.value.status == N.TABLE_RANGE
    srv.wait(good, timeout=120)
    same(read(srv.tallies(good), sc), alone(tables, sc, sources[0], 15_000, 2, 0, "mixed"), exact=True)
    with pytest.raises(N.MidsxError) as e:
        srv.tallies(bad)
    srv.release(bad)
    srv.release(good)
    with pytest.raises(N.MidsxError) as e:  # larger than the whole budget
        small = M.Server(tables, budget_bytes=1024)
        p = small.add_phantom(sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
        small.submit(p, sources[0], 10, 1, 0, "mixed", sc.specs, sc.dose_mode)
    assert e.value.status == N.OOM
    small.close()
    srv.close()
