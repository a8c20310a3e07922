"""Load driver for the request server: registers the serving mix's phantoms, submits a
seeded Poisson stream of requests at their arrival times from one thread, polls them from
another and retires them from a few reader threads (each reads results to host memory on a
stream of its own, then releases the request).  Reports throughput and request latencies.

Latency of a request = time from its arrival (submission) to the moment its results are in
host memory; the server-side part (submission to the end of its last launch) is reported
beside it.
"""
import queue
import threading
import time

import numpy as np

from . import api
from . import native as N
from . import scenes


class Mix:
    """The serving mix on one server: tables per material set (the dose classes carry no lead,
    the radiography class does, so dose requests keep a soft-tissue majorant), registered
    phantoms and one source per template."""

    def __init__(self, templates, server_kw=None):
        self.templates = templates
        self.tables = {}
        for scs in templates.values():
            for sc in scs:
                key = tuple(sc.materials)
                if key not in self.tables:
                    self.tables[key] = api.Tables(list(key), e_max=max(s.e_max for v in templates.values()
                                                                       for s in v))
        default = self.tables[tuple(templates[scenes.SERVING_CLASSES[0][0]][0].materials)]
        self.server = api.Server(default, **(server_kw or {}))
        self.pid = {}
        self.source = {}
        for name, scs in templates.items():
            for k, sc in enumerate(scs):
                t = self.tables[tuple(sc.materials)]
                self.pid[name, k] = self.server.add_phantom(sc.domain, sc.spacing, sc.origin, sc.ids, sc.background,
                                                            tables=None if t is default else t)
                self.source[name, k] = api.Source(**sc.source)

    def submit(self, req, precision="mixed"):
        sc = self.templates[req["cls"]][req["template"]]
        key = (req["cls"], req["template"])
        return self.server.submit(self.pid[key], self.source[key], req["n"], req["seed"], req.get("first", 0),
                                  precision, sc.specs, sc.dose_mode)

    def read(self, rid, req, stream=None):
        """Results of a done request in host memory (dose arrays or detector images), copied on
        `stream` (None: the legacy default stream)."""
        sc = self.templates[req["cls"]][req["template"]]
        tl = self.server.tallies(rid)
        # a history that reached a cap is counted and reported by drive(), not raised here
        out = {"stats": tl.stats(stream, allow_cap=True)}
        if sc.dose_mode:
            out["dose"] = tl.dose(stream)
        for i, spec in enumerate(sc.specs):
            if spec["kind"] == "binned":
                out["binned%d" % i] = tl.binned(i, stream)
        return out

    def close(self):
        self.server.close()


def drive(mix, requests, precision="mixed", keep=False, poll_s=0.0005, timeout=3600.0, readers=4):
    """Plays `requests` (scenes.serving_requests) against mix.server in real time.  Returns a
    dict of per-request records and summary figures; keep=True also returns the results.
    One thread polls the submitted requests; `readers` threads read finished ones to host
    memory, each on a non-blocking stream of its own, so that a burst of requests finishing
    at the end of one launch is not read one after another (ctypes calls release the GIL)."""
    n = len(requests)
    rids = [None] * n
    t_arr = [None] * n
    t_host = [None] * n
    infos = [None] * n
    results = [None] * n if keep else None
    caps = [None] * n
    errors = []
    submitted = threading.Semaphore(0)
    finished = queue.Queue()
    readers = max(1, int(readers))

    def poll():
        pending = []  # indices of submitted requests not finished yet
        next_idx = 0
        seen = 0
        deadline = time.perf_counter() + timeout
        while seen < n and time.perf_counter() < deadline:
            while submitted.acquire(blocking=False):
                pending.append(next_idx)
                next_idx += 1
            progressed = False
            for i in list(pending):
                info = mix.server.poll(rids[i])
                if info["state"] in (N.REQ_DONE, N.REQ_FAILED):
                    infos[i] = info
                    pending.remove(i)
                    seen += 1
                    finished.put(i)
                    progressed = True
            if not progressed:
                time.sleep(poll_s)
        for _ in range(readers):
            finished.put(None)

    def read():
        stream = api.Stream()
        try:
            while True:
                i = finished.get()
                if i is None:
                    break
                if infos[i]["state"] == N.REQ_DONE:
                    try:
                        res = mix.read(rids[i], requests[i], stream.handle)
                    except N.MidsxError as e:  # e.g. an energy left the tables: the request failed
                        errors.append((i, e.status))
                    else:
                        st = res["stats"]
                        caps[i] = (st["step_cap_hits"], st["compton_cap_hits"])
                        if keep:
                            results[i] = res
                else:
                    errors.append((i, infos[i]["status"]))
                t_host[i] = time.perf_counter()
                mix.server.release(rids[i])
        finally:
            stream.close()

    threads = [threading.Thread(target=poll)] + [threading.Thread(target=read) for _ in range(readers)]
    for th in threads:
        th.start()
    t0 = time.perf_counter()
    for i, req in enumerate(requests):
        delay = t0 + req["t"] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        t_arr[i] = time.perf_counter()
        rids[i] = mix.submit(req, precision)
        submitted.release()
    for th in threads:
        th.join()
    t_end = max(t for t in t_host if t is not None)
    lat = np.array([t_host[i] - t_arr[i] for i in range(n) if t_host[i] is not None])
    srv = np.array([infos[i]["t_done"] - infos[i]["t_submit"] for i in range(n) if infos[i] is not None])
    hist = sum(r["n"] for r in requests)
    span = t_end - t0
    by_cls = {}
    for c in sorted({r["cls"] for r in requests}):
        li = [t_host[i] - t_arr[i] for i in range(n) if requests[i]["cls"] == c and t_host[i] is not None]
        # where the time went (medians, ms): admission wait, wait for the first launch, the
        # launches until done, and the host side (submission, polling, reading the results)
        idx = [i for i in range(n) if requests[i]["cls"] == c and infos[i] is not None and t_host[i] is not None]
        parts = {}
        if idx:
            f = lambda a, b: 1e3 * float(np.median([infos[i][b] - infos[i][a] for i in idx]))  # noqa: E731
            parts = {"admission_wait": f("t_submit", "t_admit"), "first_launch_wait": f("t_admit", "t_first_launch"),
                     "running": f("t_first_launch", "t_done"),
                     "host_side": 1e3 * float(np.median([t_host[i] - t_arr[i] - (infos[i]["t_done"] - infos[i]["t_submit"])
                                                         for i in idx]))}
        by_cls[c] = {"requests": len(li), "p50_ms": 1e3 * float(np.median(li)) if li else None, "median_parts_ms": parts,
                     "p99_ms": 1e3 * float(np.percentile(li, 99)) if li else None,
                     "step_cap_hits": int(sum(caps[i][0] for i in range(n) if requests[i]["cls"] == c and caps[i])),
                     "compton_cap_hits": int(sum(caps[i][1] for i in range(n)
                                                 if requests[i]["cls"] == c and caps[i]))}
    out = {"requests": n, "failed": len(errors), "histories": hist, "span_s": span,
           "step_cap_hits": int(sum(c[0] for c in caps if c)), "compton_cap_hits": int(sum(c[1] for c in caps if c)),
           "histories_per_s": hist / span, "offered_histories_per_s": hist / max(requests[-1]["t"], 1e-9),
           "latency_ms": {"p50": 1e3 * float(np.median(lat)), "p99": 1e3 * float(np.percentile(lat, 99)),
                          "max": 1e3 * float(lat.max())},
           "server_latency_ms": {"p50": 1e3 * float(np.median(srv)), "p99": 1e3 * float(np.percentile(srv, 99))},
           "by_class": by_cls, "server": mix.server.stats()}
    if keep:
        out["results"] = results
    return out
