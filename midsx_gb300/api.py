"""Python view of the C ABI: table building, device handles, runs and result fetches.

Mirrors the reference's objects for the transport path:
  InteractionData(material names)  -> Tables(material ids or names)
  ComputationalDomain + VoxelGrid  -> Phantom(domain, spacing, origin, ids, background)
  PhotonSource(spectrum, direction, PointGeometry) -> Source
  VolumeTally / SurfaceTally       -> Tallies(spec list), plus the voxel dose tally
  runSimulation(...)               -> run(...)
"""
import ctypes as C
import os

import numpy as np

from . import native as N

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

WHICH = {"total": 0, "photo": 1, "coherent": 2, "incoherent": 3, "sfunc": 4, "ffactor": 5, "majorant": 6}


def material_id(name, data_dir=DATA_DIR):
    lib = N.load()
    out = C.c_int32()
    N.check(lib.midsx_catalog_id(data_dir.encode(), name.encode(), C.byref(out)), "midsx_catalog_id")
    return out.value


def material_name(mid, data_dir=DATA_DIR):
    lib = N.load()
    buf = C.create_string_buffer(256)
    N.check(lib.midsx_catalog_name(data_dir.encode(), int(mid), buf, 256), "midsx_catalog_name")
    return buf.value.decode()


class TableBlob:
    """Host FP64 tables of a material list (InteractionData)."""

    def __init__(self, materials, e_max=150e3, data_dir=DATA_DIR):
        lib = N.load()
        ids = [m if isinstance(m, int) else material_id(m, data_dir) for m in materials]
        arr = (C.c_int32 * len(ids))(*ids)
        ptr = C.POINTER(N.TableBlob)()
        N.check(lib.midsx_tables_build(data_dir.encode(), arr, len(ids), float(e_max), C.byref(ptr)),
                "midsx_tables_build")
        self.ptr = ptr
        self.ids = ids
        self.e_max = float(e_max)

    @property
    def blob(self):
        return self.ptr.contents

    def array(self, off, n):
        return np.ctypeslib.as_array(self.blob.data, shape=(self.blob.n_data,))[off:off + n]

    def iarray(self, off, n):
        return np.ctypeslib.as_array(self.blob.idata, shape=(self.blob.n_idata,))[off:off + n]

    def eval(self, material, which, x):
        lib = N.load()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        w = WHICH[which] if isinstance(which, str) else int(which)
        N.check(lib.midsx_tables_eval(self.ptr, int(material), w, N.dptr(x), N.dptr(y), x.size),
                "midsx_tables_eval")
        return y

    def mu_en(self, material, energies):
        """Mass energy-absorption coefficient mu_en/rho (cm2/g) of dense material `material` at
        `energies` (eV): photoelectric plus the electron's mean share of incoherent scatters
        under the transport's own sampling density (midsx_tables_mu_en)."""
        e = np.ascontiguousarray(energies, dtype=np.float64)
        y = np.empty_like(e)
        N.check(N.load().midsx_tables_mu_en(self.ptr, int(material), N.dptr(e), N.dptr(y), e.size),
                "midsx_tables_mu_en")
        return y

    def dense_index(self, mid):
        return self.ids.index(mid)

    def close(self):
        if self.ptr:
            N.load().midsx_tables_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tables:
    """FP64 host tables plus their device copy (FP64 + FP32)."""

    def __init__(self, materials, e_max=150e3, data_dir=DATA_DIR, blob=None):
        self.host = blob if blob is not None else TableBlob(materials, e_max, data_dir)
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.midsx_gpu_tables_create(self.host.ptr, C.byref(h)), "midsx_gpu_tables_create")
        self.handle = h

    def close(self):
        if self.handle:
            N.load().midsx_gpu_tables_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def geometry_spec(domain, spacing, origin, dims, background_id):
    g = N.GeometrySpec()
    g.domain = N.vec3(domain)
    g.spacing = N.vec3(spacing)
    g.origin = N.vec3(origin)
    g.dims = N.I3(*[int(d) for d in dims])
    g.background_id = int(background_id)
    return g


class Phantom:
    """One voxel grid inside a box domain.  ids: uint8 MIDSX material ids shaped (nz, ny, nx)
    (x fastest, the reference's voxel numbering)."""

    def __init__(self, tables, domain, spacing, origin, ids, background_id):
        ids = np.ascontiguousarray(ids, dtype=np.uint8)
        if ids.ndim != 3:
            raise ValueError("ids must be a 3-D array shaped (nz, ny, nx)")
        nz, ny, nx = ids.shape
        self.dims = (nx, ny, nz)
        self.spec = geometry_spec(domain, spacing, origin, self.dims, background_id)
        self.ids = ids
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.midsx_gpu_phantom_create(tables.handle, C.byref(self.spec), ids.ctypes.data, C.byref(h)),
                "midsx_gpu_phantom_create")
        self.handle = h
        self.grid_shapes = [ids.shape]

    @classmethod
    def from_grids(cls, tables, domain, background_id, grids):
        """A domain with several voxel grids (ComputationalDomain's voxel_grids_): grids is a
        list of (ids shaped (nz, ny, nx), spacing, origin).  A point belongs to the first grid
        in the list whose closed box holds it; voxels are numbered grid after grid."""
        self = cls.__new__(cls)
        arr = (N.GridSpec * len(grids))()
        self._grid_ids = []
        for k, (ids, spacing, origin) in enumerate(grids):
            ids = np.ascontiguousarray(ids, dtype=np.uint8)
            if ids.ndim != 3:
                raise ValueError("ids must be 3-D arrays shaped (nz, ny, nx)")
            nz, ny, nx = ids.shape
            arr[k].spacing, arr[k].origin = N.vec3(spacing), N.vec3(origin)
            arr[k].dims = N.I3(nx, ny, nz)
            arr[k].ids = ids.ctypes.data
            self._grid_ids.append(ids)
        dom = (C.c_double * 3)(*[float(x) for x in domain])
        h = C.c_void_p()
        self.handle = None
        N.check(N.load().midsx_gpu_phantom_create_grids(tables.handle, dom, int(background_id), arr, len(grids),
                                                        C.byref(h)), "midsx_gpu_phantom_create_grids")
        self.handle = h
        self.ids = self._grid_ids[0]
        self.dims = tuple(reversed(self.ids.shape))
        self.grid_shapes = [a.shape for a in self._grid_ids]
        self.spec = None
        return self

    @property
    def n_voxels(self):
        return int(sum(np.prod(sh) for sh in self.grid_shapes))

    def macro_cells(self, edge):
        """Rebuilds the macro cells of MIDSX_TRACK_MACRO_CELL with edges of `edge` voxels (a
        power of two, 1..64; the phantom starts with 8)."""
        N.check(N.load().midsx_gpu_phantom_macro_cells(self.handle, int(edge)), "midsx_gpu_phantom_macro_cells")

    def close(self):
        if self.handle:
            N.load().midsx_gpu_phantom_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def source_spec(position, direction, energy=None, spectrum=None):
    """direction: ("beam", through) | ("isotropic",) | ("rect", corner, e1, e2) |
    ("disc", center, normal, radius).  energy: mono energy in eV, or spectrum=(energies, probs)."""
    s = N.SourceSpec()
    s.position = N.vec3(position)
    kind = direction[0]
    if kind == "beam":
        s.direction_kind = N.DIR_BEAM
        s.a = N.vec3(direction[1])
    elif kind == "isotropic":
        s.direction_kind = N.DIR_ISOTROPIC
    elif kind == "rect":
        s.direction_kind = N.DIR_RECTANGLE
        s.a, s.b, s.c = N.vec3(direction[1]), N.vec3(direction[2]), N.vec3(direction[3])
    elif kind == "disc":
        s.direction_kind = N.DIR_DISC
        s.a, s.b = N.vec3(direction[1]), N.vec3(direction[2])
        s.radius = float(direction[3])
    else:
        raise ValueError("unknown direction kind %r" % (kind,))
    keep = []
    if spectrum is not None:
        e = np.ascontiguousarray(spectrum[0], dtype=np.float64)
        p = np.ascontiguousarray(spectrum[1], dtype=np.float64)
        s.spectrum_kind = N.SPEC_POLY
        s.n_bins = e.size
        s.bin_energy = N.dptr(e)
        s.bin_prob = N.dptr(p)
        keep = [e, p]
    else:
        s.spectrum_kind = N.SPEC_MONO
        s.mono_energy = float(energy)
    s._keep = keep
    return s


class Source:
    def __init__(self, position, direction, energy=None, spectrum=None):
        self.spec = source_spec(position, direction, energy, spectrum)
        self.max_energy = float(np.max(spectrum[0])) if spectrum is not None else float(energy)
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.midsx_gpu_source_create(C.byref(self.spec), C.byref(h)), "midsx_gpu_source_create")
        self.handle = h

    def close(self):
        if self.handle:
            N.load().midsx_gpu_source_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tally_specs(specs):
    """specs: list of dicts {kind: 'disc'|'rect'|'binned'|'cuboid', ...}; a disc or rect may
    add spectrum=(e_min, e_width, n_energy) for an incident-energy spectrum."""
    arr = (N.TallySpec * max(1, len(specs)))()
    for i, d in enumerate(specs):
        t = arr[i]
        k = d["kind"]
        if d.get("spectrum") is not None:
            t.e_min, t.e_width, t.n_energy = float(d["spectrum"][0]), float(d["spectrum"][1]), int(d["spectrum"][2])
        if k == "disc":
            t.kind = N.TALLY_DISC
            t.a, t.b, t.radius = N.vec3(d["center"]), N.vec3(d["normal"]), float(d["radius"])
        elif k in ("rect", "binned"):
            t.kind = N.TALLY_RECT if k == "rect" else N.TALLY_BINNED_RECT
            t.a, t.b, t.c = N.vec3(d["corner"]), N.vec3(d["edge1"]), N.vec3(d["edge2"])
            if k == "binned":
                t.nu, t.nv = int(d["nu"]), int(d["nv"])
        elif k == "cuboid":
            t.kind = N.TALLY_AACUBOID
            t.a, t.b = N.vec3(d["min"]), N.vec3(d["max"])
        else:
            raise ValueError("unknown tally kind %r" % (k,))
    return arr


class Tallies:
    def __init__(self, phantom, specs=(), dose_mode=N.DOSE_FULL):
        self.specs = list(specs)
        self.dose_mode = dose_mode
        self.phantom = phantom
        self.shapes = list(phantom.grid_shapes) if phantom is not None else None
        arr = tally_specs(self.specs)
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.midsx_gpu_tallies_create(phantom.handle if phantom is not None else None, arr,
                                             len(self.specs), int(dose_mode), C.byref(h)),
                "midsx_gpu_tallies_create")
        self.handle = h

    def reset(self, stream=None):
        N.check(N.load().midsx_gpu_tallies_reset(self.handle, stream), "midsx_gpu_tallies_reset")

    def stats(self, stream=None, allow_cap=False):
        """Run statistics.  A history that reached the step or Compton-trial cap was cut short
        (the reference's loop has no cap), so that raises MidsxError(STEP_CAP) unless the caller
        opts in with allow_cap=True (e.g. a test that sets a tiny cap on purpose)."""
        st = N.RunStats()
        N.check(N.load().midsx_gpu_fetch_stats(self.handle, C.byref(st), stream), "midsx_gpu_fetch_stats",
                allow=(N.STEP_CAP,) if allow_cap else ())
        return st.as_dict()

    def dose(self, stream=None):
        """Per-voxel dose records: arrays shaped like the phantom's grid, or, for a phantom of
        several grids, lists with one array per grid.  "sum" (eV); with DOSE_FULL or
        DOSE_BATCHES also the reference's per-deposit "sumsq" and "count"; with DOSE_BATCHES
        and at least two batches closed also "var", the batch-method variance of each voxel's
        sum (eV^2), and "batches"."""
        n = int(sum(np.prod(sh) for sh in self.shapes))
        s = np.empty(n)
        full = self.dose_mode in (N.DOSE_FULL, N.DOSE_BATCHES)
        s2 = np.empty(n) if full else None
        c = np.empty(n) if full else None
        N.check(N.load().midsx_gpu_fetch_dose(self.handle, N.dptr(s), N.dptr(s2) if full else None,
                                              N.dptr(c) if full else None, stream), "midsx_gpu_fetch_dose")
        def shaped(a):
            if len(self.shapes) == 1:
                return a.reshape(self.shapes[0])
            parts, off = [], 0
            for sh in self.shapes:
                k = int(np.prod(sh))
                parts.append(a[off:off + k].reshape(sh))
                off += k
            return parts

        out = {"sum": shaped(s)}
        if full:
            out["sumsq"] = shaped(s2)
            out["count"] = shaped(c)
        if self.dose_mode == N.DOSE_BATCHES:
            v = np.empty(n)
            b = C.c_int32()
            st = N.load().midsx_gpu_fetch_dose_variance(self.handle, N.dptr(v), C.byref(b), stream)
            if st == N.OK:
                out["var"] = shaped(v)
                out["batches"] = b.value
            elif st != N.INVALID_ARG:  # fewer than two batches: no variance yet
                N.check(st, "midsx_gpu_fetch_dose_variance")
        return out

    def scalar(self, i, stream=None):
        out = np.empty(N.SCALAR_SLOTS)
        N.check(N.load().midsx_gpu_fetch_scalar(self.handle, int(i), N.dptr(out), stream), "midsx_gpu_fetch_scalar")
        return out

    def binned(self, i, stream=None):
        d = self.specs[i]
        n = d["nu"] * d["nv"] * 4
        e = np.empty(n)
        c = np.empty(n)
        N.check(N.load().midsx_gpu_fetch_binned(self.handle, int(i), N.dptr(e), N.dptr(c), stream),
                "midsx_gpu_fetch_binned")
        return e.reshape(d["nv"], d["nu"], 4), c.reshape(d["nv"], d["nu"], 4)

    def spectrum(self, i, stream=None):
        """Incident-energy spectrum of surface tally i: (count, cosine_sum), each shaped
        (n_energy, 4) - energy bin by scatter class (0 primary, 1 single coherent, 2 single
        incoherent, 3 multiple)."""
        n = int(self.specs[i]["spectrum"][2])
        c = np.empty(n * 4)
        s = np.empty(n * 4)
        N.check(N.load().midsx_gpu_fetch_spectrum(self.handle, int(i), N.dptr(c), N.dptr(s), stream),
                "midsx_gpu_fetch_spectrum")
        return c.reshape(n, 4), s.reshape(n, 4)

    def close(self):
        if self.handle:
            N.load().midsx_gpu_tallies_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PRECISIONS = {"fp64": N.PREC_FP64, "mixed": N.PREC_MIXED}


SCHEDULERS = {"default": N.SCHED_DEFAULT, "lanes": N.SCHED_LANES, "pool": N.SCHED_POOL}


TRACKING = {"reference": N.TRACK_REFERENCE, "background_fast": N.TRACK_BACKGROUND_FAST,
            "macro_cell": N.TRACK_MACRO_CELL}


def run_config(n, seed, first=0, precision="mixed", block=0, per_sm=0, max_steps=0, max_trials=0, regroup=0,
               chunk=0, scheduler="default", tracking="reference", steps_per_pass=0, variance_batches=0,
               pass_repeats=0):
    c = N.RunConfig()
    c.pass_repeats = int(pass_repeats)
    c.variance_batches = int(variance_batches)
    c.steps_per_pass = int(steps_per_pass)
    c.tracking = TRACKING[tracking] if isinstance(tracking, str) else int(tracking)
    c.regroup = int(regroup)
    c.chunk = int(chunk)
    c.scheduler = SCHEDULERS[scheduler] if isinstance(scheduler, str) else int(scheduler)
    c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    c.n_histories = int(n)
    c.seed = int(seed)
    c.first_history = int(first)
    c.block_size = int(block)
    c.blocks_per_sm = int(per_sm)
    c.max_steps = int(max_steps)
    c.max_compton_trials = int(max_trials)
    return c


def run(tables, phantom, source, tallies, n, seed, first=0, precision="mixed", stream=None, **kw):
    """Enqueue n histories (asynchronous on `stream`, a cudaStream_t as int or None)."""
    cfg = run_config(n, seed, first, precision, **kw)
    N.check(N.load().midsx_gpu_run(tables.handle, phantom.handle, source.handle, tallies.handle, C.byref(cfg),
                                   stream), "midsx_gpu_run")


class Stream:
    """A non-blocking CUDA stream (midsx_gpu_stream_*); .handle is the cudaStream_t."""

    def __init__(self):
        h = C.c_void_p()
        N.check(N.load().midsx_gpu_stream_create(C.byref(h)), "midsx_gpu_stream_create")
        self.handle = h

    def synchronize(self):
        N.check(N.load().midsx_gpu_stream_synchronize(self.handle), "midsx_gpu_stream_synchronize")

    def close(self):
        if self.handle:
            N.load().midsx_gpu_stream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several simulations transported by one persistent launch (midsx_gpu_batch_*).
    jobs: list of (phantom, source, tallies, seed, first, n)."""

    def __init__(self, tables, jobs):
        self.tables = tables
        self.jobs = list(jobs)
        arr = (N.BatchJob * len(self.jobs))()
        for i, (ph, src, tl, seed, first, n) in enumerate(self.jobs):
            arr[i].phantom, arr[i].source, arr[i].tallies = ph.handle, src.handle, tl.handle
            arr[i].seed, arr[i].first_history, arr[i].n_histories = int(seed), int(first), int(n)
        h = C.c_void_p()
        N.check(N.load().midsx_gpu_batch_create(tables.handle, arr, len(self.jobs), C.byref(h)),
                "midsx_gpu_batch_create")
        self.handle = h

    @property
    def histories(self):
        return sum(int(j[5]) for j in self.jobs)

    def set_own_launch(self, min_histories=0):
        """Jobs of at least min_histories run as single-job launches of their own ahead of the
        persistent launch (0: the default threshold; 2**64 - 1: every job in the persistent
        launch).  Results are unchanged."""
        N.check(N.load().midsx_gpu_batch_set_own_launch(self.handle, int(min_histories)),
                "midsx_gpu_batch_set_own_launch")

    def run(self, precision="mixed", stream=None, **launch):
        cfg = run_config(0, 0, 0, precision, **launch)
        N.check(N.load().midsx_gpu_batch_run(self.handle, C.byref(cfg), stream), "midsx_gpu_batch_run")

    def capture(self, stream, precision="mixed", **launch):
        cfg = run_config(0, 0, 0, precision, **launch)
        N.check(N.load().midsx_gpu_batch_capture(self.handle, C.byref(cfg), stream), "midsx_gpu_batch_capture")

    def replay(self, stream):
        N.check(N.load().midsx_gpu_batch_replay(self.handle, stream), "midsx_gpu_batch_replay")

    def autotune(self, precision="mixed", trial=2_000_000, stream=None):
        best = N.RunConfig()
        rate = C.c_double()
        N.check(N.load().midsx_gpu_batch_autotune(self.handle, PRECISIONS[precision], int(trial), C.byref(best),
                                                  C.byref(rate), stream), "midsx_gpu_batch_autotune")
        launch = dict(block=best.block_size, per_sm=best.blocks_per_sm, regroup=best.regroup, chunk=best.chunk,
                      scheduler=best.scheduler, steps_per_pass=best.steps_per_pass, pass_repeats=best.pass_repeats)
        return launch, rate.value

    def close(self):
        if self.handle:
            N.load().midsx_gpu_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def trace_deposits(tables, phantom, source, n, seed, first=0, precision="fp64", **kw):
    cfg = run_config(n, seed, first, precision, **kw)
    out = np.empty(int(n))
    N.check(N.load().midsx_gpu_trace_deposits(tables.handle, phantom.handle, source.handle, C.byref(cfg),
                                              N.dptr(out)), "midsx_gpu_trace_deposits")
    return out


def sample(tables, kind, material, energy, n, seed, first=0, precision="fp64"):
    """Device sampler diagnostics: kind 'rayleigh' | 'compton' | 'freepath'."""
    k = {"rayleigh": 0, "compton": 1, "freepath": 2}[kind]
    o0 = np.empty(int(n))
    o1 = np.empty(int(n))
    p = PRECISIONS[precision]
    N.check(N.load().midsx_gpu_sample(tables.handle, p, k, int(material), float(energy), int(seed), int(first),
                                      int(n), N.dptr(o0), N.dptr(o1)), "midsx_gpu_sample")
    return (o0, o1) if k == 1 else o0


def table_index(tables, material, energies):
    e = np.ascontiguousarray(energies, dtype=np.float64)
    idx = np.empty(6 * e.size, dtype=np.int64)
    N.check(N.load().midsx_gpu_table_index(tables.handle, int(material), N.dptr(e), e.size,
                                           idx.ctypes.data_as(N.PI64)), "midsx_gpu_table_index")
    return idx.reshape(e.size, 6)


def run_host(tables, geom_spec, ids, source_spec_, specs, dose_mode, cfg):
    """End-to-end call from host buffers (midsx_gpu_run_host); returns (dose_sum, stats)."""
    ids = np.ascontiguousarray(ids, dtype=np.uint8)
    dose = np.empty(ids.size) if dose_mode else None
    st = N.RunStats()
    arr = tally_specs(specs)
    N.check(N.load().midsx_gpu_run_host(tables.handle, C.byref(geom_spec), ids.ctypes.data, C.byref(source_spec_),
                                        arr, len(specs), int(dose_mode), C.byref(cfg),
                                        N.dptr(dose) if dose is not None else None, C.byref(st)),
            "midsx_gpu_run_host")
    return dose, st.as_dict()


class TallyView(Tallies):
    """Read access to tallies another object owns (a request server's); closing it does
    not free them."""

    def __init__(self, handle, shape, specs=(), dose_mode=N.DOSE_FULL):
        self.handle = handle
        self.shapes = [shape]
        self.specs = list(specs)
        self.dose_mode = dose_mode
        self.phantom = None

    def close(self):
        self.handle = None


class Server:
    """Request server with continuous batching (midsx_server_*): phantoms registered once and
    kept on the device, requests admitted by HBM footprint and advanced together in batched
    launches by a native scheduler thread.  launch: launch shape (block, per_sm, regroup,
    chunk, max_steps, max_trials)."""

    def __init__(self, tables, budget_bytes=0, launch_histories=0, max_active=0, in_flight=0, **launch):
        cfg = N.ServerConfig()
        cfg.hbm_budget_bytes = int(budget_bytes)
        cfg.launch_histories = int(launch_histories)
        cfg.max_active = int(max_active)
        cfg.launches_in_flight = int(in_flight)
        cfg.launch = run_config(0, 0, 0, "mixed", **launch)
        h = C.c_void_p()
        N.check(N.load().midsx_server_create(tables.handle, C.byref(cfg), C.byref(h)), "midsx_server_create")
        self.handle = h
        self.tables = tables
        self._tables = []  # tables of registered phantoms, kept alive with the server
        self._shapes = {}
        self._requests = {}  # id -> (source kept alive, specs, dose_mode, phantom id)

    def add_phantom(self, domain, spacing, origin, ids, background_id, tables=None):
        """Registers a phantom; its requests run with `tables` (default: the server's)."""
        ids = np.ascontiguousarray(ids, dtype=np.uint8)
        nz, ny, nx = ids.shape
        spec = geometry_spec(domain, spacing, origin, (nx, ny, nz), background_id)
        pid = C.c_int32()
        if tables is not None:
            self._tables.append(tables)
        N.check(N.load().midsx_server_add_phantom(self.handle, tables.handle if tables is not None else None,
                                                  C.byref(spec), ids.ctypes.data, C.byref(pid)),
                "midsx_server_add_phantom")
        self._shapes[pid.value] = ids.shape
        return pid.value

    def submit(self, phantom, source, n, seed, first=0, precision="mixed", specs=(), dose_mode=N.DOSE_FULL):
        arr = tally_specs(list(specs))
        r = N.Request()
        r.phantom = int(phantom)
        r.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        r.dose_mode = int(dose_mode)
        r.n_tallies = len(specs)
        r.tallies = C.cast(arr, C.POINTER(N.TallySpec))
        r.source = source.handle
        r.seed, r.first_history, r.n_histories = int(seed), int(first), int(n)
        rid = C.c_uint64()
        N.check(N.load().midsx_server_submit(self.handle, C.byref(r), C.byref(rid)), "midsx_server_submit")
        self._requests[rid.value] = (source, list(specs), int(dose_mode), int(phantom))
        return rid.value

    def poll(self, rid):
        info = N.RequestInfo()
        N.check(N.load().midsx_server_poll(self.handle, int(rid), C.byref(info)), "midsx_server_poll")
        return info.as_dict()

    def wait(self, rid, timeout=600.0):
        info = N.RequestInfo()
        N.check(N.load().midsx_server_wait(self.handle, int(rid), float(timeout), C.byref(info)),
                "midsx_server_wait")
        d = info.as_dict()
        if d["state"] == N.REQ_FAILED:
            raise N.MidsxError(d["status"], "request %d" % rid)
        return d

    def tallies(self, rid):
        h = C.c_void_p()
        N.check(N.load().midsx_server_tallies(self.handle, int(rid), C.byref(h)), "midsx_server_tallies")
        _, specs, dose_mode, pid = self._requests[rid]
        return TallyView(h, self._shapes[pid], specs, dose_mode)

    def release(self, rid):
        N.check(N.load().midsx_server_release(self.handle, int(rid)), "midsx_server_release")
        self._requests.pop(rid, None)

    def stats(self):
        st = N.ServerStats()
        N.check(N.load().midsx_server_get_stats(self.handle, C.byref(st)), "midsx_server_get_stats")
        return st.as_dict()

    def now(self):
        t = C.c_double()
        N.check(N.load().midsx_server_now(self.handle, C.byref(t)), "midsx_server_now")
        return t.value

    def close(self):
        if self.handle:
            N.load().midsx_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
