"""CPU oracle of the transport path - TEST INFRASTRUCTURE ONLY.

A C++/OpenMP restatement of MIDSX's reference transport loop (oracle/oracle.cpp), used by
tests/, __graft_entry__.smoke() and the CPU legs of bench.py as the checker and the timed
CPU baseline.  Nothing in midsx_gb300/ imports this package.

Parity is pinned by the reference's own fixtures where they exist (tests/golden/) and by
the physics checks in tests/; see oracle.cpp for the deviations forced by testing.

The oracle runs on its own interaction tables (oracle/tables.py restates the reference's
table construction in numpy from the element data files), never on the product's: run()
and the samplers take any object with the blob layout of include/midsx_gpu.h (.ptr), and
tables_for(scene) gives the oracle's tables of a scene.  Only the table-index test hands the
product's arrays to oracle.table_index, to check the device's searches on identical arrays.
"""
import ctypes as C
import os

import numpy as np

from midsx_gb300 import native as N
from midsx_gb300.api import geometry_spec, source_spec, tally_specs

from . import tables  # noqa: E402  (the oracle's own table build)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
RNG_PHILOX, RNG_MT19937 = 0, 1

PD = C.POINTER(C.c_double)


class OracleResult(C.Structure):
    _fields_ = [("dose_sum", PD), ("dose_sumsq", PD), ("dose_count", PD), ("scalar", PD),
                ("binned_energy", PD), ("binned_count", PD), ("history_deposit", PD),
                ("stats", N.RunStats), ("run_time", C.c_double),
                ("spectrum_count", PD), ("spectrum_cosine", PD), ("raw_spec", C.c_int32), ("reserved", C.c_int32),
                ("raw_cap", C.c_int64), ("raw_energy", PD), ("raw_cosine", PD), ("raw_n", C.c_int64),
                ("dose_var_hist", PD)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("oracle not built; run midsx_gb300.build.build()")
        lib = C.CDLL(LIB)
        lib.oracle_run.restype = C.c_int
        lib.oracle_run.argtypes = [C.POINTER(N.TableBlob), C.POINTER(N.GeometrySpec), C.c_void_p,
                                   C.POINTER(N.SourceSpec), C.POINTER(N.TallySpec), C.c_int, C.c_uint64,
                                   C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(OracleResult)]
        lib.oracle_run_grids.restype = C.c_int
        lib.oracle_run_grids.argtypes = [C.POINTER(N.TableBlob), C.POINTER(C.c_double), C.c_int,
                                         C.POINTER(N.GridSpec), C.c_int, C.POINTER(N.SourceSpec),
                                         C.POINTER(N.TallySpec), C.c_int, C.c_uint64, C.c_uint64, C.c_uint64,
                                         C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(OracleResult)]
        lib.oracle_sample.restype = C.c_int
        lib.oracle_sample.argtypes = [C.POINTER(N.TableBlob), C.c_int, C.c_int, C.c_double, C.c_uint64,
                                      C.c_uint64, C.c_int64, C.c_int, PD, PD]
        lib.oracle_table_index.restype = C.c_int
        lib.oracle_table_index.argtypes = [C.POINTER(N.TableBlob), C.c_int, PD, C.c_int64,
                                           C.POINTER(C.c_int64)]
        lib.oracle_philox.restype = None
        lib.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.oracle_generator_script.restype = C.c_int
        lib.oracle_generator_script.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_int32), C.c_int64, PD]
        _lib = lib
    return _lib


def run(blob, domain, spacing, origin, ids, background_id, source, specs=(), n=1000, seed=1, first=0,
        rng=RNG_PHILOX, threads=0, max_steps=0, max_trials=0, dose=True, history=False, grids=None, raw_spec=None):
    """blob: midsx_gb300.TableBlob; ids shaped (nz, ny, nx); source: dict(position, direction,
    energy|spectrum) as for midsx_gb300.source_spec; specs: tally dicts.  grids: optional list
    of (ids, spacing, origin) for a domain of several grids (then spacing, origin and ids are
    ignored and dose arrays come as one list entry per grid).  raw_spec: index of a surface
    tally whose raw primary IncidentEnergy / EntranceCosine vectors are returned (out["raw"])."""
    lib = load()
    shapes = None
    if grids is not None:
        garr = (N.GridSpec * len(grids))()
        gkeep = []
        for k, (gids, gsp, gor) in enumerate(grids):
            gids = np.ascontiguousarray(gids, dtype=np.uint8)
            gz, gy, gx = gids.shape
            garr[k].spacing, garr[k].origin, garr[k].dims = N.vec3(gsp), N.vec3(gor), N.I3(gx, gy, gz)
            garr[k].ids = gids.ctypes.data
            gkeep.append(gids)
        shapes = [a.shape for a in gkeep]
        ids = np.concatenate([a.ravel() for a in gkeep])
    else:
        ids = np.ascontiguousarray(ids, dtype=np.uint8)
        nz, ny, nx = ids.shape
        g = geometry_spec(domain, spacing, origin, (nx, ny, nz), background_id)
    s = source_spec(**source)
    arr = tally_specs(list(specs))
    res = OracleResult()
    keep = {}
    nvox = ids.size
    if dose:
        for k in ("dose_sum", "dose_sumsq", "dose_count", "dose_var_hist"):
            keep[k] = np.zeros(nvox)
            setattr(res, k, N.dptr(keep[k]))
    n_scalar = len(specs)
    keep["scalar"] = np.zeros(max(1, n_scalar) * N.SCALAR_SLOTS)
    res.scalar = N.dptr(keep["scalar"])
    nb = sum(d["nu"] * d["nv"] * 4 for d in specs if d["kind"] == "binned")
    keep["binned_energy"] = np.zeros(max(1, nb))
    keep["binned_count"] = np.zeros(max(1, nb))
    res.binned_energy = N.dptr(keep["binned_energy"])
    res.binned_count = N.dptr(keep["binned_count"])
    if history:
        keep["history_deposit"] = np.zeros(int(n))
        res.history_deposit = N.dptr(keep["history_deposit"])
    ns = sum(int(d["spectrum"][2]) * 4 for d in specs if d.get("spectrum") is not None)
    keep["spectrum_count"] = np.zeros(max(1, ns))
    keep["spectrum_cosine"] = np.zeros(max(1, ns))
    res.spectrum_count = N.dptr(keep["spectrum_count"])
    res.spectrum_cosine = N.dptr(keep["spectrum_cosine"])
    res.raw_spec = -1 if raw_spec is None else int(raw_spec)
    if raw_spec is not None:
        # a primary crosses a plane once per history (a straight line, one direction; twice
        # only if the crossing falls exactly on a step boundary)
        keep["raw_energy"] = np.zeros(2 * int(n))
        keep["raw_cosine"] = np.zeros(2 * int(n))
        res.raw_cap = 2 * int(n)
        res.raw_energy = N.dptr(keep["raw_energy"])
        res.raw_cosine = N.dptr(keep["raw_cosine"])
    if grids is not None:
        dom = (C.c_double * 3)(*[float(x) for x in domain])
        rc = lib.oracle_run_grids(blob.ptr, dom, int(background_id), garr, len(grids), C.byref(s), arr, len(specs),
                                  int(seed), int(first), int(n), int(rng), int(threads), int(max_steps),
                                  int(max_trials), C.byref(res))
    else:
        rc = lib.oracle_run(blob.ptr, C.byref(g), ids.ctypes.data, C.byref(s), arr, len(specs), int(seed),
                            int(first), int(n), int(rng), int(threads), int(max_steps), int(max_trials),
                            C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle_run failed with code %d" % rc)
    out = {"stats": res.stats.as_dict(), "run_time": res.run_time}

    def shaped(a):
        if shapes is None:
            return a.reshape(ids.shape)
        parts, off = [], 0
        for sh in shapes:
            k = int(np.prod(sh))
            parts.append(a[off:off + k].reshape(sh))
            off += k
        return parts

    if dose:
        out["dose"] = {"sum": shaped(keep["dose_sum"]), "sumsq": shaped(keep["dose_sumsq"]),
                       "var_hist": shaped(keep["dose_var_hist"]),
                       "count": shaped(keep["dose_count"])}
    out["scalar"] = [keep["scalar"][i * N.SCALAR_SLOTS:(i + 1) * N.SCALAR_SLOTS] for i in range(n_scalar)]
    binned, off = [], 0
    for d in specs:
        if d["kind"] == "binned":
            k = d["nu"] * d["nv"] * 4
            binned.append((keep["binned_energy"][off:off + k].reshape(d["nv"], d["nu"], 4),
                           keep["binned_count"][off:off + k].reshape(d["nv"], d["nu"], 4)))
            off += k
        else:
            binned.append(None)
    out["binned"] = binned
    spectra, off = [], 0
    for d in specs:
        if d.get("spectrum") is not None:
            k = int(d["spectrum"][2]) * 4
            spectra.append((keep["spectrum_count"][off:off + k].reshape(-1, 4),
                            keep["spectrum_cosine"][off:off + k].reshape(-1, 4)))
            off += k
        else:
            spectra.append(None)
    out["spectrum"] = spectra
    if raw_spec is not None:
        out["raw"] = (keep["raw_energy"][:res.raw_n].copy(), keep["raw_cosine"][:res.raw_n].copy())
    if history:
        out["history_deposit"] = keep["history_deposit"]
    return out


def sample(blob, kind, material, energy, n, seed, first=0, rng=RNG_PHILOX):
    lib = load()
    k = {"rayleigh": 0, "compton": 1, "freepath": 2}[kind]
    o0 = np.empty(int(n))
    o1 = np.empty(int(n))
    rc = lib.oracle_sample(blob.ptr, k, int(material), float(energy), int(seed), int(first), int(n), int(rng),
                           N.dptr(o0), N.dptr(o1))
    if rc != 0:
        raise RuntimeError("oracle_sample failed")
    return (o0, o1) if k == 1 else o0


def table_index(blob, material, energies):
    lib = load()
    e = np.ascontiguousarray(energies, dtype=np.float64)
    idx = np.empty(6 * e.size, dtype=np.int64)
    rc = lib.oracle_table_index(blob.ptr, int(material), N.dptr(e), e.size, idx.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise RuntimeError("oracle_table_index failed")
    return idx.reshape(e.size, 6)


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_philox(c, k, o)
    return list(o)


GEN_DRAW, GEN_EVENT, GEN_STEP, GEN_SEGMENT = 0, 1, 2, 3


def generator_script(seed, history, ops):
    """The oracle's Philox-mode generator of one history driven by `ops` (GEN_*): the values
    of its draws, in order."""
    lib = load()
    ops = np.ascontiguousarray(ops, dtype=np.int32)
    out = np.empty(int(np.sum(ops == GEN_DRAW)))
    if lib.oracle_generator_script(int(seed), int(history), ops.ctypes.data_as(C.POINTER(C.c_int32)), ops.size,
                                   N.dptr(out)) != 0:
        raise RuntimeError("oracle_generator_script: unknown op")
    return out


def tables_for(scene):
    """The oracle's own tables (oracle.tables.OracleTables) of a scene's material list."""
    return tables.tables(tuple(int(m) for m in scene.materials), float(scene.e_max))


def tables_like(t):
    """The oracle's own tables of the same materials and e_max as the product's Tables or
    TableBlob `t` (built by oracle/tables.py, not taken from `t`)."""
    host = getattr(t, "host", t)
    return tables.tables(tuple(int(m) for m in host.ids), float(host.e_max))


def run_batches(blob, batches, n, seed=1, first=0, rng=RNG_PHILOX, reduce=None, **kw):
    """run() split into `batches` runs over consecutive history ranges (with the mt19937
    generator, each batch seeded on its own), summed; out["dose"]["var"] is the batch-method
    variance of each voxel's sum, B / (B - 1) sum_b (S_b - S / B)^2 - the estimator of the
    device's MIDSX_DOSE_BATCHES tallies, batch for batch on the same Philox streams.  With
    `reduce` (a function of a batch's dose-sum array, e.g. block sums) the variance is that of
    the reduced sums, and out["dose"]["batch_sums"] holds the B reduced batch sums."""
    B = int(batches)
    if B < 2 or B > n:
        raise ValueError("2 <= batches <= n")
    out, sums, start = None, [], int(first)
    for b in range(B):
        nb = n // B + (1 if b < n % B else 0)
        r = run(blob, n=nb, seed=seed if rng == RNG_PHILOX else seed * 1009 + b, first=start, rng=rng, **kw)
        start += nb
        if "dose" in r:
            a = np.array(r["dose"]["sum"], dtype=np.float64)
            sums.append(reduce(a) if reduce else a)
        out = r if out is None else _add_results(out, r)
    if sums:
        S = np.stack(sums)
        out["dose"]["var"] = B / (B - 1) * ((S - S.mean(axis=0)) ** 2).sum(axis=0)
        out["dose"]["batches"] = B
        if reduce:
            out["dose"]["batch_sums"] = S
    return out


def _add_results(a, b):
    """Sum of two run() results (counts, sums and arrays; run times added)."""
    if isinstance(a, dict):
        return {k: _add_results(a[k], b[k]) for k in a}
    if isinstance(a, (list, tuple)):
        return type(a)(_add_results(x, y) for x, y in zip(a, b))
    if a is None:
        return None
    return a + b
