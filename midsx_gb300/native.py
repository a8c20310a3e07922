"""ctypes binding of the C ABI in include/midsx_gpu.h.

The structures mirror the header field for field.  Loading fails loudly when the shared
library has not been built: there is no CPU fallback in the product path.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

MAX_MATERIALS = 32
SCALAR_SLOTS = 40
MAX_ENERGY_BINS = 65536

OK, INVALID_ARG, OOM, TIMEOUT, STEP_CAP, TABLE_RANGE, CUDA_ERROR, NOT_FOUND, IO_ERROR = range(9)
PREC_FP64, PREC_MIXED = 0, 1
SCHED_DEFAULT, SCHED_LANES, SCHED_POOL = 0, 1, 2
TRACK_REFERENCE, TRACK_BACKGROUND_FAST, TRACK_MACRO_CELL = 0, 1, 2
MACRO_CELL = 8  # voxels per macro-cell edge (MIDSX_MACRO_CELL)
DIR_BEAM, DIR_ISOTROPIC, DIR_RECTANGLE, DIR_DISC = range(4)
SPEC_MONO, SPEC_POLY = 0, 1
TALLY_DISC, TALLY_RECT, TALLY_BINNED_RECT, TALLY_AACUBOID = 1, 2, 3, 4
DOSE_OFF, DOSE_SUM, DOSE_FULL, DOSE_BATCHES = 0, 1, 2, 3

D3 = C.c_double * 3
I3 = C.c_int32 * 3


class LinTable(C.Structure):
    _fields_ = [("x", C.c_int64), ("lx", C.c_int64), ("ly", C.c_int64), ("n", C.c_int32),
                ("reserved", C.c_int32)]


class SplineTable(C.Structure):
    _fields_ = [("knot_e", C.c_int64), ("knot_u", C.c_int64), ("ctrl", C.c_int64),
                ("n_ctrl", C.c_int32), ("degree", C.c_int32), ("lx_min", C.c_double),
                ("lx_max", C.c_double)]


class RitaTable(C.Structure):
    _fields_ = [("energy", C.c_int64), ("log_energy", C.c_int64), ("row_start", C.c_int64),
                ("x", C.c_int64), ("y", C.c_int64), ("a", C.c_int64), ("b", C.c_int64),
                ("n_energy", C.c_int32), ("n_rows", C.c_int32)]


class MaterialTable(C.Structure):
    _fields_ = [("id", C.c_int32), ("reserved", C.c_int32), ("density", C.c_double),
                ("total", LinTable), ("photo", LinTable), ("sfunc", LinTable),
                ("ffactor", LinTable), ("coh", SplineTable), ("incoh", SplineTable),
                ("rita", RitaTable)]


class TableBlob(C.Structure):
    _fields_ = [("version", C.c_int32), ("n_materials", C.c_int32), ("e_max", C.c_double),
                ("majorant", LinTable), ("mat", MaterialTable * MAX_MATERIALS),
                ("n_data", C.c_int64), ("data", C.POINTER(C.c_double)),
                ("n_idata", C.c_int64), ("idata", C.POINTER(C.c_int64))]


class GeometrySpec(C.Structure):
    _fields_ = [("domain", D3), ("spacing", D3), ("origin", D3), ("dims", I3),
                ("background_id", C.c_int32)]


class GridSpec(C.Structure):
    _fields_ = [("spacing", D3), ("origin", D3), ("dims", I3), ("reserved", C.c_int32), ("ids", C.c_void_p)]


class SourceSpec(C.Structure):
    _fields_ = [("position", D3), ("direction_kind", C.c_int32), ("spectrum_kind", C.c_int32),
                ("a", D3), ("b", D3), ("c", D3), ("radius", C.c_double),
                ("mono_energy", C.c_double), ("n_bins", C.c_int32), ("reserved", C.c_int32),
                ("bin_energy", C.POINTER(C.c_double)), ("bin_prob", C.POINTER(C.c_double))]


class TallySpec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nu", C.c_int32), ("nv", C.c_int32),
                ("n_energy", C.c_int32), ("a", D3), ("b", D3), ("c", D3),
                ("radius", C.c_double), ("e_min", C.c_double), ("e_width", C.c_double)]


class RunConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_steps", C.c_int32),
                ("max_compton_trials", C.c_int32), ("block_size", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("regroup", C.c_int32), ("chunk", C.c_int32),
                ("scheduler", C.c_int32), ("tracking", C.c_int32), ("steps_per_pass", C.c_int32),
                ("variance_batches", C.c_int32), ("pass_repeats", C.c_int32), ("seed", C.c_uint64),
                ("first_history", C.c_uint64), ("n_histories", C.c_uint64)]


class BatchJob(C.Structure):
    _fields_ = [("phantom", C.c_void_p), ("source", C.c_void_p), ("tallies", C.c_void_p),
                ("seed", C.c_uint64), ("first_history", C.c_uint64), ("n_histories", C.c_uint64)]


class RunStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "histories", "steps", "voxel_fetches", "photo", "coherent", "incoherent",
        "compton_trials", "step_cap_hits", "compton_cap_hits", "edge_clamps",
        "tally_words")] + [(n, C.c_double) for n in (
            "source_energy", "deposited_grid", "deposited_background", "escaped_energy")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


VP = C.c_void_p
PD = C.POINTER(C.c_double)
PI64 = C.POINTER(C.c_int64)

REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("launch_histories", C.c_uint64),
                ("max_active", C.c_int32), ("launches_in_flight", C.c_int32), ("launch", RunConfig)]


class Request(C.Structure):
    _fields_ = [("phantom", C.c_int32), ("precision", C.c_int32), ("dose_mode", C.c_int32),
                ("n_tallies", C.c_int32), ("tallies", C.POINTER(TallySpec)), ("source", VP),
                ("seed", C.c_uint64), ("first_history", C.c_uint64), ("n_histories", C.c_uint64)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("launches", C.c_int32), ("reserved", C.c_int32),
                ("histories_scheduled", C.c_uint64), ("histories_done", C.c_uint64),
                ("footprint_bytes", C.c_uint64), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_first_launch", C.c_double), ("t_done", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "submitted", "admitted", "completed", "failed", "launches", "histories", "budget_bytes",
        "bytes_in_use", "peak_bytes_in_use", "resident_phantom_bytes", "phantom_uploads",
        "phantom_evictions")] + [(n, C.c_int32) for n in ("queued", "active", "max_active_seen", "reserved")] + [
        ("busy_seconds", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


_SIGNATURES = {
    "midsx_tables_build": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.c_int32, C.c_double,
                                     C.POINTER(C.POINTER(TableBlob))]),
    "midsx_tables_free": (None, [C.POINTER(TableBlob)]),
    "midsx_catalog_id": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_int32)]),
    "midsx_catalog_name": (C.c_int, [C.c_char_p, C.c_int32, C.c_char_p, C.c_int32]),
    "midsx_tables_eval": (C.c_int, [C.POINTER(TableBlob), C.c_int32, C.c_int32, PD, PD, C.c_int64]),
    "midsx_tables_mu_en": (C.c_int, [C.POINTER(TableBlob), C.c_int32, PD, PD, C.c_int64]),
    "midsx_status_string": (C.c_char_p, [C.c_int]),
    "midsx_last_error": (C.c_char_p, []),
    "midsx_gpu_tables_create": (C.c_int, [C.POINTER(TableBlob), C.POINTER(VP)]),
    "midsx_gpu_tables_destroy": (C.c_int, [VP]),
    "midsx_gpu_phantom_create": (C.c_int, [VP, C.POINTER(GeometrySpec), C.c_void_p, C.POINTER(VP)]),
    "midsx_gpu_phantom_destroy": (C.c_int, [VP]),
    "midsx_gpu_phantom_macro_cells": (C.c_int, [VP, C.c_int32]),
    "midsx_gpu_phantom_create_grids": (C.c_int, [VP, C.POINTER(C.c_double), C.c_int32, C.POINTER(GridSpec), C.c_int32,
                                                 C.POINTER(VP)]),
    "midsx_gpu_source_create": (C.c_int, [C.POINTER(SourceSpec), C.POINTER(VP)]),
    "midsx_gpu_source_destroy": (C.c_int, [VP]),
    "midsx_gpu_tallies_create": (C.c_int, [VP, C.POINTER(TallySpec), C.c_int32, C.c_int32, C.POINTER(VP)]),
    "midsx_gpu_tallies_destroy": (C.c_int, [VP]),
    "midsx_gpu_tallies_reset": (C.c_int, [VP, VP]),
    "midsx_gpu_run": (C.c_int, [VP, VP, VP, VP, C.POINTER(RunConfig), VP]),
    "midsx_gpu_fetch_stats": (C.c_int, [VP, C.POINTER(RunStats), VP]),
    "midsx_gpu_fetch_dose": (C.c_int, [VP, PD, PD, PD, VP]),
    "midsx_gpu_fetch_dose_variance": (C.c_int, [VP, PD, C.POINTER(C.c_int32), VP]),
    "midsx_gpu_fetch_scalar": (C.c_int, [VP, C.c_int32, PD, VP]),
    "midsx_gpu_fetch_binned": (C.c_int, [VP, C.c_int32, PD, PD, VP]),
    "midsx_gpu_fetch_spectrum": (C.c_int, [VP, C.c_int32, PD, PD, VP]),
    "midsx_gpu_run_host": (C.c_int, [VP, C.POINTER(GeometrySpec), C.c_void_p, C.POINTER(SourceSpec),
                                     C.POINTER(TallySpec), C.c_int32, C.c_int32, C.POINTER(RunConfig),
                                     PD, C.POINTER(RunStats)]),
    "midsx_gpu_sample": (C.c_int, [VP, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                   C.c_uint64, C.c_int64, PD, PD]),
    "midsx_gpu_table_index": (C.c_int, [VP, C.c_int32, PD, C.c_int64, PI64]),
    "midsx_gpu_probe_sectors": (C.c_int, [VP, C.c_uint64, C.c_int32, C.c_uint64, C.c_uint32,
                                         C.POINTER(C.c_uint64), VP]),
    "midsx_gpu_stream_create": (C.c_int, [C.POINTER(VP)]),
    "midsx_gpu_stream_destroy": (C.c_int, [VP]),
    "midsx_gpu_stream_synchronize": (C.c_int, [VP]),
    "midsx_gpu_batch_create": (C.c_int, [VP, C.POINTER(BatchJob), C.c_int32, C.POINTER(VP)]),
    "midsx_gpu_batch_destroy": (C.c_int, [VP]),
    "midsx_gpu_batch_set_own_launch": (C.c_int, [VP, C.c_uint64]),
    "midsx_gpu_batch_run": (C.c_int, [VP, C.POINTER(RunConfig), VP]),
    "midsx_gpu_batch_capture": (C.c_int, [VP, C.POINTER(RunConfig), VP]),
    "midsx_gpu_batch_replay": (C.c_int, [VP, VP]),
    "midsx_gpu_batch_autotune": (C.c_int, [VP, C.c_int32, C.c_uint64, C.POINTER(RunConfig), PD, VP]),
    "midsx_gpu_trace_deposits": (C.c_int, [VP, VP, VP, C.POINTER(RunConfig), PD]),
    "midsx_gpu_trace_deposits_noalloc": (C.c_int, [VP, VP, VP, C.POINTER(RunConfig), PD, VP]),
    "midsx_server_create": (C.c_int, [VP, C.POINTER(ServerConfig), C.POINTER(VP)]),
    "midsx_server_destroy": (C.c_int, [VP]),
    "midsx_server_add_phantom": (C.c_int, [VP, VP, C.POINTER(GeometrySpec), C.c_void_p, C.POINTER(C.c_int32)]),
    "midsx_server_submit": (C.c_int, [VP, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "midsx_server_poll": (C.c_int, [VP, C.c_uint64, C.POINTER(RequestInfo)]),
    "midsx_server_wait": (C.c_int, [VP, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
    "midsx_server_tallies": (C.c_int, [VP, C.c_uint64, C.POINTER(VP)]),
    "midsx_server_release": (C.c_int, [VP, C.c_uint64]),
    "midsx_server_get_stats": (C.c_int, [VP, C.POINTER(ServerStats)]),
    "midsx_server_now": (C.c_int, [VP, PD]),
}

_lib = None


def library_path():
    return _build.LIB_MAIN


def load():
    """Load libmidsx_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError("libmidsx_gb300.so is not built; run midsx_gb300.build.build() "
                           "(or __graft_entry__.build()) first")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class MidsxError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.midsx_last_error().decode(errors="replace")
        super().__init__("%s failed: %s (%s)" % (where, lib.midsx_status_string(status).decode(), msg))
        self.status = status


def check(status, where, allow=()):
    if status != OK and status not in allow:
        raise MidsxError(status, where)
    return status


def dptr(a):
    return a.ctypes.data_as(PD)


def vec3(v):
    return D3(*[float(x) for x in v])
