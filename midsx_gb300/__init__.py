"""midsx_gb300 - GB300-native (CUDA sm_103a) photon-history transport of MIDSX.

The C ABI (include/midsx_gpu.h) is implemented by lib/libmidsx_gb300.so; the C++ API of
MIDSX (include/MIDSX/Core.h) by lib/libmidsx_core.so.  This package binds the C ABI for
Python callers, tests and the benchmark.
"""
from . import build, derived, native  # noqa: F401
from .api import (DATA_DIR, Batch, Phantom, Server, Source, Stream, Tables, TableBlob, Tallies,  # noqa: F401
                  geometry_spec, material_id, material_name, run, run_config, run_host,
                  sample, source_spec, table_index, tally_specs, trace_deposits)
