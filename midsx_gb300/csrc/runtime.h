// Internal interface between the transport library (transport.cu) and the request server
// (server.cu): packed job records, launches over records already on the device, and
// stream-ordered tallies and phantom storage drawn from a memory pool, so that a scheduler
// thread can admit and retire requests while kernels run without a device-wide
// synchronisation (cudaMalloc/cudaFree and cudaMemcpy would wait for the running launches).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "midsx_gpu.h"

namespace midsx {
namespace rt {

// Size in bytes of one device job record (a DevJob).
size_t job_record_bytes();

// Validates one job (handles made with `tables`, dose tally sized for the phantom, source
// energy inside the tables and, for the mixed form, under its fixed-point limit; tallies
// empty or of the same precision) and writes its device record into host memory `dst`.
// step_cap (optional) receives the job's default per-history step cap (derived from its
// domain, source and tables).
midsx_status pack_job(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                      midsx_tallies_h tallies, uint64_t seed, uint64_t first, uint64_t n, int precision,
                      void* dst, uint32_t* step_cap = nullptr);

// One batched launch over n_jobs records at `dev_jobs` with history offsets `dev_prefix`
// (n_jobs + 1 words, last = total) and history counters `dev_counter` (1 + n_jobs words: the
// launch's and each job's) zeroed here, on `s`.
// spectra: some job's tallies keep an incident-energy spectrum (tallies_spectra), which the
// lane-parking kernel scores.  step_cap: the launch's default per-history step cap (the
// largest of its jobs' pack_job caps), used when cfg.max_steps is 0.
midsx_status launch_packed(midsx_tables_h tables, const void* dev_jobs, int n_jobs,
                           const unsigned long long* dev_prefix, unsigned long long total,
                           unsigned long long* dev_counter, const midsx_run_config& cfg, cudaStream_t s,
                           bool spectra = false, uint32_t step_cap = 100000);
bool tallies_spectra(midsx_tallies_h t);

// Device bytes the tallies of (specs, dose_mode) take for a phantom of n_voxels voxels.
size_t tallies_footprint(size_t n_voxels, const midsx_tally_spec* specs, int n_specs, int dose_mode);

// Tallies whose storage comes from `pool`, allocated, filled and zeroed in order on `s`.
midsx_status tallies_create_async(midsx_phantom_h phantom, const midsx_tally_spec* specs, int n_specs,
                                  int dose_mode, cudaMemPool_t pool, cudaStream_t s, midsx_tallies_h* out);
// Returns their storage to the pool in order on `s` and deletes the handle.
void tallies_destroy_async(midsx_tallies_h t, cudaStream_t s);
void set_tallies_precision(midsx_tallies_h t, int precision);

// Phantom storage: the dense (material-index) voxel bytes, their size, and rebinding of the
// handle to storage the caller owns (nullptr = not resident).
size_t phantom_voxels(midsx_phantom_h p);
midsx_status phantom_download(midsx_phantom_h p, std::vector<uint8_t>& dense);
uint8_t* phantom_storage(midsx_phantom_h p);
void phantom_bind(midsx_phantom_h p, uint8_t* dense_ids);
// Frees the handle's own storage (synchronously) so that it can be rebound to pool memory.
void phantom_drop_storage(midsx_phantom_h p);
// Deletes the handle without touching its storage.
void phantom_delete_handle(midsx_phantom_h p);

int tables_device(midsx_tables_h t);

}  // namespace rt
}  // namespace midsx
