/*
 * midsx_gpu.h - C ABI of the GB300 photon-history transport path.
 *
 * This is the boundary between MIDSX's C++ API (ComputationalDomain, InteractionData,
 * PhotonSource, VolumeTally/SurfaceTally, PhysicsEngine, runSimulation) and the CUDA
 * kernels that replace the reference's OpenMP history loop.  Plain C types only: no
 * torch, no C++ classes, no exceptions.  Every function returns a midsx_status; the
 * C++ layer (include/MIDSX/Core) turns statuses into the reference's exception types.
 *
 * Reference interfaces replaced (paths inside the MIDSX repository):
 *   runSimulation(...)                 include/MIDSX/Core/run_simulation.h:24-27
 *   PhysicsEngine::transportPhoton     src/MIDSX/Core/physics_engine.cpp:17-79
 *   InteractionData / MaterialData     src/MIDSX/Core/interaction_data.cpp:3-73,
 *                                      src/MIDSX/Core/material_data.cpp:9-170
 *   ComputationalDomain::getVoxel      src/MIDSX/Core/computational_domain.cpp:16-31
 *   PhotonSource::generatePhoton       src/MIDSX/Core/source.cpp:150-155
 *   VolumeTally / SurfaceTally         src/MIDSX/Core/volume_tally.cpp, surface_tally.cpp
 *   Voxel dose (VectorValue per voxel) src/MIDSX/Core/physics_engine.cpp:160-168
 *
 * Units follow the reference: lengths in cm, energies in eV, cross sections in 1/cm.
 * Handles are not thread-safe; distinct handles may be used from distinct threads.
 * All device work is enqueued on the caller's CUDA stream (`stream`, a cudaStream_t
 * passed as void*; NULL = legacy default stream).
 */
#ifndef MIDSX_GPU_H
#define MIDSX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum midsx_status {
    MIDSX_OK = 0,
    MIDSX_INVALID_ARG = 1,   /* bad pointer, size, enum or geometry */
    MIDSX_OOM = 2,           /* host or device allocation failed */
    MIDSX_TIMEOUT = 3,       /* a host wait passed its deadline */
    MIDSX_STEP_CAP = 4,      /* some history hit the step or Compton-trial cap (run stats) */
    MIDSX_TABLE_RANGE = 5,   /* an energy outside the built tables was requested */
    MIDSX_CUDA_ERROR = 6,    /* a CUDA runtime call failed; see midsx_last_error() */
    MIDSX_NOT_FOUND = 7,     /* unknown material name or id */
    MIDSX_IO_ERROR = 8       /* data file missing or malformed */
} midsx_status;

typedef enum midsx_precision {
    MIDSX_PREC_FP64 = 0,   /* plain form: FP64 transport, FP64 atomic tallies */
    MIDSX_PREC_MIXED = 1   /* FP32 transport, 64-bit fixed-point integer tallies */
} midsx_precision;

/* Materials of one table set: the TG-195 Case 5 voxel volume of the reference's CT example
 * (cpp_simulations/CT_w_voxelized_solid) holds 20.  32 is also the width of a macro cell's
 * material mask.  The photon caches in shared memory grow with the count: launches whose
 * default block would not fit take a smaller one. */
#define MIDSX_MAX_MATERIALS 32
#define MIDSX_MAX_SPECTRUM_BINS 1024
#define MIDSX_MAX_TALLIES 64

/* ------------------------------------------------------------------ host tables --- */
/* A LogLogLinear table (src/MIDSX/Core/interpolators.cpp:33-76): node energies x (raw,
 * searched), log10 x and log10 y.  Fields are offsets into midsx_table_blob.data. */
typedef struct midsx_lin_table {
    int64_t x, lx, ly;
    int32_t n, reserved;
} midsx_lin_table;

/* A LogLogSpline (src/MIDSX/Core/interpolators.cpp:3-31): cubic B-spline in
 * u = (log10 E - lx_min) / (lx_max - lx_min) with knots knot_u[n_ctrl + degree + 1] and
 * control points ctrl[n_ctrl].  knot_e holds 10^(lx_min + u * (lx_max - lx_min)) for each
 * knot, so that the span is found by comparing raw energies. */
typedef struct midsx_spline_table {
    int64_t knot_e, knot_u, ctrl;
    int32_t n_ctrl, degree;
    double lx_min, lx_max;
} midsx_spline_table;

/* PENELOPE RITA tables of the Rayleigh cosine (src/MIDSX/Core/probability_dist.cpp:62-287).
 * Energy k has rows [idata[row_start + k], idata[row_start + k + 1]) of x, y, a, b. */
typedef struct midsx_rita_table {
    int64_t energy, log_energy, row_start, x, y, a, b;
    int32_t n_energy, n_rows;
} midsx_rita_table;

typedef struct midsx_material_table {
    int32_t id;              /* MIDSX material id (uint8 voxel value) */
    int32_t reserved;
    double density;          /* g/cm3 */
    midsx_lin_table total;   /* total macroscopic cross section, 1/cm */
    midsx_lin_table photo;   /* photoionisation, 1/cm */
    midsx_lin_table sfunc;   /* incoherent scattering function S(x) */
    midsx_lin_table ffactor; /* coherent form factor F(x) */
    midsx_spline_table coh;  /* coherent cross section, 1/cm */
    midsx_spline_table incoh;/* incoherent cross section, 1/cm */
    midsx_rita_table rita;   /* Rayleigh cosine sampler */
} midsx_material_table;

typedef struct midsx_table_blob {
    int32_t version;
    int32_t n_materials;
    double e_max;                 /* RITA tables cover energies up to this (eV) */
    midsx_lin_table majorant;     /* global majorant mu_max(E), 1/cm */
    midsx_material_table mat[MIDSX_MAX_MATERIALS];
    int64_t n_data;
    double* data;
    int64_t n_idata;
    int64_t* idata;
} midsx_table_blob;

/* Builds the FP64 tables of `n` materials (by MIDSX id, in this order = dense material
 * index 0..n-1) from the data files in `data_dir` (epdl_photon.bin, materials.txt,
 * elements.txt).  Replaces InteractionData(material_names) (src/MIDSX/Core/
 * interaction_data.cpp:3-73).  RITA tables are built for energy nodes up to the first
 * node >= e_max.  The blob is host memory; free it with midsx_tables_free. */
midsx_status midsx_tables_build(const char* data_dir, const int32_t* material_ids, int32_t n,
                                double e_max, midsx_table_blob** out);
void midsx_tables_free(midsx_table_blob* blob);

/* Material catalogue lookups (replace InteractionDataHelpers::convertMaterial*,
 * include/MIDSX/Core/material_helpers.h:110-121).  name_out receives up to cap bytes. */
midsx_status midsx_catalog_id(const char* data_dir, const char* name, int32_t* id_out);
midsx_status midsx_catalog_name(const char* data_dir, int32_t id, char* name_out, int32_t cap);

/* Composition of catalogue material `id` (MaterialProperties, src/MIDSX/Core/
 * material_properties.cpp:10-77): density (g/cm3) and up to `cap` (Z, weight fraction,
 * atomic weight g/mol) entries; *n receives the number of elements. */
midsx_status midsx_catalog_material(const char* data_dir, int32_t id, double* density, int32_t* n,
                                    int32_t* z, double* weight, double* atomic_weight, int32_t cap);

/* Rayleigh cosine of material `material` at energy E for the uniform y by the RITA inverse
 * of the built tables (ContinuousInversion::sample, src/MIDSX/Core/probability_dist.cpp:73-88). */
midsx_status midsx_tables_rita(const midsx_table_blob* blob, int32_t material, double energy, double y,
                               double* mu);

/* Host evaluation of the built tables, for checks and for the C++ API getters
 * (MaterialData::interpolate*, include/MIDSX/Core/material_data.h:95-143).
 * which: 0 total, 1 photo, 2 coherent (spline), 3 incoherent (spline), 4 S(x), 5 F(x),
 *        6 majorant (material ignored). */
midsx_status midsx_tables_eval(const midsx_table_blob* blob, int32_t material, int32_t which,
                               const double* x, double* y, int64_t n);

/* Mass energy-absorption coefficient mu_en/rho (cm2/g) of `material` at energies x (eV),
 * the coefficient MaterialData::interpolateMassEnergyAbsorptionCoefficient returns
 * (include/MIDSX/Core/material_data.h:143) for DerivedQuantity::getPrimaryAirKerma.  The
 * reference reads NIST tables from its database; here it follows from the built tables and
 * the transport's own deposition model: a photoelectric absorption deposits the photon's
 * energy, an incoherent scatter the electron's share of it (src/MIDSX/Core/
 * photon_interactions.cpp:43-141), so mu_en = mu_photo + mu_incoh * <1 - k'/k>, the mean over
 * the Klein-Nishina x S(x) angular distribution (Gauss-Legendre quadrature over cos theta).
 * Fluorescence escape and bremsstrahlung are not modelled by the transport and not here. */
midsx_status midsx_tables_mu_en(const midsx_table_blob* blob, int32_t material, const double* x, double* y,
                                int64_t n);

const char* midsx_status_string(midsx_status s);
const char* midsx_last_error(void);

/* ---------------------------------------------------------------- device handles --- */
typedef struct midsx_gpu_tables* midsx_tables_h;
typedef struct midsx_gpu_phantom* midsx_phantom_h;
typedef struct midsx_gpu_source* midsx_source_h;
typedef struct midsx_gpu_tallies* midsx_tallies_h;

/* Copies the FP64 tables to the device and derives the FP32 copies used by the mixed
 * path.  Replaces the per-thread table reads of the reference.  Synchronous. */
midsx_status midsx_gpu_tables_create(const midsx_table_blob* blob, midsx_tables_h* out);
midsx_status midsx_gpu_tables_destroy(midsx_tables_h t);

/* ComputationalDomain with one voxel grid (src/MIDSX/Core/computational_domain.cpp:16-31,
 * src/MIDSX/Core/voxel_grid.cpp:43-59,119-128): domain box [0, domain], background
 * material outside the grid, grid of dims[0]*dims[1]*dims[2] uint8 material ids,
 * x fastest, voxel size `spacing`, lower corner `origin`. */
typedef struct midsx_geometry_spec {
    double domain[3];
    double spacing[3];
    double origin[3];
    int32_t dims[3];
    int32_t background_id;   /* MIDSX material id of the background */
} midsx_geometry_spec;

/* Uploads voxel material ids (MIDSX ids, `ids` is host memory) and remaps them to the
 * dense material index of `tables` on the device.  Fails with MIDSX_NOT_FOUND if a voxel
 * id is not among the tables' materials.  Synchronous. */
midsx_status midsx_gpu_phantom_create(midsx_tables_h tables, const midsx_geometry_spec* geom,
                                      const uint8_t* ids, midsx_phantom_h* out);
midsx_status midsx_gpu_phantom_destroy(midsx_phantom_h p);

/* A domain with several voxel grids: ComputationalDomain's voxel_grids_
 * (src/MIDSX/Core/computational_domain.cpp:23-31, 92-104).  A point belongs to the first grid,
 * in the given order, whose closed box [origin, origin + dims * spacing] holds it, else to the
 * background material.  The phantom's voxels are numbered grid after grid (grid g's voxels
 * follow all voxels of grids 0..g-1), which is the layout of its dose tally. */
#define MIDSX_MAX_GRIDS 16
typedef struct midsx_grid_spec {
    double spacing[3];
    double origin[3];        /* lower corner in the domain (cm) */
    int32_t dims[3];
    int32_t reserved;
    const uint8_t* ids;      /* host memory: dims[0]*dims[1]*dims[2] MIDSX ids, x fastest */
} midsx_grid_spec;

midsx_status midsx_gpu_phantom_create_grids(midsx_tables_h tables, const double* domain, int32_t background_id,
                                            const midsx_grid_spec* grids, int32_t n_grids, midsx_phantom_h* out);

/* Rebuilds the phantom's macro cells (MIDSX_TRACK_MACRO_CELL) with edges of `edge` voxels, a
 * power of two in [1, 64]; the phantom is created with MIDSX_MACRO_CELL.  Synchronous; no run
 * may use the phantom meanwhile. */
midsx_status midsx_gpu_phantom_macro_cells(midsx_phantom_h p, int32_t edge);

/* PhotonSource (src/MIDSX/Core/source.cpp:44-155).  Geometry is a point (PointGeometry).
 * Directionality:
 *   BEAM:        a = pass-through point
 *   ISOTROPIC:   theta ~ U[0,pi], phi ~ U[0,2pi)  (the reference's definition)
 *   RECTANGLE:   a = corner, b = edge1, c = edge2 (edges orthogonal)
 *   DISC:        a = center, b = normal, radius; r ~ U[0,R], theta ~ U[0,2pi)
 * Spectrum: MONO (mono_energy) or POLY (n_bins energies with probabilities,
 * DiscreteInversion of src/MIDSX/Core/probability_dist.cpp:11-60). */
typedef enum midsx_direction_kind {
    MIDSX_DIR_BEAM = 0, MIDSX_DIR_ISOTROPIC = 1, MIDSX_DIR_RECTANGLE = 2, MIDSX_DIR_DISC = 3
} midsx_direction_kind;
typedef enum midsx_spectrum_kind { MIDSX_SPEC_MONO = 0, MIDSX_SPEC_POLY = 1 } midsx_spectrum_kind;

typedef struct midsx_source_spec {
    double position[3];
    int32_t direction_kind;
    int32_t spectrum_kind;
    double a[3], b[3], c[3];
    double radius;
    double mono_energy;
    int32_t n_bins;
    int32_t reserved;
    const double* bin_energy;    /* host pointers, n_bins each */
    const double* bin_prob;
} midsx_source_spec;

midsx_status midsx_gpu_source_create(const midsx_source_spec* spec, midsx_source_h* out);
midsx_status midsx_gpu_source_destroy(midsx_source_h s);

/* Tallies.  Scalar tallies hold, per scatter class (primary, single coherent, single
 * incoherent, multiple - src/MIDSX/Core/volume_quantity.cpp:53-67), count / sum / sum of
 * squares of each vector quantity and a count for each count quantity:
 *   surface (DISC: a = center, b = unit normal, radius; RECT: a = corner, b = edge1,
 *   c = edge2): IncidentEnergy[3x4], EntranceCosine[3x4], NumberOfPhotons[4]
 *   volume (AACUBOID: a = min corner, b = max corner):
 *   EnergyDeposition[3x4], IncidentEnergy[3x4], NumberOfPhotons[4], NumberOfInteractions[4]
 * BINNED_RECT is a RECT split into nu x nv bins (bin (i,j) equals a RectangularSurfaceTally
 * over that cell); per bin and class it holds the incident energy sum and photon count.
 * A DISC or RECT with n_energy > 0 also keeps an incident-energy spectrum: n_energy bins
 * [e_min + k e_width, e_min + (k+1) e_width) eV, per bin and class the number of crossings
 * and the sum of their entrance cosines.  It replaces the raw IncidentEnergy/EntranceCosine
 * vectors that DerivedQuantity::getPrimaryFluence scans (src/MIDSX/Core/derived_quantities.cpp:
 * 3-45): with bins centred on the source's energies every primary photon sits at a bin centre.
 * Batched launches (midsx_gpu_batch_*, the request server) with a spectrum tally run the
 * lane-parking scheduler with reference tracking (MIDSX_SCHED_POOL or another tracking is
 * refused with MIDSX_INVALID_ARG there); single runs take any scheduler and tracking.
 * The voxel dose tally (per grid voxel: deposit count, sum, sum of squares - the summary
 * of the reference's Voxel::dose VectorValue) is enabled by dose_mode. */
typedef enum midsx_tally_kind {
    MIDSX_TALLY_SURFACE_DISC = 1,
    MIDSX_TALLY_SURFACE_RECT = 2,
    MIDSX_TALLY_SURFACE_BINNED_RECT = 3,
    MIDSX_TALLY_VOLUME_AACUBOID = 4
} midsx_tally_kind;

typedef enum midsx_dose_mode {
    MIDSX_DOSE_OFF = 0,
    MIDSX_DOSE_SUM = 1,      /* energy sum per voxel only */
    MIDSX_DOSE_FULL = 2,     /* count, sum and sum of squares per voxel */
    MIDSX_DOSE_BATCHES = 3   /* FULL plus the batch-method variance of each voxel's sum */
} midsx_dose_mode;

/* Batch-method variance (MIDSX_DOSE_BATCHES).  The reference's per-voxel sigma
 * (src/MIDSX/Core/quantity.cpp:37-45) is the spread of single deposits, which is not the
 * uncertainty of a voxel's dose when a history deposits more than once in the voxel.  The batch
 * method is: a run of N histories is split into B batches of (nearly) N / B histories - disjoint
 * history-id ranges, so independent - and the variance of a voxel's total is B s^2, s^2 the
 * sample variance of its B batch sums.  Each midsx_gpu_run into such tallies closes one batch
 * at its end, or cfg->variance_batches batches when that is 2 or more (the run is split into
 * that many launches over consecutive history ranges); the batch sums are folded into a running
 * mean and sum of squared deviations per voxel (Welford) on the device.  Batched launches do not
 * close batches, and the request server does not take this mode.  The tallies take 16 more
 * bytes per voxel. */

#define MIDSX_MAX_ENERGY_BINS 65536

typedef struct midsx_tally_spec {
    int32_t kind;
    int32_t nu, nv;          /* bins of a BINNED_RECT along edge1, edge2 */
    int32_t n_energy;        /* DISC / RECT: incident-energy spectrum bins (0 = none) */
    double a[3], b[3], c[3];
    double radius;
    double e_min, e_width;   /* spectrum: lower edge and bin width (eV) */
} midsx_tally_spec;

#define MIDSX_SCALAR_SLOTS 40  /* doubles returned per scalar tally, see midsx_gpu_fetch_scalar */

midsx_status midsx_gpu_tallies_create(midsx_phantom_h phantom, const midsx_tally_spec* specs,
                                      int32_t n_specs, int32_t dose_mode, midsx_tallies_h* out);
midsx_status midsx_gpu_tallies_destroy(midsx_tallies_h t);
/* Zeroes every accumulator and the run statistics (enqueued on stream). */
midsx_status midsx_gpu_tallies_reset(midsx_tallies_h t, void* stream);

/* How a warp keeps its lanes busy; results do not depend on it (every history keeps its own
 * Philox stream).  LANES: each lane holds one history and parks it on an event until
 * `regroup` lanes wait.  POOL: each warp holds 64 photons in shared memory; a lane whose
 * photon needs an event takes another at once and the warp runs events 32 at a time. */
typedef enum midsx_scheduler {
    MIDSX_SCHED_DEFAULT = 0,
    MIDSX_SCHED_LANES = 1,
    MIDSX_SCHED_POOL = 2
} midsx_scheduler;

/* Flight sampling.  REFERENCE: Woodcock tracking against the global majorant everywhere
 * (src/MIDSX/Core/physics_engine.cpp:28-79, interaction_data.cpp:42-73).  BACKGROUND_FAST:
 * outside every voxel grid the medium is the background material alone, so its own
 * attenuation is an exact majorant there: a flight that starts in the background is sampled
 * with it and ends at a real collision, out of the domain, or - at the first grid it enters -
 * 1e-4 cm inside that grid, that last stretch against the global majorant (so that no flight
 * ends on a face where a tally plane may lie).
 * Unbiased (same distributions) but not the reference's random-number use, so results agree
 * with REFERENCE statistically, not history by history.  Photon-pool scheduler only. */
typedef enum midsx_tracking {
    MIDSX_TRACK_REFERENCE = 0,
    MIDSX_TRACK_BACKGROUND_FAST = 1,
    MIDSX_TRACK_MACRO_CELL = 2
} midsx_tracking;
/* MACRO_CELL adds local majorants inside the grids to BACKGROUND_FAST: every grid is split
 * into cells of MIDSX_MACRO_CELL^3 voxels (midsx_gpu_phantom_macro_cells changes the edge),
 * each with the set of materials it holds.  A flight inside a grid draws one optical depth
 * -ln U and spends it cell by cell along the ray, a cell's majorant being the largest
 * attenuation among its own materials at the photon's energy; where the depth runs out a
 * voxel is fetched and the collision is real with probability mu(voxel) / mu(cell).  A flight
 * that reaches its grid's face (or crosses 16 cells) goes on for 1e-4 cm past that face
 * against the global majorant and ends there unless it collides; the photon continues in its
 * next step.  Unbiased, statistically equal to REFERENCE; photon pool only.  Where grids
 * overlap, the cells of a later grid that meet an earlier grid's box take every material of
 * the tables (the first grid owns the overlap).  A phantom's cells are built on its first
 * MACRO_CELL run (or when it joins a batch or a server launch): that call synchronises the
 * device once. */
#define MIDSX_MACRO_CELL 8

typedef struct midsx_run_config {
    int32_t precision;           /* midsx_precision */
    int32_t max_steps;           /* per-history step cap (0 = derived per job: 16 crossings of the
                                    domain diagonal at the largest majorant between min(1 keV,
                                    the source's lowest energy) and the tables' e_max, at least
                                    100000; hits are counted and make the fetches report
                                    MIDSX_STEP_CAP) */
    int32_t max_compton_trials;  /* Kahn/S(x) rejection cap (0 = 100000) */
    int32_t block_size;          /* 0 = tuned default */
    int32_t blocks_per_sm;       /* 0 = tuned default */
    int32_t regroup;             /* events (real collisions, history starts) a warp gathers before
                                    it runs them together, 1..32 (0 = tuned default) */
    int32_t chunk;               /* lane-parking scheduler: history ids a lane reserves per fetch
                                    (0 = 1) */
    int32_t scheduler;           /* midsx_scheduler */
    int32_t tracking;            /* midsx_tracking */
    int32_t steps_per_pass;      /* batched photon-pool launches: Woodcock steps a lane takes
                                    between the warp's list bookkeeping, 1..4 (0 = tuned
                                    default: 2 for the FP32 form with reference tracking, the
                                    request server's launches included, else 1).  Single runs
                                    use the default, fixed at compile time. */
    int32_t variance_batches;    /* MIDSX_DOSE_BATCHES tallies: batches this run is split into
                                    (0 or 1: the run is one batch); at most 1024 */
    int32_t pass_repeats;        /* batched photon-pool launches: passes repeated without the
                                    pool's list bookkeeping while fewer than 16 lanes of a warp
                                    wait, 1..16 (0 = tuned default: 8 for the FP32 form with
                                    reference tracking, else 1).  Single runs use the default,
                                    fixed at compile time. */
    uint64_t seed;
    uint64_t first_history;      /* history ids [first, first + n) select Philox streams */
    uint64_t n_histories;
} midsx_run_config;

/* Transports n_histories photons and accumulates into `tallies` (asynchronous on stream).
 * Replaces runSimulation's history loop (src/MIDSX/Core/run_simulation.cpp:13-35).
 * Random numbers: Philox4x32-10 keyed by seed, one counter stream per history id, so a
 * run split into several calls over disjoint history ranges equals one call.  Every draw is
 * a 32-bit word: an interaction's draws (interaction type, samplers, azimuth) come four to a
 * block, starting a new block; a flight segment's Woodcock steps (free path, delta test) two
 * to a block of a counter range of their own.  Both precisions draw the same words. */
midsx_status midsx_gpu_run(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                           midsx_tallies_h tallies, const midsx_run_config* cfg, void* stream);

typedef struct midsx_run_stats {
    uint64_t histories;
    uint64_t steps;              /* Woodcock steps, including the final escaping one */
    uint64_t voxel_fetches;      /* steps that landed inside the voxel grid */
    uint64_t photo, coherent, incoherent;
    uint64_t compton_trials;
    uint64_t step_cap_hits, compton_cap_hits, edge_clamps;
    uint64_t tally_words;        /* tally accumulator updates (atomics issued) */
    double source_energy;        /* eV, sum over histories */
    double deposited_grid;       /* eV deposited in grid voxels */
    double deposited_background; /* eV deposited outside the grid */
    double escaped_energy;       /* eV carried out of the domain */
} midsx_run_stats;

/* The fetch functions synchronise `stream` and copy to host memory. */
midsx_status midsx_gpu_fetch_stats(midsx_tallies_h t, midsx_run_stats* out, void* stream);
/* Voxel dose: any of the three outputs may be NULL; each has n_voxels entries. */
midsx_status midsx_gpu_fetch_dose(midsx_tallies_h t, double* sum, double* sumsq, double* count,
                                  void* stream);
/* Batch-method variance of each voxel's dose sum (MIDSX_DOSE_BATCHES tallies, at least two
 * batches closed): var[n_voxels] = B / (B - 1) * sum_b (S_b - S / B)^2 over the B batch sums
 * S_b, eV^2; *n_batches (may be NULL) receives B.  Synchronises `stream`. */
midsx_status midsx_gpu_fetch_dose_variance(midsx_tallies_h t, double* var, int32_t* n_batches, void* stream);
/* Scalar tally `index` (0-based among the specs): MIDSX_SCALAR_SLOTS doubles, layout
 * [q][class][n, sum, sumsq] for the two vector quantities (24 values) followed by
 * [q][class] counts for the count quantities (8 values; surfaces use the first 4). */
midsx_status midsx_gpu_fetch_scalar(midsx_tallies_h t, int32_t index, double* out, void* stream);
/* Binned surface tally `index`: energy[nu*nv*4] (eV, [bin_v][bin_u][class]) and
 * count[nu*nv*4]. */
midsx_status midsx_gpu_fetch_binned(midsx_tallies_h t, int32_t index, double* energy,
                                    double* count, void* stream);
/* Incident-energy spectrum of surface tally `index` (n_energy > 0): count[n_energy*4] and
 * cosine[n_energy*4] ([energy bin][class]; either may be NULL). */
midsx_status midsx_gpu_fetch_spectrum(midsx_tallies_h t, int32_t index, double* count, double* cosine,
                                      void* stream);

/* One call from host memory to host memory: uploads the phantom ids, runs, and reads the
 * dose sum and statistics back; nothing stays on the device.  (The C++ PhysicsEngine keeps
 * its tables, phantom and tallies resident across runs instead.) */
midsx_status midsx_gpu_run_host(midsx_tables_h tables, const midsx_geometry_spec* geom,
                                const uint8_t* ids, const midsx_source_spec* source,
                                const midsx_tally_spec* specs, int32_t n_specs, int32_t dose_mode,
                                const midsx_run_config* cfg, double* dose_sum_out,
                                midsx_run_stats* stats_out);

/* Non-blocking CUDA stream helpers for C callers without the CUDA runtime headers. */
midsx_status midsx_gpu_stream_create(void** stream_out);
midsx_status midsx_gpu_stream_destroy(void* stream);
midsx_status midsx_gpu_stream_synchronize(void* stream);  /* with the MIDSX_WAIT_TIMEOUT_S deadline */

/* ---------------------------------------------------------------- batched launches --- */
/* Several independent simulations (different phantoms, sources, tallies, history counts and
 * seeds; one shared set of tables) transported by one persistent launch: history indices
 * over the concatenation of the jobs are handed out dynamically to the lanes, so jobs of
 * very different sizes finish together.  No reference counterpart (MIDSX runs one simulation
 * per runSimulation call); each job's results equal those of a single run of that job with
 * the same seed and history range (same Philox streams, integer tallies in the mixed form). */
#define MIDSX_MAX_BATCH_JOBS 64
typedef struct midsx_gpu_batch* midsx_batch_h;

typedef struct midsx_batch_job {
    midsx_phantom_h phantom;   /* created with the batch's tables */
    midsx_source_h source;
    midsx_tallies_h tallies;
    uint64_t seed;
    uint64_t first_history;    /* histories [first + e * n, first + (e + 1) * n) in epoch e */
    uint64_t n_histories;
} midsx_batch_job;

midsx_status midsx_gpu_batch_create(midsx_tables_h tables, const midsx_batch_job* jobs, int32_t n_jobs,
                                    midsx_batch_h* out);
midsx_status midsx_gpu_batch_destroy(midsx_batch_h b);
/* Large jobs: a job of at least `min_histories` histories runs as a single-job launch of its
 * own, ahead of the persistent launch of the others, on the same stream (and in the same
 * captured graph); results are unchanged (same history ids and streams).  A long job gains
 * nothing from sharing a launch - its own launch's tail is a small share of its time - and
 * runs faster in the single-job kernel, whose job lives in the constant bank instead of
 * shared memory.  0 restores the default, 16 loads of the GPU's resident photon slots
 * (28,672 histories per SM: 4.4e6 on 152 SMs); UINT64_MAX keeps every job in the persistent
 * launch.  Synchronous; call it outside a stream capture. */
midsx_status midsx_gpu_batch_set_own_launch(midsx_batch_h b, uint64_t min_histories);
/* One persistent launch over every job (cfg: precision and launch shape; its seed/first/n are
 * unused) - the large jobs first in launches of their own (midsx_gpu_batch_set_own_launch),
 * with the default single-job launch shape - then the batch's epoch advances so that the
 * next run transports the next histories. */
midsx_status midsx_gpu_batch_run(midsx_batch_h b, const midsx_run_config* cfg, void* stream);
/* Captures one run (counter reset, persistent launch, epoch advance) into a CUDA graph on
 * `stream`; midsx_gpu_batch_replay launches it.  Replays advance the epoch like runs. */
midsx_status midsx_gpu_batch_capture(midsx_batch_h b, const midsx_run_config* cfg, void* stream);
midsx_status midsx_gpu_batch_replay(midsx_batch_h b, void* stream);
/* Times candidate launch shapes (scheduler, block size, blocks per SM, regroup threshold, steps per
 * pass and pass repeats of the photon pool,
 * histories per fetch) on `trial_histories` histories spread over the jobs in proportion to
 * their sizes, returns the fastest in *best (precision as given) and its histories/s; the
 * trial runs leave the jobs' tallies reset and the epoch unchanged.  Synchronous. */
midsx_status midsx_gpu_batch_autotune(midsx_batch_h b, int32_t precision, uint64_t trial_histories,
                                      midsx_run_config* best, double* best_rate, void* stream);

/* ------------------------------------------------------------------ request server --- */
/* A request loop on one GPU with continuous batching.  No reference counterpart (MIDSX runs
 * one simulation per runSimulation call, src/MIDSX/Core/run_simulation.cpp:6-41).
 *  - The tables and every registered phantom stay on the device across requests; a phantom
 *    is evicted (least recently used, no request using it) only when an admission needs its
 *    memory, and uploaded again from the server's host copy when a request needs it.
 *  - A request names a registered phantom, a source handle (the caller's; it must outlive the
 *    request), tally specs, a dose mode, a seed, a history range and a precision.  It is
 *    admitted in arrival order when a job slot is free and its footprint (its tallies, plus
 *    its phantom when that is not resident) fits the HBM budget.
 *  - A scheduler thread keeps up to `launches_in_flight` batched launches queued on the GPU.
 *    Each launch splits `launch_histories` among the admitted requests with histories left:
 *    three quarters go to the requests with the fewest histories left, each taking all it
 *    needs in turn (shortest remaining first), and the rest is shared equally by the others,
 *    so a small request that arrives while large ones run finishes in its next launch and
 *    large requests keep progressing.
 *  - History ids, not launch boundaries, select the Philox streams: a request's results equal
 *    those of a single midsx_gpu_run of the same phantom, source, tallies, seed and range -
 *    bit for bit in the mixed form, to FP64 rounding order in the FP64 form.
 * Calls are thread-safe.  Times are seconds on the server's monotonic clock. */
typedef struct midsx_gpu_server* midsx_server_h;

typedef struct midsx_server_config {
    uint64_t hbm_budget_bytes;   /* phantoms + request tallies (0 = 90% of the free memory) */
    uint64_t launch_histories;   /* histories per batched launch (0 = 4,000,000) */
    int32_t max_active;          /* admitted requests, 1..64 (0 = 64) */
    int32_t launches_in_flight;  /* 1..4 (0 = 2) */
    midsx_run_config launch;     /* launch shape and caps; precision, seed and range unused */
} midsx_server_config;

typedef struct midsx_request {
    int32_t phantom;                 /* id from midsx_server_add_phantom */
    int32_t precision;               /* midsx_precision */
    int32_t dose_mode;               /* midsx_dose_mode */
    int32_t n_tallies;
    const midsx_tally_spec* tallies; /* copied at submission */
    midsx_source_h source;
    uint64_t seed;
    uint64_t first_history;
    uint64_t n_histories;
} midsx_request;

typedef enum midsx_request_state {
    MIDSX_REQ_QUEUED = 0,
    MIDSX_REQ_RUNNING = 1,
    MIDSX_REQ_DONE = 2,
    MIDSX_REQ_FAILED = 3
} midsx_request_state;

typedef struct midsx_request_info {
    int32_t state;               /* midsx_request_state */
    int32_t status;              /* midsx_status of a failed request */
    int32_t launches;            /* batched launches the request took part in */
    int32_t reserved;
    uint64_t histories_scheduled;
    uint64_t histories_done;
    uint64_t footprint_bytes;    /* device bytes charged at admission */
    double t_submit, t_admit, t_first_launch, t_done;  /* -1 until reached */
} midsx_request_info;

typedef struct midsx_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint64_t launches, histories;
    uint64_t budget_bytes, bytes_in_use, peak_bytes_in_use, resident_phantom_bytes;
    uint64_t phantom_uploads, phantom_evictions;
    int32_t queued, active, max_active_seen, reserved;
    double busy_seconds;         /* sum of launch durations (device events) */
} midsx_server_stats;

midsx_status midsx_server_create(midsx_tables_h tables, const midsx_server_config* cfg, midsx_server_h* out);
/* Stops the scheduler after the launches in flight, frees every request and phantom. */
midsx_status midsx_server_destroy(midsx_server_h s);
/* Registers a phantom with the tables its requests run with (NULL = the server's tables; the
 * tables must outlive the server); synchronous.  Each launch runs requests of one (tables,
 * precision) group: a phantom without lead need not take the lead-dominated majorant of
 * another request.  The server keeps a host copy of the dense voxel grid for uploads after
 * an eviction. */
midsx_status midsx_server_add_phantom(midsx_server_h s, midsx_tables_h tables, const midsx_geometry_spec* geom,
                                      const uint8_t* ids, int32_t* phantom_id);
midsx_status midsx_server_submit(midsx_server_h s, const midsx_request* r, uint64_t* request_id);
midsx_status midsx_server_poll(midsx_server_h s, uint64_t request_id, midsx_request_info* out);
/* Waits until the request is done or failed, or timeout_s passes (MIDSX_TIMEOUT). */
midsx_status midsx_server_wait(midsx_server_h s, uint64_t request_id, double timeout_s, midsx_request_info* out);
/* The tallies of a done request, to read with midsx_gpu_fetch_*; valid until release.  They
 * belong to the server: midsx_gpu_tallies_destroy refuses them. */
midsx_status midsx_server_tallies(midsx_server_h s, uint64_t request_id, midsx_tallies_h* out);
/* Returns a finished request's memory to the budget and forgets the request. */
midsx_status midsx_server_release(midsx_server_h s, uint64_t request_id);
midsx_status midsx_server_get_stats(midsx_server_h s, midsx_server_stats* out);
midsx_status midsx_server_now(midsx_server_h s, double* t);

/* ----------------------------------------------------------- sampler diagnostics --- */
/* Draw n samples of one sampler on the device with the transport kernel's own device
 * functions and Philox streams (history id = first + i, draw counter from 0).  Used by the
 * KS tests against the CPU samplers (reference check: tests/distributions/distributions.cpp).
 * kind: 0 Rayleigh cos(theta) (RITA), 1 Compton (out0 = cos theta, out1 = E'/E),
 *       2 free path in `material` at energy E (out0 = s, cm), 3 table index of the
 *       majorant / material total / S(x) / RITA lookups for the given energies (out0..). */
midsx_status midsx_gpu_sample(midsx_tables_h tables, int32_t precision, int32_t kind,
                              int32_t material, double energy, uint64_t seed, uint64_t first,
                              int64_t n, double* out0, double* out1);
/* Runs cfg->n_histories histories without tallies and writes, per history, the energy
 * deposited in grid voxels (hist_dep, host memory).  Used to compare trajectories history
 * by history with the CPU oracle driven by the same Philox streams.  Synchronous. */
midsx_status midsx_gpu_trace_deposits(midsx_tables_h tables, midsx_phantom_h phantom,
                                      midsx_source_h source, const midsx_run_config* cfg,
                                      double* hist_dep);
/* Allocation-free form of midsx_gpu_trace_deposits.  No counterpart in the reference: MIDSX
 * runs on the CPU and never faces this constraint.  It exists for callers that must not
 * allocate device memory while they run - a service that reserves its whole GPU memory budget
 * at start-up and treats any later allocation as a failure, a host application whose device
 * memory belongs to its own pool allocator, or a latency-critical loop that cannot afford the
 * device-wide synchronisation cudaFree implies.  It calls no cudaMalloc, cudaFree or other
 * allocating routine: its scratch (run counters and one double per history) is a fixed array
 * in the library's device code, 8 MiB plus 256 bytes on every GPU that loads the library,
 * held until the process exits.  Limits: at most 1,048,576 histories per call, and reference
 * tracking only (cfg->tracking = MIDSX_TRACK_REFERENCE: the other modes build macro cells,
 * which allocate); other requests fail with MIDSX_INVALID_ARG before any device work.  Each
 * call looks up the array's device address (cudaGetSymbolAddress) with the caller's device
 * current; the first call on a device also loads the library's device code there, so make
 * that first call before any stream capture.  All calls on a device share the one array,
 * which keeps the last call's contents (the call clears its counters itself), so calls whose
 * device work overlaps (different streams, different host threads) race on it; serialise
 * them.  Inputs and the host output hist_dep (n_histories doubles) are the caller's.  The
 * call is synchronous: it returns when the results are in hist_dep. */
midsx_status midsx_gpu_trace_deposits_noalloc(midsx_tables_h tables, midsx_phantom_h phantom,
                                              midsx_source_h source, const midsx_run_config* cfg,
                                              double* hist_dep, void* stream);
/* Table indices found on the device for energies e[n] (FP64 path, the bucketed searches the
 * transport kernel uses): idx[6*n] = majorant, material total, S(x) at x = e (as momentum
 * transfer), coherent-spline span, incoherent-spline span, RITA energy row.  An entry is
 * -1000 where the FP32 path's bucketed search at float(e) differs from a full search of the
 * FP32 node array (a self-check of the FP32 bucket tables). */
midsx_status midsx_gpu_table_index(midsx_tables_h tables, int32_t material, const double* e,
                                   int64_t n, int64_t* idx);

/* ------------------------------------------------------------ measurement probe --- */
/* Random 32 B sector probe (measurement only; no reference counterpart).  Enqueues on
 * `stream` about `requests` accesses to pseudo-random 32 B sectors of the device buffer
 * `buf`: mode 0 loads 4 bytes cached in L2 only, mode 1 adds 1 to a 64-bit word (a device
 * atomic whose result is unused).  These are the transport kernel's access forms (voxel-ID
 * fetches, tally read-modify-writes); timed over a footprint that fits the L2 and one that
 * does not, they give the L2 and HBM ceilings for that traffic.  `bytes`: a power of two from
 * 32 to 2^37; `buf` 32-byte aligned.  *issued receives the request count actually enqueued
 * (rounded up to fill the launch). */
midsx_status midsx_gpu_probe_sectors(void* buf, uint64_t bytes, int32_t mode, uint64_t requests,
                                     uint32_t seed, uint64_t* issued, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MIDSX_GPU_H */
