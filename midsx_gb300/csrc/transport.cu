// transport.cu - GB300 (sm_103a) kernels of MIDSX's photon-history loop and their C ABI.
//
// Each lane of a warp owns one history at a time (history ids strided by the number of
// threads) and starts its next history as soon as the current one ends; the history's
// state (position, direction, energy, scatter counts, Philox counter) lives in registers.
// A loop iteration is the reference's Woodcock step (src/MIDSX/Core/physics_engine.cpp:28-79):
// majorant free path, domain test, voxel material fetch, delta test; real collisions are
// parked and run by the warp together (kernel_body.cuh).  Tallies are scored per step instead
// of after the history (processTallies, physics_engine.cpp:192-210); all tallies are sums,
// so the order does not change the result.
//
// Energy-dependent table values (majorant and every material's total cross section)
// change only when the energy changes (Compton); they are evaluated once per energy and
// kept in shared memory per thread, so a step costs one log, one voxel load and two
// compares.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/midsx_gpu.h"
#include "device.cuh"
#include "tables_internal.h"

namespace midsx {

// ------------------------------------------------------------------- statistics ---
enum StatSlot {
    kStHistories = 0, kStSteps, kStFetches, kStPhoto, kStCoh, kStIncoh, kStTrials, kStStepCap,
    kStTrialCap, kStEdge, kStWords, kStSourceE, kStDepGrid, kStDepBg, kStEscE, kStRangeErr,
    kStNonFinite, kStCount
};
constexpr double kFxStat = 1024.0;  // fixed-point scale of statistics energies (per eV)

struct DevSource {
    double pos[3];
    int dir_kind, spec_kind;
    double a[3], b[3], c[3];  // beam point | rect corner,e1,e2 | disc center,u,v
    double radius, mono;
    int n_bins;
    const double* energy;
    const double* cdf;
    // FP32 copies for the mixed form
    float f_pos[3], f_a[3], f_b[3], f_c[3];
    float f_radius, f_mono;
    const float* f_energy;
    const float* f_cdf;
    // guide tables of the CDF search (kCdfGuide + 1 entries each, FP64 and FP32 CDF):
    // guide[k] = lower_bound(cdf, k / kCdfGuide), so lower_bound(cdf, u) for u in
    // [k / kCdfGuide, (k + 1) / kCdfGuide] lies in [guide[k], guide[k + 1]]
    const int* guide;
    const int* f_guide;
};
constexpr int kCdfGuide = 256;  // a power of two: k / kCdfGuide and u * kCdfGuide are exact

// Voxel grids after the first of a domain (ComputationalDomain::voxel_grids_[1..]).  The
// FP32 copies are what the mixed form computes with: float origin and extent, and the
// reciprocal of the float spacing, as make_geo derives them for the first grid.
struct DevGrid {
    double origin[3], spacing[3], ext[3];
    float f_origin[3], f_ext[3], f_ispc[3];
    int dims[3];
    int offset;       // number of the grid's first voxel in the phantom (ids and dose tally)
    int cdims[3];     // macro cells along each axis
    int cell_offset;  // number of the grid's first macro cell in the phantom
};

// Macro cells: 2^cell_shift voxels along each edge (fewer at the grid's far faces), a bit
// mask of the dense material indices present, cells x fastest, grid after grid.
constexpr int kCellShiftDefault = 3;
static_assert((1 << kCellShiftDefault) == MIDSX_MACRO_CELL, "MIDSX_MACRO_CELL is the default edge");

struct DevGeom {
    double domain[3], origin[3], spacing[3], ext[3];
    int dims[3];
    int background;
    const uint8_t* ids;     // every grid's dense material indices, grid after grid
    int n_grids;            // grids of the domain (1 = the first alone)
    const DevGrid* extra;   // n_grids - 1 further grids (device memory), in first-hit order
    const uint32_t* cells;  // macro-cell material masks of every grid
    int cdims[3];           // macro cells of the first grid along each axis
    int cell_shift;         // macro-cell edge = 2^cell_shift voxels
};

// One simulation: geometry, source, tallies and its history range [first, first + n) of its
// own Philox key.  A launch runs one job (by value in RunParams) or a batch (device array).
struct DevJob {
    DevGeom G;
    DevSource S;
    const DevTally* tallies;
    int n_tallies;
    int dose_stride;  // 0 = no dose tally, 1 = sum, 4 = count/sum/sumsq record
    unsigned long long* dose;
    unsigned long long* stats;  // kStCount counters of this job
    uint64_t seed, first, n;
    uint32_t step_cap;  // default per-history step cap of this job (derived_step_cap)
};

// Geometry of one job in the working precision (ComputationalDomain with one voxel grid).
template <typename R>
struct Geo {
    V3<R> dom, org, ext, spc, ispc;
    int nx, ny, nz, bg;
    const uint8_t* ids;
    int n_grids;           // grids of the domain; the first is held above
    const DevGrid* extra;  // the others, in first-hit order
};

template <typename R>
MIDSX_HD Geo<R> make_geo(const DevGeom& G) {
    Geo<R> g;
    g.dom = {R(G.domain[0]), R(G.domain[1]), R(G.domain[2])};
    g.org = {R(G.origin[0]), R(G.origin[1]), R(G.origin[2])};
    g.ext = {R(G.ext[0]), R(G.ext[1]), R(G.ext[2])};
    g.spc = {R(G.spacing[0]), R(G.spacing[1]), R(G.spacing[2])};
    g.ispc = {R(1) / g.spc.x, R(1) / g.spc.y, R(1) / g.spc.z};
    g.nx = G.dims[0];
    g.ny = G.dims[1];
    g.nz = G.dims[2];
    g.bg = G.background;
    g.ids = G.ids;
    g.n_grids = G.n_grids;
    g.extra = G.extra;
    return g;
}

constexpr int kMaxBatchJobs = 64;  // jobs of one batched launch (geometry staged in shared memory)
// scheduler of MIDSX_SCHED_DEFAULT: the photon pool (cone-beam dose workload, 1e7 histories:
// 2.65e8 histories/s against 2.27e8 for lane parking in FP32, 3.3e7 against 2.1e7 in FP64)
constexpr int kDefaultScheduler = MIDSX_SCHED_POOL;

struct RunParams {
    DevTables T;
    DevJob job0;                            // single-job launch
    const DevJob* jobs;                     // batched launch: n_jobs descriptors (device)
    int n_jobs;
    const unsigned long long* prefix;       // batched launch: n_jobs + 1 history offsets (device)
    unsigned long long* counter;            // histories handed out so far (zeroed before launch)
    unsigned long long* job_counters;       // batched photon pool: each job's own (counter + 1 ...)
    unsigned long long total;               // histories of this launch
    const unsigned long long* epoch;        // optional: history ids advance by n per epoch
    int max_steps, max_trials;
    int tracking;   // midsx_tracking
    int regroup;    // lanes of a warp that wait for an event before the warp runs the events
    int chunk;      // histories a lane reserves per fetch
    double* trace;  // optional (single job): energy deposited in grid voxels per history
    int spectra;    // some tally of the launch keeps an incident-energy spectrum
    int steps_per_pass;  // photon pool: Woodcock steps per pass of the warp loop
    int pass_repeats;    // photon pool, batched: passes repeated between list bookkeeping
    int server;          // launched by the request server (its own steps_per_pass default)
    uint32_t round_keys[20];  // single-job launch: Philox key schedule of job0.seed
    Geo<float> geo_f;         // single-job launch: job0's geometry in either precision,
    Geo<double> geo_d;        // read by the kernels from the constant bank
};

__device__ __forceinline__ const Geo<float>& job0_geo(const RunParams& P, float) { return P.geo_f; }
__device__ __forceinline__ const Geo<double>& job0_geo(const RunParams& P, double) { return P.geo_d; }

// Default Woodcock steps per pass of the photon-pool loop.  FP32 reference tracking: 2
// against 1 measured +5.5 to +10 % on the cone-beam dose workload and +6 % on the 64-job
// batch (3, 4 and 6 were slower than 1); a pass of two steps also computes one Philox block
// for both (HistoryRng's step stream), which made two steps pay for the request server's
// short mixed launches too (+11 % histories/s at 200 requests/s, lower p50 and p99 for every
// class; with one step per pass and one block per step they had measured -10 %).  The FP64
// form (-2.3 % with 2) and the opt-in modes whose steps are long (a background flight, a
// cell walk; -8 to -9 % with 2) keep one.  Batched launches: passes repeated between the
// pool's list bookkeeping (pass_repeats in kernel_pool.cuh; the server's launches take one
// repeat); single-job launches fix both at compile time.
inline int default_pass_repeats(int precision, int tracking, bool server) {
    return precision == MIDSX_PREC_MIXED && tracking == MIDSX_TRACK_REFERENCE && !server ? 8 : 1;
}
inline int default_steps_per_pass(int precision, int tracking, bool server) {
    (void)server;
    return precision == MIDSX_PREC_MIXED && tracking == MIDSX_TRACK_REFERENCE ? 2 : 1;
}

// -------------------------------------------------------------------- atomics ---
template <bool MX>
struct Acc;

template <>
struct Acc<false> {  // FP64 plain form
    __device__ static void energy(unsigned long long* p, double v) { atomicAdd(reinterpret_cast<double*>(p), v); }
    __device__ static void energy2(unsigned long long* p, double v) {
        atomicAdd(reinterpret_cast<double*>(p), v * v);
    }
    __device__ static void cosine(unsigned long long* p, double v) { atomicAdd(reinterpret_cast<double*>(p), v); }
    __device__ static void cosine2(unsigned long long* p, double v) {
        atomicAdd(reinterpret_cast<double*>(p), v * v);
    }
};

// 64-bit fixed point, exact and order independent.  Values arrive in FP32 and are scaled by
// powers of two and converted with 32-bit conversions (no double-precision instruction):
// energies up to kMixedMaxEnergy eV (energy^2 / 16 stays below 2^32), cosines in [0, 1].
constexpr double kMixedMaxEnergy = 262144.0;
template <>
struct Acc<true> {
    __device__ static void energy(unsigned long long* p, float v) {
        atomicAdd(p, (unsigned long long)__float2uint_rn(v * float(kFxEnergy)));
    }
    __device__ static void energy2(unsigned long long* p, float v) {
        atomicAdd(p, (unsigned long long)__float2uint_rn(v * v * float(kFxEnergy2)));
    }
    __device__ static void cosine(unsigned long long* p, float v) {
        atomicAdd(p, (unsigned long long)__float2uint_rn(v * float(kFxCosine)));
    }
    __device__ static void cosine2(unsigned long long* p, float v) {
        atomicAdd(p, (unsigned long long)__float2uint_rn(v * v * float(kFxCosine)));
    }
};

__device__ __forceinline__ void count1(unsigned long long* p) { atomicAdd(p, 1ull); }

// ------------------------------------------------------------------ tally scoring ---
// VectorVolumeQuantity / VectorSurfaceQuantity::measure: skip zero values, else add
// (count, sum, sum of squares) to the class.
template <typename R, bool MX>
__device__ __forceinline__ void vec_energy(unsigned long long* acc, int q, int cls, R v, uint32_t& words) {
    if (v == R(0)) return;
    unsigned long long* s = acc + q * 12 + cls * 3;
    count1(s);
    Acc<MX>::energy(s + 1, v);
    Acc<MX>::energy2(s + 2, v);
    ++words;  // one accumulator record (count, sum, sum of squares) updated
}

template <typename R, bool MX>
__device__ __forceinline__ void vec_cosine(unsigned long long* acc, int q, int cls, R v, uint32_t& words) {
    if (v == R(0)) return;
    unsigned long long* s = acc + q * 12 + cls * 3;
    count1(s);
    Acc<MX>::cosine(s + 1, v);
    Acc<MX>::cosine2(s + 2, v);
    ++words;
}

// One step segment [p0, p0 + s d) against every scalar/binned tally.  SPEC: also the
// incident-energy spectra - compiled into the lane-parking kernel only, which runs every
// launch with a spectrum tally: in the photon-pool kernel the spectrum code, inline or out of
// line, cost the cone-beam dose workload (no tally at all) 5 %.
// cls0: class of the photon at the step start (surface quantities use initial_photon);
// cls1: class of final_photon (post-interaction counts if the step interacted, else
// a default Photon = primary), used by volume quantities.
template <typename R, bool MX, bool SPEC = true>
__device__ __forceinline__ void score_tallies(const DevTally* tallies, int n_tallies, const V3<R>& p0, const V3<R>& d,
                                           R s, R E, int cls0, int cls1, bool interact, R dep, uint32_t& words) {
    for (int ti = 0; ti < n_tallies; ++ti) {
        const DevTally& T = tallies[ti];
        const int kind = T.kind;
        if (kind == MIDSX_TALLY_VOLUME_AACUBOID) {
            // AACuboidVolumeTally::determineVolumeTraversal (volume_tally.cpp:38-91)
            R lo[3], hi[3];
            const R pp[3] = {p0.x, p0.y, p0.z};
            const R dd[3] = {d.x, d.y, d.z};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (fabs_(dd[i]) < R(kEps)) {
                    lo[i] = -R(INFINITY);
                    hi[i] = R(INFINITY);
                    continue;
                }
                lo[i] = (pickr<R>(T.a[i], T.fa[i]) - pp[i]) / dd[i];
                hi[i] = (pickr<R>(T.b[i], T.fb[i]) - pp[i]) / dd[i];
                if (lo[i] > hi[i]) {
                    R tmp = lo[i];
                    lo[i] = hi[i];
                    hi[i] = tmp;
                }
            }
            R enter = lo[0] > lo[1] ? lo[0] : lo[1];
            enter = enter > lo[2] ? enter : lo[2];
            R exit_ = hi[0] < hi[1] ? hi[0] : hi[1];
            exit_ = exit_ < hi[2] ? exit_ : hi[2];
            if (enter > exit_ || exit_ < R(0) || enter > s) continue;  // MISSES
            bool counted;
            R e_dep;
            if (enter <= R(0)) {
                counted = true;
                e_dep = (exit_ >= s) ? dep : R(0);  // STAYS keeps the deposit, EXITS zeroes it
            } else {
                counted = false;
                e_dep = (exit_ < s) ? R(0) : dep;   // PASSES_THROUGH zeroes, LANDS_INSIDE keeps
            }
            unsigned long long* acc = T.acc;
            vec_energy<R, MX>(acc, 0, cls1, e_dep, words);
            if (!counted) {
                vec_energy<R, MX>(acc, 1, cls1, E, words);
                count1(acc + 24 + cls1);
                ++words;
            }
            if (interact) {
                count1(acc + 28 + cls1);
                ++words;
            }
            continue;
        }
        // SurfaceTally::willPassThrough (surface_tally.cpp:16-34)
        V3<R> nrm = {pickr<R>(T.norm[0], T.fnorm[0]), pickr<R>(T.norm[1], T.fnorm[1]), pickr<R>(T.norm[2], T.fnorm[2])};
        R ec = dot(d, nrm);
        if (fabs_(ec) < R(kEps) || ec < R(0)) continue;
        V3<R> a = {pickr<R>(T.a[0], T.fa[0]), pickr<R>(T.a[1], T.fa[1]), pickr<R>(T.a[2], T.fa[2])};
        V3<R> w = {a.x - p0.x, a.y - p0.y, a.z - p0.z};
        R t = dot(w, nrm) / ec;
        if (t > s || t < R(0)) continue;
        V3<R> ip = {p0.x + t * d.x, p0.y + t * d.y, p0.z + t * d.z};
        V3<R> rel = {ip.x - a.x, ip.y - a.y, ip.z - a.z};
        if (kind == MIDSX_TALLY_SURFACE_DISC) {
            if (sqrt_(dot(rel, rel)) > pickr<R>(T.radius, T.fradius)) continue;
        } else {
            V3<R> e1 = {pickr<R>(T.b[0], T.fb[0]), pickr<R>(T.b[1], T.fb[1]), pickr<R>(T.b[2], T.fb[2])};
            V3<R> e2 = {pickr<R>(T.c[0], T.fc[0]), pickr<R>(T.c[1], T.fc[1]), pickr<R>(T.c[2], T.fc[2])};
            R u = dot(e1, rel), v = dot(e2, rel);
            if (u < R(0) || u > pickr<R>(T.e1e1, T.fe1e1) || v < R(0) || v > pickr<R>(T.e2e2, T.fe2e2)) continue;
            if (kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
                int iu = int(u / pickr<R>(T.e1e1, T.fe1e1) * R(T.nu));
                int iv = int(v / pickr<R>(T.e2e2, T.fe2e2) * R(T.nv));
                iu = iu >= T.nu ? T.nu - 1 : iu;
                iv = iv >= T.nv ? T.nv - 1 : iv;
                unsigned long long* bin = T.acc + (size_t(iv) * T.nu + iu) * 8 + cls0 * 2;
                Acc<MX>::energy(bin, E);
                count1(bin + 1);
                ++words;
                continue;
            }
        }
        unsigned long long* acc = T.acc;
        vec_energy<R, MX>(acc, 0, cls0, E, words);
        vec_cosine<R, MX>(acc, 1, cls0, ec, words);
        count1(acc + 24 + cls0);
        ++words;
        if constexpr (SPEC) {
            if (T.n_energy > 0) {
                // incident-energy spectrum: [crossings, entrance-cosine sum] per bin and class
                const int kb = energy_bin<R>(T, E);
                if (kb >= 0) {
                    unsigned long long* sp = acc + MIDSX_SCALAR_SLOTS + (size_t(kb) * 4 + cls0) * 2;
                    count1(sp);
                    Acc<MX>::cosine(sp + 1, ec);
                    ++words;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ source sampling ---
// PhotonSource::generatePhoton: position (PointGeometry), direction, energy, in that order.
// The FP32 form reads the source's FP32 copies (no double-precision instruction on the path).
template <typename R>
__device__ __forceinline__ V3<R> src3(const double* d, const float* f) {
    if constexpr (sizeof(R) == 8)
        return {d[0], d[1], d[2]};
    else
        return {f[0], f[1], f[2]};
}

template <typename R>
__device__ __forceinline__ void sample_source(const DevSource& S, HistoryRng& rng, V3<R>& pos, V3<R>& dir, R& E) {
    pos = src3<R>(S.pos, S.f_pos);
    const V3<R> A = src3<R>(S.a, S.f_a), B = src3<R>(S.b, S.f_b), Cc = src3<R>(S.c, S.f_c);
    V3<R> d;
    switch (S.dir_kind) {
        case MIDSX_DIR_BEAM:
            d = {A.x - pos.x, A.y - pos.y, A.z - pos.z};
            break;
        case MIDSX_DIR_ISOTROPIC: {
            R theta = R(kPi) * uniform<R>(rng);
            R phi = R(2 * kPi) * uniform<R>(rng);
            R st, ct, sp, cp;
            sincos_(theta, &st, &ct);
            sincos_(phi, &sp, &cp);
            d = {st * cp, st * sp, ct};
            break;
        }
        case MIDSX_DIR_RECTANGLE: {
            R a1 = uniform<R>(rng);
            R a2 = uniform<R>(rng);
            d = {A.x + a1 * B.x + a2 * Cc.x - pos.x, A.y + a1 * B.y + a2 * Cc.y - pos.y,
                 A.z + a1 * B.z + a2 * Cc.z - pos.z};
            break;
        }
        default: {  // DISC
            R theta = R(2 * kPi) * uniform<R>(rng);
            R radius;
            if constexpr (sizeof(R) == 8)
                radius = S.radius;
            else
                radius = S.f_radius;
            R r = radius * uniform<R>(rng);
            R st, ct;
            sincos_(theta, &st, &ct);
            d = {A.x + r * (B.x * ct + Cc.x * st) - pos.x, A.y + r * (B.y * ct + Cc.y * st) - pos.y,
                 A.z + r * (B.z * ct + Cc.z * st) - pos.z};
            break;
        }
    }
    R nd = sqrt_(dot(d, d));
    const R ind = R(1) / nd;  // one division
    dir = {d.x * ind, d.y * ind, d.z * ind};
    if (S.spec_kind == MIDSX_SPEC_MONO) {
        if constexpr (sizeof(R) == 8)
            E = S.mono;
        else
            E = S.f_mono;
    } else {
        // DiscreteInversion::sample: energy[lower_bound(cdf, U)], clamped to the last bin; the
        // guide table narrows the search to the nodes between two guide points (same index)
        const R u = uniform<R>(rng);
        const int g = min(int(u * R(kCdfGuide)), kCdfGuide - 1);
        int idx;
        if constexpr (sizeof(R) == 8)
            idx = lower_index(S.cdf, S.guide[g], S.guide[g + 1], u);
        else
            idx = lower_index(S.f_cdf, S.f_guide[g], S.f_guide[g + 1], u);
        if (idx >= S.n_bins) idx = S.n_bins - 1;
        if constexpr (sizeof(R) == 8)
            E = S.energy[idx];
        else
            E = S.f_energy[idx];
    }
}

// -------------------------------------------------------------------- the kernel ---
#include "kernel_body.cuh"
#include "tally_warp.cuh"
#include "kernel_pool.cuh"
// ------------------------------------------------------------- diagnostics kernels ---
template <typename R>
__global__ void sample_kernel(const DevTables T, int kind, int m, double energy, uint64_t seed, uint64_t first,
                              int64_t n, double* out0, double* out1) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HistoryRng rng;
    rng.init(seed, first + uint64_t(i));
    const R E = R(energy);
    const DevMaterial& Mt = T.mat[m];
    if (kind == 0) {
        R mu = R(0);
        bool ok = rita_sample<R>(T, Mt.rita, E, uniform<R>(rng), mu);
        out0[i] = ok ? double(mu) : NAN;
    } else if (kind == 1) {
        const R alpha = R(T.alpha);
        const R k = E / R(kMec2);
        const R r1p = (R(1) + R(2) * k) / (R(9) + R(2) * k);
        const R s_max = lin_lookup<R>(T, Mt.sfunc, alpha * k * sqrt_(R(2)));
        R mu = R(1), kp = k;
        for (int trial = 0; trial < 100000; ++trial) {
            R r1 = uniform<R>(rng), r2 = uniform<R>(rng), r3 = uniform<R>(rng);
            R chi;
            if (r1 <= r1p) {
                chi = R(1) + R(2) * k * r2;
                if (!(r3 <= R(4) * (R(1) / chi - R(1) / (chi * chi)))) continue;
            } else {
                chi = (R(1) + R(2) * k) / (R(1) + R(2) * k * r2);
                R tt = R(1) / k - chi / k + R(1);
                if (!(R(2) * r3 <= tt * tt + R(1) / chi)) continue;
            }
            kp = k / chi;
            mu = R(1) + R(1) / k - R(1) / kp;
            R x = alpha * k * sqrt_(R(1) - mu);
            if (uniform<R>(rng) <= lin_lookup<R>(T, Mt.sfunc, x) / s_max) break;
        }
        out0[i] = double(mu);
        out1[i] = double(kp / k);
    } else {
        R mu_max = lin_lookup<R>(T, T.majorant, E);
        out0[i] = double(-log_(uniform<R>(rng)) / mu_max);
    }
}

__global__ void index_kernel(const DevTables T, int m, const double* e, int64_t n, int64_t* idx) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double E = e[i];
    const DevMaterial& Mt = T.mat[m];
    // the indices the transport kernel uses (bucketed searches, FP64)
    long long r[6] = {lin_index_bk<double>(T, T.majorant, E), lin_index_bk<double>(T, Mt.total, E),
                      lin_index_bk<double>(T, Mt.sfunc, E), spline_span_bk<double>(T, Mt.coh, E),
                      spline_span_bk<double>(T, Mt.incoh, E), rita_row_bk<double>(T, Mt.rita, E)};
    // the FP32 bucketed searches must equal full searches of the FP32 node arrays
    const float Ef = float(E);
    const float* F = T.f;
    const long long f_bk[6] = {lin_index_bk<float>(T, T.majorant, Ef), lin_index_bk<float>(T, Mt.total, Ef),
                               lin_index_bk<float>(T, Mt.sfunc, Ef), spline_span_bk<float>(T, Mt.coh, Ef),
                               spline_span_bk<float>(T, Mt.incoh, Ef), rita_row_bk<float>(T, Mt.rita, Ef)};
    const long long f_full[6] = {lin_index(F + T.majorant.x, T.majorant.n, Ef), lin_index(F + Mt.total.x, Mt.total.n, Ef),
                                 lin_index(F + Mt.sfunc.x, Mt.sfunc.n, Ef),
                                 spline_span(F + Mt.coh.knot_e, Mt.coh.n_ctrl, Mt.coh.degree, Ef),
                                 spline_span(F + Mt.incoh.knot_e, Mt.incoh.n_ctrl, Mt.incoh.degree, Ef),
                                 lower_index(F + Mt.rita.energy, 0, Mt.rita.n_energy, Ef) - 1};
    for (int k = 0; k < 6; ++k) idx[6 * i + k] = (f_bk[k] == f_full[k]) ? r[k] : -1000;
}

__global__ void remap_kernel(const uint8_t* in, uint8_t* out, const uint8_t* lut, size_t n, int* bad) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (; i < n; i += stride) {
        uint8_t v = lut[in[i]];
        if (v == 0xFF) {
            atomicExch(bad, 1);
            v = 0;
        }
        out[i] = v;
    }
}

// Material mask of each macro cell of one grid: OR of 1 << material over the cell's voxels.
__global__ void cell_mask_kernel(const uint8_t* ids, int nx, int ny, int nz, int cnx, int cny, int cnz, int shift,
                                 uint32_t* cells) {
    const size_t n = size_t(cnx) * cny * cnz;
    const int edge = 1 << shift;
    for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
        const int cx = int(c % cnx), cy = int((c / cnx) % cny), cz = int(c / (size_t(cnx) * cny));
        const int x0 = cx << shift, y0 = cy << shift, z0 = cz << shift;
        const int x1 = min(x0 + edge, nx), y1 = min(y0 + edge, ny), z1 = min(z0 + edge, nz);
        uint32_t m = 0;
        for (int z = z0; z < z1; ++z)
            for (int y = y0; y < y1; ++y) {
                const uint8_t* row = ids + (size_t(z) * ny + y) * nx;
                for (int x = x0; x < x1; ++x) m |= 1u << (row[x] & 31);
            }
        cells[c] = m;
    }
}

// ORs `bits` into the cells [lo, hi] (inclusive) of one grid's cell array.
__global__ void cell_or_box_kernel(uint32_t* cells, int cnx, int cny, int lx, int ly, int lz, int hx, int hy, int hz,
                                   uint32_t bits) {
    const int wx = hx - lx + 1, wy = hy - ly + 1, wz = hz - lz + 1;
    const size_t n = size_t(wx) * wy * wz;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const int x = lx + int(i % wx), y = ly + int((i / wx) % wy), z = lz + int(i / (size_t(wx) * wy));
        cells[(size_t(z) * cny + y) * cnx + x] |= bits;
    }
}

__global__ void f64_to_f32_kernel(const double* in, float* out, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = float(in[i]);
}

}  // namespace midsx

// =========================================================================== C ABI ===
using namespace midsx;

struct midsx_gpu_tables {
    DevTables T;
    double* d = nullptr;
    float* f = nullptr;
    float* fs = nullptr;  // FP32 LogLogLinear slopes (computed in FP64), same offsets as d
    double* ds = nullptr;  // the FP64 slopes themselves
    int* rows = nullptr;
    int* bk = nullptr;
    int32_t ids[MIDSX_MAX_MATERIALS];
    int device = 0;
    int sm_count = 0;
    size_t max_smem = 0;  // opt-in shared memory of one block
    std::vector<double> maj_x, maj_mu;  // host copy of the majorant's nodes (eV, 1/cm)
};

struct midsx_gpu_phantom {
    DevGeom G;
    uint8_t* ids = nullptr;
    size_t n_voxels = 0;                       // all grids
    DevGrid* extra = nullptr;                  // grids after the first (device)
    uint32_t* cells = nullptr;                 // macro-cell material masks (device), built on first use
    int cell_shift = 3;                        // their edge, 2^cell_shift voxels
    std::vector<midsx_grid_spec> grids;        // every grid's geometry (ids pointers cleared)
    std::vector<DevGrid> host_extra;           // host copy of `extra`
    const midsx_gpu_tables* tables = nullptr;  // the tables its dense material indices refer to
};

struct midsx_gpu_source {
    DevSource S;
    double* buf = nullptr;
    double max_energy = 0;
    double min_energy = 0;  // lowest energy the source emits (a bin of non-zero weight)
};

struct midsx_gpu_tallies {
    size_t n_voxels = 0;
    int dose_mode = 0;
    int dose_stride = 0;
    unsigned long long* dose = nullptr;
    std::vector<DevTally> host_specs;
    DevTally* specs = nullptr;
    unsigned long long* acc = nullptr;  // all scalar/binned accumulators
    size_t acc_words = 0;
    unsigned long long* stats = nullptr;
    int precision = -1;   // precision of the accumulated contents, -1 = empty
    bool pooled = false;  // one pool block starting at `stats`, owned by a request server
    bool spectra = false; // some surface tally keeps an incident-energy spectrum
    // MIDSX_DOSE_BATCHES: per voxel the running mean and sum of squared deviations of the
    // batch sums (Welford); each dose record's fourth word holds the sum at the last close
    double* batch = nullptr;
    int batches_closed = 0;
};

namespace {

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

// Runs `f` when the scope ends unless release() was called: the early error returns of a
// create function free what it has allocated so far, and scratch buffers are freed on every
// return.
template <typename F>
struct ScopeExit {
    F f;
    bool armed = true;
    ~ScopeExit() {
        if (armed) f();
    }
    void release() { armed = false; }
};
template <typename F>
ScopeExit<F> scope_exit(F f) {
    return ScopeExit<F>{f};
}

#define CUDA_TRY(call)                                          \
    do {                                                        \
        if (!cuda_ok((call), #call)) return MIDSX_CUDA_ERROR;   \
    } while (0)

// Waits for `stream` with a deadline (MIDSX_WAIT_TIMEOUT_S, default 1800 s) by polling, so
// that a host never blocks forever on a device that stopped answering.
midsx_status wait_stream(void* stream) {
    double limit = 1800.0;
    if (const char* env = std::getenv("MIDSX_WAIT_TIMEOUT_S")) limit = std::atof(env);
    auto t0 = std::chrono::steady_clock::now();
    int spins = 0;
    for (;;) {
        cudaError_t e = cudaStreamQuery(static_cast<cudaStream_t>(stream));
        if (e == cudaSuccess) return MIDSX_OK;
        if (e != cudaErrorNotReady) {
            cuda_ok(e, "cudaStreamQuery");
            return MIDSX_CUDA_ERROR;
        }
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > limit) {
            set_last_error("stream wait exceeded deadline");
            return MIDSX_TIMEOUT;
        }
        if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

void fill_lin(DevLin& o, const midsx_lin_table& t) {
    o.x = int(t.x);
    o.lx = int(t.lx);
    o.ly = int(t.ly);
    o.n = t.n;
}
void fill_spline(DevSpline& o, const midsx_spline_table& t) {
    o.knot_e = int(t.knot_e);
    o.knot_u = int(t.knot_u);
    o.ctrl = int(t.ctrl);
    o.n_ctrl = t.n_ctrl;
    o.degree = t.degree;
    o.lx_min = t.lx_min;
    o.lx_max = t.lx_max;
    o.f_lx_min = float(t.lx_min);
    o.f_lx_max = float(t.lx_max);
}

constexpr int kScalarWords = MIDSX_SCALAR_SLOTS;

// Bucket tables of the searched node arrays (lookup.h).  Energies: binade slices of 1/128
// octave from 128 eV to 256 keV; momentum transfer: 1/64 octave from 2^-8 to 2^5 1/A.
// Queries outside a window fall in its first or last slice, which still gives the exact
// index (over a longer search range).
constexpr int kBucketBits[2] = {7, 6};
constexpr double kBucketLo[2] = {128.0, 1.0 / 256.0};
constexpr int kBucketOctaves[2] = {11, 13};

double slice_lo_d(long long key, int kbits) {
    unsigned long long bits = (unsigned long long)key << (52 - kbits);
    double v;
    std::memcpy(&v, &bits, 8);
    return v;
}
float slice_lo_f(long long key, int kbits) {
    unsigned int bits = (unsigned int)((unsigned long long)key << (23 - kbits));
    float v;
    std::memcpy(&v, &bits, 4);
    return v;
}

struct BucketBuilder {
    std::vector<int> data;
    BucketSpec spec[2][2];
    BucketBuilder() {
        for (int k = 0; k < 2; ++k) {
            int nb = kBucketOctaves[k] << kBucketBits[k];
            spec[k][0] = {kBucketBits[k], bucket_key(kBucketLo[k], kBucketBits[k]), nb};
            spec[k][1] = {kBucketBits[k], bucket_key(float(kBucketLo[k]), kBucketBits[k]), nb};
        }
    }
    // mode 0: upper_bound over [lo, hi) (lo = 0, hi = n for LogLogLinear; the knot range for
    // a spline span); mode 1: lower_bound over [0, n) (RITA energies).
    template <typename R>
    int add(const double* x64, int n, int kind, int mode, int lo, int hi) {
        const BucketSpec& s = spec[kind][sizeof(R) == 8 ? 0 : 1];
        std::vector<R> x;
        x.resize(size_t(n));
        for (int i = 0; i < n; ++i) x[size_t(i)] = R(x64[i]);
        int off = int(data.size());
        data.push_back(lo);
        for (int b = 1; b < s.nb; ++b) {
            R q = (sizeof(R) == 8) ? R(slice_lo_d(s.base + b, s.kbits)) : R(slice_lo_f(s.base + b, s.kbits));
            int r = mode == 0 ? int(std::upper_bound(x.begin(), x.end(), q) - x.begin())
                              : int(std::lower_bound(x.begin(), x.end(), q) - x.begin());
            data.push_back(std::min(std::max(r, lo), hi));
        }
        data.push_back(hi);
        return off;
    }
    void lin(const double* D, DevLin& L, int kind) {
        L.kind = kind;
        L.bk_d = add<double>(D + L.x, L.n, kind, 0, 0, L.n);
        L.bk_f = add<float>(D + L.x, L.n, kind, 0, 0, L.n);
    }
    void spline(const double* D, DevSpline& S) {
        int nk = S.n_ctrl + S.degree + 1;
        S.bk_d = add<double>(D + S.knot_e, nk, 0, 0, S.degree - 1, nk - S.degree - 1);
        S.bk_f = add<float>(D + S.knot_e, nk, 0, 0, S.degree - 1, nk - S.degree - 1);
    }
    void rita(const double* D, DevRita& Rt) {
        Rt.bk_d = add<double>(D + Rt.energy, Rt.n_energy, 0, 1, 0, Rt.n_energy);
        Rt.bk_f = add<float>(D + Rt.energy, Rt.n_energy, 0, 1, 0, Rt.n_energy);
    }
};

}  // namespace

extern "C" midsx_status midsx_gpu_tables_create(const midsx_table_blob* blob, midsx_tables_h* out) {
    if (!blob || !out || blob->n_materials < 1 || blob->n_materials > MIDSX_MAX_MATERIALS ||
        blob->n_data <= 0 || blob->n_data > (int64_t(1) << 31) || !blob->data || !blob->idata) {
        set_last_error("midsx_gpu_tables_create: invalid blob");
        return MIDSX_INVALID_ARG;
    }
    auto* h = new midsx_gpu_tables();
    std::memset(&h->T, 0, sizeof(h->T));
    auto guard = scope_exit([h] { midsx_gpu_tables_destroy(h); });
    CUDA_TRY(cudaGetDevice(&h->device));
    CUDA_TRY(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device));
    int optin = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    h->max_smem = size_t(optin);
    size_t nd = size_t(blob->n_data), ni = size_t(blob->n_idata);
    if (!cuda_ok(cudaMalloc(&h->d, nd * sizeof(double)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&h->f, nd * sizeof(float)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&h->rows, ni * sizeof(int)), "cudaMalloc"))
        return MIDSX_OOM;
    std::vector<int> rows(ni);
    for (size_t i = 0; i < ni; ++i) rows[i] = int(blob->idata[i]);
    CUDA_TRY(cudaMemcpy(h->d, blob->data, nd * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->rows, rows.data(), ni * sizeof(int), cudaMemcpyHostToDevice));
    f64_to_f32_kernel<<<unsigned((nd + 255) / 256), 256>>>(h->d, h->f, nd);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    // FP32 spline knots: interior knots of the FP64 vector that round to the knot before them
    // (parameters of grid energies a few meV apart) would give the FP32 basis recursion a
    // zero-width span and 0/0; each is raised to the next float above its predecessor, so the
    // FP32 knot vector increases wherever the FP64 one does (a shift of a few ulps)
    for (int m = 0; m < blob->n_materials; ++m) {
        for (const midsx_spline_table* sp : {&blob->mat[m].coh, &blob->mat[m].incoh}) {
            const int nk = sp->n_ctrl + sp->degree + 1;
            const double* kd = blob->data + sp->knot_u;
            std::vector<float> kf(static_cast<size_t>(nk));
            bool changed = false;
            for (int i = 0; i < nk; ++i) {
                kf[size_t(i)] = float(kd[i]);
                if (i > 0 && kd[i] > kd[i - 1] && !(kf[size_t(i)] > kf[size_t(i) - 1])) {
                    kf[size_t(i)] = std::nextafter(kf[size_t(i) - 1], 2.0f);
                    changed = true;
                }
            }
            if (changed)
                CUDA_TRY(cudaMemcpy(h->f + sp->knot_u, kf.data(), kf.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    DevTables& T = h->T;
    T.d = h->d;
    T.f = h->f;
    T.rows = h->rows;
    T.n_materials = blob->n_materials;
    T.alpha = kMec2 / (std::sqrt(2.0) * 4.135667662e-15 * 299792458E2 * 1E8);
    T.alpha_f = float(T.alpha);
    T.e_max = blob->e_max;
    fill_lin(T.majorant, blob->majorant);
    for (int32_t i = 0; i < blob->majorant.n; ++i) {
        h->maj_x.push_back(blob->data[blob->majorant.x + i]);
        h->maj_mu.push_back(std::pow(10.0, blob->data[blob->majorant.ly + i]));
    }
    for (int m = 0; m < blob->n_materials; ++m) {
        const midsx_material_table& s = blob->mat[m];
        DevMaterial& d = T.mat[m];
        fill_lin(d.total, s.total);
        fill_lin(d.sfunc, s.sfunc);
        fill_spline(d.coh, s.coh);
        fill_spline(d.incoh, s.incoh);
        d.rita.energy = int(s.rita.energy);
        d.rita.log_energy = int(s.rita.log_energy);
        d.rita.row_start = int(s.rita.row_start);
        d.rita.x = int(s.rita.x);
        d.rita.y = int(s.rita.y);
        d.rita.a = int(s.rita.a);
        d.rita.b = int(s.rita.b);
        d.rita.n_energy = s.rita.n_energy;
        h->ids[m] = s.id;
    }
    // Slopes of every LogLogLinear table: (ly[i] - ly[i-1]) / (lx[i] - lx[i-1]) in FP64 - the
    // quotient an FP64 lookup computes, bit for bit (IEEE division) - and rounded once for the
    // FP32 lookups (0 where two nodes share a log10 energy even in FP64)
    {
        std::vector<float> slopes(nd, 0.0f);
        std::vector<double> dslopes(nd, 0.0);
        auto add = [&](const midsx_lin_table& L) {
            const double* lx = blob->data + L.lx;
            const double* ly = blob->data + L.ly;
            for (int32_t i = 1; i < L.n; ++i) {
                const double dx = lx[i] - lx[i - 1];
                const double v = dx != 0.0 ? (ly[i] - ly[i - 1]) / dx : 0.0;
                slopes[size_t(L.ly + i)] = std::isfinite(v) ? float(v) : 0.0f;
                dslopes[size_t(L.ly + i)] = std::isfinite(v) ? v : 0.0;
            }
        };
        add(blob->majorant);
        for (int m = 0; m < blob->n_materials; ++m) {
            const midsx_material_table& s = blob->mat[m];
            add(s.total);
            add(s.photo);
            add(s.sfunc);
            add(s.ffactor);
        }
        if (!cuda_ok(cudaMalloc(&h->fs, nd * sizeof(float)), "cudaMalloc")) return MIDSX_OOM;
        CUDA_TRY(cudaMemcpy(h->fs, slopes.data(), nd * sizeof(float), cudaMemcpyHostToDevice));
        T.fs = h->fs;
        if (!cuda_ok(cudaMalloc(&h->ds, nd * sizeof(double)), "cudaMalloc")) return MIDSX_OOM;
        CUDA_TRY(cudaMemcpy(h->ds, dslopes.data(), nd * sizeof(double), cudaMemcpyHostToDevice));
        T.ds = h->ds;
    }
    // bucket tables for every searched node array, FP64 and FP32 queries
    BucketBuilder bb;
    const double* D = blob->data;
    bb.lin(D, T.majorant, 0);
    for (int m = 0; m < blob->n_materials; ++m) {
        DevMaterial& d = T.mat[m];
        bb.lin(D, d.total, 0);
        bb.lin(D, d.sfunc, 1);
        bb.spline(D, d.coh);
        bb.spline(D, d.incoh);
        bb.rita(D, d.rita);
    }
    for (int k = 0; k < 2; ++k)
        for (int p = 0; p < 2; ++p) T.bs[k][p] = bb.spec[k][p];
    if (!cuda_ok(cudaMalloc(&h->bk, bb.data.size() * sizeof(int)), "cudaMalloc")) return MIDSX_OOM;
    CUDA_TRY(cudaMemcpy(h->bk, bb.data.data(), bb.data.size() * sizeof(int), cudaMemcpyHostToDevice));
    T.bk = h->bk;
    guard.release();
    *out = h;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tables_destroy(midsx_tables_h t) {
    if (!t) return MIDSX_INVALID_ARG;
    cudaFree(t->d);
    cudaFree(t->f);
    cudaFree(t->fs);
    cudaFree(t->ds);
    cudaFree(t->rows);
    cudaFree(t->bk);
    delete t;
    return MIDSX_OK;
}

namespace {

// Uploads the grids' voxel ids (concatenated, grid after grid), remaps them to the tables'
// dense material indices and fills the domain description.
// Macro-cell masks of every grid with edges of 2^shift voxels (synchronous); the cells of a
// grid that meet an earlier grid's box (the earlier grid owns the overlap) take every
// material of the tables.  Replaces the phantom's previous cells.
midsx_status build_cells(midsx_gpu_phantom* p, int shift) {
    if (!p->ids) {
        set_last_error("the phantom's voxels are not resident");
        return MIDSX_INVALID_ARG;
    }
    const int n_grids = int(p->grids.size());
    auto cdim = [shift](int n) { return (n + (1 << shift) - 1) >> shift; };
    std::vector<size_t> cell_off(size_t(n_grids) + 1, 0);
    for (int k = 0; k < n_grids; ++k) {
        size_t c = 1;
        for (int i = 0; i < 3; ++i) c *= size_t(cdim(p->grids[size_t(k)].dims[i]));
        cell_off[size_t(k) + 1] = cell_off[size_t(k)] + c;
    }
    uint32_t* cells = nullptr;
    if (!cuda_ok(cudaMalloc(&cells, cell_off.back() * sizeof(uint32_t)), "cudaMalloc")) return MIDSX_OOM;
    const uint32_t all_bits =
        p->tables->T.n_materials >= 32 ? ~0u : ((1u << p->tables->T.n_materials) - 1u);
    const int sms = p->tables->sm_count;
    bool good = true;
    size_t voff = 0;
    for (int k = 0; good && k < n_grids; ++k) {
        const midsx_grid_spec& g = p->grids[size_t(k)];
        const int cnx = cdim(g.dims[0]), cny = cdim(g.dims[1]), cnz = cdim(g.dims[2]);
        uint32_t* gc = cells + cell_off[size_t(k)];
        cell_mask_kernel<<<sms * 4, 256>>>(p->ids + voff, g.dims[0], g.dims[1], g.dims[2], cnx, cny, cnz, shift, gc);
        good = cuda_ok(cudaGetLastError(), "cell_mask_kernel");
        for (int j = 0; good && j < k; ++j) {
            const midsx_grid_spec& e = p->grids[size_t(j)];
            int lo[3], hi[3];
            bool meets = true;
            for (int i = 0; i < 3; ++i) {
                const double csz = g.spacing[i] * double(1 << shift);
                const double a = e.origin[i] - g.origin[i], b = a + e.dims[i] * e.spacing[i];
                const double ext = g.dims[i] * g.spacing[i];
                if (b < 0 || a > ext) meets = false;
                const int cmax = cdim(g.dims[i]);
                lo[i] = std::max(0, std::min(cmax - 1, int(std::floor(a / csz)) - 1));
                hi[i] = std::max(0, std::min(cmax - 1, int(std::floor(b / csz)) + 1));
            }
            if (!meets) continue;
            cell_or_box_kernel<<<sms, 256>>>(gc, cnx, cny, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], all_bits);
            good = cuda_ok(cudaGetLastError(), "cell_or_box_kernel");
        }
        voff += size_t(g.dims[0]) * g.dims[1] * g.dims[2];
    }
    for (int k = 1; k < n_grids; ++k) {
        DevGrid& d = p->host_extra[size_t(k) - 1];
        for (int i = 0; i < 3; ++i) d.cdims[i] = cdim(d.dims[i]);
        d.cell_offset = int(cell_off[size_t(k)]);
    }
    if (good && n_grids > 1)
        good = cuda_ok(cudaMemcpy(p->extra, p->host_extra.data(), sizeof(DevGrid) * p->host_extra.size(),
                                  cudaMemcpyHostToDevice),
                       "cudaMemcpy");
    if (good) good = cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (!good) {
        cudaFree(cells);
        return MIDSX_CUDA_ERROR;
    }
    cudaFree(p->cells);
    p->cells = cells;
    p->cell_shift = shift;
    p->G.cells = cells;
    p->G.cell_shift = shift;
    for (int i = 0; i < 3; ++i) p->G.cdims[i] = cdim(p->grids[0].dims[i]);
    return MIDSX_OK;
}

midsx_status phantom_create_impl(midsx_tables_h tables, const double* domain, int32_t background_id,
                                 const midsx_grid_spec* grids, int n_grids, midsx_phantom_h* out) {
    if (!tables || !domain || !grids || !out || n_grids < 1 || n_grids > MIDSX_MAX_GRIDS) {
        set_last_error("midsx_gpu_phantom_create: invalid argument (1..16 grids)");
        return MIDSX_INVALID_ARG;
    }
    size_t total = 0;
    for (int k = 0; k < n_grids; ++k) {
        const midsx_grid_spec& g = grids[k];
        for (int i = 0; i < 3; ++i) {
            if (g.dims[i] < 1 || !(g.spacing[i] > 0) || !(domain[i] > 0)) {
                set_last_error("midsx_gpu_phantom_create: bad geometry");
                return MIDSX_INVALID_ARG;
            }
        }
        if (!g.ids) {
            set_last_error("midsx_gpu_phantom_create: missing voxel ids");
            return MIDSX_INVALID_ARG;
        }
        total += size_t(g.dims[0]) * g.dims[1] * g.dims[2];
    }
    if (total > size_t(0x7fffffff)) {
        set_last_error("midsx_gpu_phantom_create: more than 2^31 - 1 voxels");
        return MIDSX_INVALID_ARG;
    }
    uint8_t lut[256];
    std::memset(lut, 0xFF, sizeof(lut));
    int bg = -1;
    for (int m = 0; m < tables->T.n_materials; ++m) {
        lut[tables->ids[m] & 0xFF] = uint8_t(m);
        if (tables->ids[m] == background_id) bg = m;
    }
    if (bg < 0) {
        set_last_error("background material not in tables");
        return MIDSX_NOT_FOUND;
    }
    auto* p = new midsx_gpu_phantom();
    p->n_voxels = total;
    uint8_t *raw = nullptr, *dlut = nullptr;
    int* bad = nullptr;
    auto release = [&]() {
        cudaFree(raw);
        cudaFree(dlut);
        cudaFree(bad);
    };
    if (!cuda_ok(cudaMalloc(&p->ids, total), "cudaMalloc") || !cuda_ok(cudaMalloc(&raw, total), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&dlut, 256), "cudaMalloc") || !cuda_ok(cudaMalloc(&bad, sizeof(int)), "cudaMalloc") ||
        (n_grids > 1 && !cuda_ok(cudaMalloc(&p->extra, sizeof(DevGrid) * (n_grids - 1)), "cudaMalloc"))) {
        release();
        midsx_gpu_phantom_destroy(p);
        return MIDSX_OOM;
    }
    std::vector<DevGrid> extra;
    size_t off = 0;
    for (int k = 0; k < n_grids; ++k) {
        const midsx_grid_spec& g = grids[k];
        const size_t n = size_t(g.dims[0]) * g.dims[1] * g.dims[2];
        if (!cuda_ok(cudaMemcpy(raw + off, g.ids, n, cudaMemcpyHostToDevice), "cudaMemcpy")) {
            release();
            midsx_gpu_phantom_destroy(p);
            return MIDSX_CUDA_ERROR;
        }
        if (k > 0) {
            DevGrid d;
            std::memset(&d, 0, sizeof(d));
            for (int i = 0; i < 3; ++i) {
                d.origin[i] = g.origin[i];
                d.spacing[i] = g.spacing[i];
                d.ext[i] = double(g.dims[i]) * g.spacing[i];  // VoxelGrid::setDimSpace
                d.dims[i] = g.dims[i];
                d.f_origin[i] = float(d.origin[i]);
                d.f_ext[i] = float(d.ext[i]);
                d.f_ispc[i] = 1.0f / float(d.spacing[i]);
            }
            d.offset = int(off);
            extra.push_back(d);
        }
        off += n;
    }
    // the grids after the first (their macro-cell fields are filled when the cells are built)
    bool good = cuda_ok(cudaMemcpy(dlut, lut, 256, cudaMemcpyHostToDevice), "cudaMemcpy") &&
                cuda_ok(cudaMemset(bad, 0, sizeof(int)), "cudaMemset") &&
                (extra.empty() || cuda_ok(cudaMemcpy(p->extra, extra.data(), sizeof(DevGrid) * extra.size(),
                                                     cudaMemcpyHostToDevice),
                                          "cudaMemcpy"));
    int hbad = 0;
    if (good) {
        remap_kernel<<<tables->sm_count * 8, 256>>>(raw, p->ids, dlut, total, bad);
        good = cuda_ok(cudaGetLastError(), "remap_kernel") &&
               cuda_ok(cudaMemcpy(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
    release();
    if (!good) {
        midsx_gpu_phantom_destroy(p);
        return MIDSX_CUDA_ERROR;
    }
    if (hbad) {
        midsx_gpu_phantom_destroy(p);
        set_last_error("voxel material id not among the tables' materials");
        return MIDSX_NOT_FOUND;
    }
    DevGeom& G = p->G;
    const midsx_grid_spec& g0 = grids[0];
    for (int i = 0; i < 3; ++i) {
        G.domain[i] = domain[i];
        G.origin[i] = g0.origin[i];
        G.spacing[i] = g0.spacing[i];
        G.dims[i] = g0.dims[i];
        G.ext[i] = double(g0.dims[i]) * g0.spacing[i];  // VoxelGrid::setDimSpace
    }
    G.background = bg;
    G.ids = p->ids;
    G.n_grids = n_grids;
    G.extra = p->extra;
    p->tables = tables;
    p->grids.assign(grids, grids + n_grids);
    for (auto& gs : p->grids) gs.ids = nullptr;
    p->host_extra = extra;
    p->cell_shift = kCellShiftDefault;
    *out = p;
    return MIDSX_OK;
}

// The macro cells a MIDSX_TRACK_MACRO_CELL launch reads, built on first use.
midsx_status ensure_cells(midsx_gpu_phantom* p) { return p->cells ? MIDSX_OK : build_cells(p, p->cell_shift); }

}  // namespace

extern "C" midsx_status midsx_gpu_phantom_create(midsx_tables_h tables, const midsx_geometry_spec* g,
                                                 const uint8_t* ids, midsx_phantom_h* out) {
    if (!tables || !g || !ids || !out) return MIDSX_INVALID_ARG;
    midsx_grid_spec one;
    std::memset(&one, 0, sizeof(one));
    for (int i = 0; i < 3; ++i) {
        one.spacing[i] = g->spacing[i];
        one.origin[i] = g->origin[i];
        one.dims[i] = g->dims[i];
    }
    one.ids = ids;
    return phantom_create_impl(tables, g->domain, g->background_id, &one, 1, out);
}

extern "C" midsx_status midsx_gpu_phantom_create_grids(midsx_tables_h tables, const double* domain,
                                                       int32_t background_id, const midsx_grid_spec* grids,
                                                       int32_t n_grids, midsx_phantom_h* out) {
    return phantom_create_impl(tables, domain, background_id, grids, n_grids, out);
}

extern "C" midsx_status midsx_gpu_phantom_macro_cells(midsx_phantom_h p, int32_t edge) {
    if (!p || edge < 1 || edge > 64 || (edge & (edge - 1))) {
        set_last_error("midsx_gpu_phantom_macro_cells: edge is a power of two in [1, 64]");
        return MIDSX_INVALID_ARG;
    }
    int shift = 0;
    while ((1 << shift) < edge) ++shift;
    if (!p->ids) {  // not resident: built with this edge when first needed
        cudaFree(p->cells);
        p->cells = nullptr;
        p->G.cells = nullptr;
        p->cell_shift = shift;
        return MIDSX_OK;
    }
    return build_cells(p, shift);
}

extern "C" midsx_status midsx_gpu_phantom_destroy(midsx_phantom_h p) {
    if (!p) return MIDSX_INVALID_ARG;
    cudaFree(p->ids);
    cudaFree(p->extra);
    cudaFree(p->cells);
    delete p;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_source_create(const midsx_source_spec* spec, midsx_source_h* out) {
    if (!spec || !out || spec->direction_kind < 0 || spec->direction_kind > 3 || spec->spectrum_kind < 0 ||
        spec->spectrum_kind > 1) {
        set_last_error("midsx_gpu_source_create: invalid spec");
        return MIDSX_INVALID_ARG;
    }
    auto* s = new midsx_gpu_source();
    auto guard = scope_exit([s] { midsx_gpu_source_destroy(s); });
    DevSource& S = s->S;
    std::memset(&S, 0, sizeof(S));
    for (int i = 0; i < 3; ++i) {
        S.pos[i] = spec->position[i];
        S.a[i] = spec->a[i];
        S.b[i] = spec->b[i];
        S.c[i] = spec->c[i];
    }
    S.dir_kind = spec->direction_kind;
    S.spec_kind = spec->spectrum_kind;
    S.radius = spec->radius;
    S.mono = spec->mono_energy;
    if (spec->direction_kind == MIDSX_DIR_RECTANGLE) {
        double d = spec->b[0] * spec->c[0] + spec->b[1] * spec->c[1] + spec->b[2] * spec->c[2];
        if (std::fabs(d) >= 1e-9) {
            set_last_error("Edges are not orthogonal");
            return MIDSX_INVALID_ARG;
        }
    }
    if (spec->direction_kind == MIDSX_DIR_DISC) {
        // DiscIsotropicDirectionality::setUAndV (source.cpp:117-129)
        const double* n = spec->b;
        double u[3], v[3];
        auto cross = [](const double* a, const double* b, double* o) {
            o[0] = a[1] * b[2] - a[2] * b[1];
            o[1] = a[2] * b[0] - a[0] * b[2];
            o[2] = a[0] * b[1] - a[1] * b[0];
        };
        auto normalize = [](double* a) {
            double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            if (l > 0)
                for (int i = 0; i < 3; ++i) a[i] /= l;
        };
        const double xh[3] = {1, 0, 0}, yh[3] = {0, 1, 0};
        if (std::fabs(n[0]) < 1e-9)
            cross(n, yh, u);
        else
            cross(n, xh, u);
        normalize(u);
        cross(n, u, v);
        normalize(v);
        for (int i = 0; i < 3; ++i) {
            S.b[i] = u[i];
            S.c[i] = v[i];
        }
    }
    if (spec->spectrum_kind == MIDSX_SPEC_POLY) {
        int nb = spec->n_bins;
        if (nb < 1 || nb > MIDSX_MAX_SPECTRUM_BINS || !spec->bin_energy || !spec->bin_prob) {
            set_last_error("bad spectrum");
            return MIDSX_INVALID_ARG;
        }
        // DiscreteInversion: normalise (if the sum differs from 1) then cumulative sum
        std::vector<double> h(2 * size_t(nb));
        double sum = 0;
        for (int i = 0; i < nb; ++i) sum += spec->bin_prob[i];
        double acc = 0;
        s->min_energy = INFINITY;
        for (int i = 0; i < nb; ++i) {
            double p = (sum != 1.0) ? spec->bin_prob[i] / sum : spec->bin_prob[i];
            acc = (i == 0) ? p : acc + p;
            h[i] = spec->bin_energy[i];
            h[nb + i] = acc;
            s->max_energy = std::max(s->max_energy, spec->bin_energy[i]);
            if (spec->bin_prob[i] > 0) s->min_energy = std::min(s->min_energy, spec->bin_energy[i]);
        }
        if (!(s->min_energy < INFINITY)) s->min_energy = s->max_energy;
        // device buffer: FP64 energies and CDF, their FP32 copies, then the guide tables of
        // the FP64 and FP32 CDF searches (the same comparison as the device's lower_index; a
        // CDF that is not monotone keeps the full range in every guide interval)
        std::vector<float> hf(2 * size_t(nb));
        for (size_t i = 0; i < hf.size(); ++i) hf[i] = float(h[i]);
        const bool monotone = std::is_sorted(h.begin() + nb, h.end()) && std::is_sorted(hf.begin() + nb, hf.end());
        std::vector<int> guide(2 * size_t(kCdfGuide + 1));
        for (int k = 0; k <= kCdfGuide; ++k) {
            const double qd = double(k) / kCdfGuide;
            const float qf = float(k) / float(kCdfGuide);
            guide[size_t(k)] = monotone ? int(std::lower_bound(h.begin() + nb, h.end(), qd) - (h.begin() + nb))
                                        : (k == kCdfGuide ? nb : 0);
            guide[size_t(kCdfGuide + 1 + k)] =
                monotone ? int(std::lower_bound(hf.begin() + nb, hf.end(), qf) - (hf.begin() + nb))
                         : (k == kCdfGuide ? nb : 0);
        }
        const size_t bytes = h.size() * sizeof(double) + hf.size() * sizeof(float) + guide.size() * sizeof(int);
        CUDA_TRY(cudaMalloc(&s->buf, bytes));
        CUDA_TRY(cudaMemcpy(s->buf, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        float* fbuf = reinterpret_cast<float*>(s->buf + h.size());
        CUDA_TRY(cudaMemcpy(fbuf, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice));
        int* gbuf = reinterpret_cast<int*>(fbuf + hf.size());
        CUDA_TRY(cudaMemcpy(gbuf, guide.data(), guide.size() * sizeof(int), cudaMemcpyHostToDevice));
        S.n_bins = nb;
        S.energy = s->buf;
        S.cdf = s->buf + nb;
        S.f_energy = fbuf;
        S.f_cdf = fbuf + nb;
        S.guide = gbuf;
        S.f_guide = gbuf + kCdfGuide + 1;
    } else {
        if (!(spec->mono_energy > 0)) {
            set_last_error("bad mono energy");
            return MIDSX_INVALID_ARG;
        }
        s->max_energy = spec->mono_energy;
        s->min_energy = spec->mono_energy;
    }
    for (int i = 0; i < 3; ++i) {
        S.f_pos[i] = float(S.pos[i]);
        S.f_a[i] = float(S.a[i]);
        S.f_b[i] = float(S.b[i]);
        S.f_c[i] = float(S.c[i]);
    }
    S.f_radius = float(S.radius);
    S.f_mono = float(S.mono);
    guard.release();
    *out = s;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_source_destroy(midsx_source_h s) {
    if (!s) return MIDSX_INVALID_ARG;
    cudaFree(s->buf);
    delete s;
    return MIDSX_OK;
}

namespace {

// Validates the tally specs and lays out the handle on the host: device records with
// accumulator offsets (relative to `acc`, fixed once it is allocated), accumulator and dose
// sizes.  Allocates nothing on the device.
midsx_status tallies_layout(size_t n_voxels, const midsx_tally_spec* specs, int32_t n_specs, int32_t dose_mode,
                            midsx_gpu_tallies* t) {
    if (n_specs < 0 || n_specs > MIDSX_MAX_TALLIES || (n_specs > 0 && !specs) || dose_mode < 0 ||
        dose_mode > MIDSX_DOSE_BATCHES) {
        set_last_error("midsx_gpu_tallies_create: invalid argument");
        return MIDSX_INVALID_ARG;
    }
    t->dose_mode = dose_mode;
    t->dose_stride = dose_mode == 0 ? 0 : (dose_mode == 1 ? 1 : 4);
    t->n_voxels = n_voxels;
    size_t words = 0;
    for (int i = 0; i < n_specs; ++i) {
        const midsx_tally_spec& s = specs[i];
        DevTally d;
        std::memset(&d, 0, sizeof(d));
        d.kind = s.kind;
        d.nu = s.nu;
        d.nv = s.nv;
        d.n_energy = s.n_energy;
        d.e_min = s.e_min;
        d.e_width = s.e_width;
        const bool scalar_surface = s.kind == MIDSX_TALLY_SURFACE_DISC || s.kind == MIDSX_TALLY_SURFACE_RECT;
        if (s.n_energy < 0 || s.n_energy > MIDSX_MAX_ENERGY_BINS || (s.n_energy > 0 && !scalar_surface) ||
            (s.n_energy > 0 && !(s.e_width > 0.0 && std::isfinite(s.e_width) && std::isfinite(s.e_min)))) {
            set_last_error("energy spectrum: DISC or RECT tally, 0 < n_energy <= MIDSX_MAX_ENERGY_BINS, e_width > 0");
            return MIDSX_INVALID_ARG;
        }
        for (int k = 0; k < 3; ++k) {
            d.a[k] = s.a[k];
            d.b[k] = s.b[k];
            d.c[k] = s.c[k];
        }
        d.radius = s.radius;
        if (s.kind == MIDSX_TALLY_SURFACE_DISC) {
            for (int k = 0; k < 3; ++k) d.norm[k] = s.b[k];  // DiscSurfaceTally keeps norm as given
        } else if (s.kind == MIDSX_TALLY_SURFACE_RECT || s.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
            double dd = s.b[0] * s.c[0] + s.b[1] * s.c[1] + s.b[2] * s.c[2];
            if (std::fabs(dd) >= 1e-9) {
                set_last_error("Edges are not orthogonal");
                return MIDSX_INVALID_ARG;
            }
            double n[3] = {s.b[1] * s.c[2] - s.b[2] * s.c[1], s.b[2] * s.c[0] - s.b[0] * s.c[2],
                           s.b[0] * s.c[1] - s.b[1] * s.c[0]};
            double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; ++k) d.norm[k] = n[k] / l;
            d.e1e1 = s.b[0] * s.b[0] + s.b[1] * s.b[1] + s.b[2] * s.b[2];
            d.e2e2 = s.c[0] * s.c[0] + s.c[1] * s.c[1] + s.c[2] * s.c[2];
            if (s.kind == MIDSX_TALLY_SURFACE_BINNED_RECT && (s.nu < 1 || s.nv < 1)) {
                set_last_error("binned tally needs nu, nv >= 1");
                return MIDSX_INVALID_ARG;
            }
        } else if (s.kind != MIDSX_TALLY_VOLUME_AACUBOID) {
            set_last_error("unknown tally kind");
            return MIDSX_INVALID_ARG;
        }
        for (int k = 0; k < 3; ++k) {
            d.fa[k] = float(d.a[k]);
            d.fb[k] = float(d.b[k]);
            d.fc[k] = float(d.c[k]);
            d.fnorm[k] = float(d.norm[k]);
        }
        d.fradius = float(d.radius);
        d.fe1e1 = float(d.e1e1);
        d.fe2e2 = float(d.e2e2);
        d.fe_min = float(d.e_min);
        d.fe_width = float(d.e_width);
        d.acc = reinterpret_cast<unsigned long long*>(words);  // offset, fixed after allocation
        // a spectrum follows the scalar words: [bin][class][crossings, cosine sum]
        words += (s.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) ? size_t(s.nu) * s.nv * 8
                                                              : kScalarWords + size_t(d.n_energy) * 8;
        t->host_specs.push_back(d);
        if (d.n_energy > 0) t->spectra = true;
    }
    t->acc_words = words;
    return MIDSX_OK;
}

// Device bytes of a laid-out handle: statistics (+ the launch counter word), accumulators,
// tally records and the dose grid.
size_t tallies_bytes(const midsx_gpu_tallies* t) {
    return (kStCount + 1) * 8 + t->acc_words * 8 + t->host_specs.size() * sizeof(DevTally) +
           t->n_voxels * size_t(t->dose_stride) * 8 + (t->dose_mode == MIDSX_DOSE_BATCHES ? t->n_voxels * 16 : 0);
}

}  // namespace

extern "C" midsx_status midsx_gpu_tallies_create(midsx_phantom_h phantom, const midsx_tally_spec* specs,
                                                 int32_t n_specs, int32_t dose_mode, midsx_tallies_h* out) {
    if (!out || (dose_mode > 0 && !phantom)) {
        set_last_error("midsx_gpu_tallies_create: invalid argument");
        return MIDSX_INVALID_ARG;
    }
    auto* t = new midsx_gpu_tallies();
    auto guard = scope_exit([t] { midsx_gpu_tallies_destroy(t); });
    midsx_status lst = tallies_layout(phantom ? phantom->n_voxels : 0, specs, n_specs, dose_mode, t);
    if (lst != MIDSX_OK) return lst;
    const size_t words = t->acc_words;
    // run statistics plus one word: the launch's history counter
    if (!cuda_ok(cudaMalloc(&t->stats, (kStCount + 1) * sizeof(unsigned long long)), "cudaMalloc") ||
        (words && !cuda_ok(cudaMalloc(&t->acc, words * 8), "cudaMalloc")) ||
        (n_specs && !cuda_ok(cudaMalloc(&t->specs, n_specs * sizeof(DevTally)), "cudaMalloc")) ||
        (t->dose_stride &&
         !cuda_ok(cudaMalloc(&t->dose, t->n_voxels * t->dose_stride * sizeof(unsigned long long)), "cudaMalloc")) ||
        (dose_mode == MIDSX_DOSE_BATCHES && !cuda_ok(cudaMalloc(&t->batch, t->n_voxels * 16), "cudaMalloc")))
        return MIDSX_OOM;
    for (auto& d : t->host_specs) d.acc = t->acc + reinterpret_cast<size_t>(d.acc);
    if (n_specs)
        CUDA_TRY(cudaMemcpy(t->specs, t->host_specs.data(), n_specs * sizeof(DevTally), cudaMemcpyHostToDevice));
    midsx_status st = midsx_gpu_tallies_reset(t, nullptr);
    if (st != MIDSX_OK) return st;
    CUDA_TRY(cudaDeviceSynchronize());
    guard.release();
    *out = t;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tallies_destroy(midsx_tallies_h t) {
    if (!t) return MIDSX_INVALID_ARG;
    if (t->pooled) {
        set_last_error("these tallies belong to a request server: release the request instead");
        return MIDSX_INVALID_ARG;
    }
    cudaFree(t->dose);
    cudaFree(t->batch);
    cudaFree(t->specs);
    cudaFree(t->acc);
    cudaFree(t->stats);
    delete t;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tallies_reset(midsx_tallies_h t, void* stream) {
    if (!t) return MIDSX_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaMemsetAsync(t->stats, 0, kStCount * sizeof(unsigned long long), s));
    if (t->acc_words) CUDA_TRY(cudaMemsetAsync(t->acc, 0, t->acc_words * 8, s));
    if (t->dose) CUDA_TRY(cudaMemsetAsync(t->dose, 0, t->n_voxels * t->dose_stride * 8, s));
    if (t->batch) CUDA_TRY(cudaMemsetAsync(t->batch, 0, t->n_voxels * 16, s));
    t->batches_closed = 0;
    t->precision = -1;
    return MIDSX_OK;
}

namespace {

// Checks that a job's handles belong together: phantom made with `tables`, dose tally sized
// for the phantom, source energies inside the tables.
midsx_status check_job(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                       midsx_tallies_h tallies, const std::string& what) {
    if (!phantom || !source || !tallies || phantom->tables != tables) {
        set_last_error(what + ": missing handle or phantom made with other tables");
        return MIDSX_INVALID_ARG;
    }
    if (tallies->dose && tallies->n_voxels != phantom->n_voxels) {
        set_last_error(what + ": dose tally size differs from the phantom");
        return MIDSX_INVALID_ARG;
    }
    if (source->max_energy > tables->T.e_max) {
        set_last_error(what + ": source energy above the tables' e_max");
        return MIDSX_TABLE_RANGE;
    }
    return MIDSX_OK;
}

// Default per-history step cap of a job.  The reference's history loop has no cap
// (src/MIDSX/Core/physics_engine.cpp:22); the device loop needs one so that it always ends, and
// it must not bias results: a straight flight across the domain at energy E takes on average
// (domain diagonal) x mu_max(E) Woodcock steps.  The cap allows 16 such crossings at the largest
// majorant between E_floor = min(1 keV, the source's lowest energy) and the tables' e_max,
// far beyond what a history reaches: photons scattered down to a few keV are absorbed long
// before (photoelectric absorption dominates there).  At least 100,000, at most 2^31 - 1.
uint32_t derived_step_cap(const midsx_gpu_tables* tables, midsx_phantom_h phantom, midsx_source_h source) {
    const double e_floor = std::min(1e3, source->min_energy > 0 ? source->min_energy : 1e3);
    const std::vector<double>& x = tables->maj_x;
    const std::vector<double>& mu = tables->maj_mu;
    double mu_hi = 0;
    for (size_t i = 0; i < x.size(); ++i)
        if (x[i] >= e_floor && x[i] <= tables->T.e_max) mu_hi = std::max(mu_hi, mu[i]);
    // LogLogLinear value at e_floor itself (between nodes)
    const size_t k = size_t(std::upper_bound(x.begin(), x.end(), e_floor) - x.begin());
    if (k == 0 || k >= x.size()) {
        mu_hi = std::max(mu_hi, k == 0 ? (mu.empty() ? 0.0 : mu.front()) : mu.back());
    } else {
        const double t = (std::log10(e_floor) - std::log10(x[k - 1])) / (std::log10(x[k]) - std::log10(x[k - 1]));
        mu_hi = std::max(mu_hi, std::pow(10.0, std::log10(mu[k - 1]) + t * (std::log10(mu[k]) - std::log10(mu[k - 1]))));
    }
    const double* d = phantom->G.domain;
    const double diag = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double cap = std::ceil(16.0 * diag * mu_hi);
    if (!(cap > 1e5)) return 100000u;
    return cap >= 2147483647.0 ? 2147483647u : uint32_t(cap);
}

void fill_job(DevJob& J, midsx_phantom_h phantom, midsx_source_h source, midsx_tallies_h tallies, uint64_t seed,
              uint64_t first, uint64_t n) {
    J.G = phantom->G;
    J.S = source->S;
    J.tallies = tallies->specs;
    J.n_tallies = int(tallies->host_specs.size());
    J.dose_stride = tallies->dose_stride;
    J.dose = tallies->dose;
    J.stats = tallies->stats;
    J.seed = seed;
    J.first = first;
    J.n = n;
    J.step_cap = derived_step_cap(phantom->tables, phantom, source);
}

template <typename R, bool MULTI>
midsx_status launch_typed(midsx_tables_h tables, const RunParams& P, const midsx_run_config& cfg, int block,
                          cudaStream_t s) {
    const size_t smem = kernel_smem<R>(P.n_jobs, MULTI, tables->T.n_materials, block);
    if (smem > 48 * 1024)
        CUDA_TRY(cudaFuncSetAttribute(transport_kernel<R, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(smem)));
    int per_sm = cfg.blocks_per_sm;
    if (per_sm <= 0) {
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<R, MULTI>, block, smem));
        per_sm = std::max(per_sm, 1);
    }
    uint64_t want = (P.total + block - 1) / block;
    uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(want, uint64_t(tables->sm_count) * per_sm));
    transport_kernel<R, MULTI><<<unsigned(grid), block, smem, s>>>(P);
    CUDA_TRY(cudaGetLastError());
    return MIDSX_OK;
}

template <typename R, bool MULTI, int TRACK, bool SPEC>
midsx_status launch_pool(midsx_tables_h tables, const RunParams& P, const midsx_run_config& cfg, int block,
                         cudaStream_t s) {
    const size_t smem = pool_smem<R>(P.n_jobs, MULTI, tables->T.n_materials, block);
    if (smem > 48 * 1024)
        CUDA_TRY(cudaFuncSetAttribute(transport_pool_kernel<R, MULTI, TRACK, SPEC>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = cfg.blocks_per_sm;
    if (per_sm <= 0) {
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_pool_kernel<R, MULTI, TRACK, SPEC>, block,
                                                               smem));
        per_sm = std::max(per_sm, 1);
    }
    if (per_sm < 1) {
        set_last_error("the photon pool does not fit the shared memory of an SM");
        return MIDSX_INVALID_ARG;
    }
    // a warp keeps two photons per lane in flight
    uint64_t want = (P.total + 2 * uint64_t(block) - 1) / (2 * uint64_t(block));
    uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(want, uint64_t(tables->sm_count) * per_sm));
    transport_pool_kernel<R, MULTI, TRACK, SPEC><<<unsigned(grid), block, smem, s>>>(P);
    CUDA_TRY(cudaGetLastError());
    return MIDSX_OK;
}

template <typename R, bool MULTI>
midsx_status launch_pool(midsx_tables_h tables, const RunParams& P, const midsx_run_config& cfg, int block,
                         cudaStream_t s) {
    // spectra: single-job launches only (batched launches with spectra run the lane-parking
    // kernel), so that their instantiations stay few
    if constexpr (!MULTI) {
        if (P.spectra) {
            switch (P.tracking) {
                case MIDSX_TRACK_BACKGROUND_FAST:
                    return launch_pool<R, false, MIDSX_TRACK_BACKGROUND_FAST, true>(tables, P, cfg, block, s);
                case MIDSX_TRACK_MACRO_CELL:
                    return launch_pool<R, false, MIDSX_TRACK_MACRO_CELL, true>(tables, P, cfg, block, s);
                default:
                    return launch_pool<R, false, MIDSX_TRACK_REFERENCE, true>(tables, P, cfg, block, s);
            }
        }
    }
    switch (P.tracking) {
        case MIDSX_TRACK_BACKGROUND_FAST:
            return launch_pool<R, MULTI, MIDSX_TRACK_BACKGROUND_FAST, false>(tables, P, cfg, block, s);
        case MIDSX_TRACK_MACRO_CELL:
            return launch_pool<R, MULTI, MIDSX_TRACK_MACRO_CELL, false>(tables, P, cfg, block, s);
        default:
            return launch_pool<R, MULTI, MIDSX_TRACK_REFERENCE, false>(tables, P, cfg, block, s);
    }
}

// Shared-memory bytes of a launch of either scheduler.
size_t launch_smem(int n_jobs, bool multi, bool mixed, bool pool, int n_materials, int block) {
    if (pool) return mixed ? pool_smem<float>(n_jobs, multi, n_materials, block)
                           : pool_smem<double>(n_jobs, multi, n_materials, block);
    return mixed ? kernel_smem<float>(n_jobs, multi, n_materials, block)
                 : kernel_smem<double>(n_jobs, multi, n_materials, block);
}

// Completes the launch parameters from cfg, zeroes the history counter and launches.  The
// per-history trace is written by the lane-parking kernel only.
midsx_status launch_kernel(midsx_tables_h tables, RunParams& P, const midsx_run_config& cfg, bool multi,
                           void* stream) {
    if (cfg.scheduler < MIDSX_SCHED_DEFAULT || cfg.scheduler > MIDSX_SCHED_POOL) {
        set_last_error("unknown scheduler");
        return MIDSX_INVALID_ARG;
    }
    if (cfg.tracking < MIDSX_TRACK_REFERENCE || cfg.tracking > MIDSX_TRACK_MACRO_CELL) {
        set_last_error("unknown tracking");
        return MIDSX_INVALID_ARG;
    }
    // batched launches with spectra run the lane-parking kernel (reference tracking)
    if (P.spectra && multi && (cfg.scheduler == MIDSX_SCHED_POOL || cfg.tracking != MIDSX_TRACK_REFERENCE)) {
        set_last_error("batched launches with incident-energy spectra run the lane-parking scheduler with reference "
                       "tracking");
        return MIDSX_INVALID_ARG;
    }
    const bool pool = cfg.scheduler != MIDSX_SCHED_LANES && P.trace == nullptr && !(P.spectra && multi) &&
                      (cfg.scheduler == MIDSX_SCHED_POOL || kDefaultScheduler == MIDSX_SCHED_POOL);
    if (cfg.tracking != MIDSX_TRACK_REFERENCE && !pool) {
        set_last_error("background fast and macro-cell tracking run in the photon-pool scheduler only");
        return MIDSX_INVALID_ARG;
    }
    P.tracking = cfg.tracking;
    if (cfg.steps_per_pass < 0 || cfg.steps_per_pass > 4) {
        set_last_error("steps_per_pass is 0 (default) or 1..4");
        return MIDSX_INVALID_ARG;
    }
    P.steps_per_pass = cfg.steps_per_pass > 0 ? cfg.steps_per_pass
                                               : default_steps_per_pass(cfg.precision, cfg.tracking, P.server != 0);
    P.pass_repeats = cfg.pass_repeats > 0 ? std::min(cfg.pass_repeats, 16)
                                          : default_pass_repeats(cfg.precision, cfg.tracking, P.server != 0);
    // cfg.max_steps = 0: the cap the caller derived from the jobs' geometry (P.max_steps)
    if (cfg.max_steps > 0) P.max_steps = cfg.max_steps;
    if (P.max_steps <= 0) P.max_steps = 100000;
    P.max_trials = cfg.max_compton_trials > 0 ? cfg.max_compton_trials : 100000;
    P.regroup = cfg.regroup > 0 ? std::min(cfg.regroup, 32) : (pool ? 32 : 24);
    P.chunk = cfg.chunk > 0 ? std::min(cfg.chunk, 64) : 1;
    const bool mixed = cfg.precision == MIDSX_PREC_MIXED;
    const int max_block = pool ? 128 : 256;
    int block = cfg.block_size > 0 ? cfg.block_size : max_block;
    if (block > max_block || block % 32) {
        set_last_error(max_block == 128 ? "block_size must be a multiple of 32 up to 128 (photon pool)"
                                        : "block_size must be a multiple of 32 up to 256");
        return MIDSX_INVALID_ARG;
    }
    // the per-photon caches hold every material: with many materials the default block
    // shrinks until its shared memory fits
    const int M = tables->T.n_materials;
    if (cfg.block_size <= 0)
        while (block > 32 && launch_smem(P.n_jobs, multi, mixed, pool, M, block) > tables->max_smem) block /= 2;
    if (launch_smem(P.n_jobs, multi, mixed, pool, M, block) > tables->max_smem) {
        set_last_error("the shared memory of a " + std::to_string(block) + "-thread block (caches of " +
                       std::to_string(M) + " materials) exceeds the device's: use a smaller block_size");
        return MIDSX_INVALID_ARG;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the launch's history counter and, for batched launches, each job's (the words after it)
    P.job_counters = multi ? P.counter + 1 : nullptr;
    CUDA_TRY(cudaMemsetAsync(P.counter, 0, sizeof(unsigned long long) * (multi ? 1 + size_t(P.n_jobs) : 1), s));
    if (pool) {
        if (mixed) return multi ? launch_pool<float, true>(tables, P, cfg, block, s)
                                : launch_pool<float, false>(tables, P, cfg, block, s);
        return multi ? launch_pool<double, true>(tables, P, cfg, block, s)
                     : launch_pool<double, false>(tables, P, cfg, block, s);
    }
    if (mixed) return multi ? launch_typed<float, true>(tables, P, cfg, block, s)
                            : launch_typed<float, false>(tables, P, cfg, block, s);
    return multi ? launch_typed<double, true>(tables, P, cfg, block, s)
                 : launch_typed<double, false>(tables, P, cfg, block, s);
}

// Closes batch k (1-based) of a MIDSX_DOSE_BATCHES tally: per voxel the sum accumulated
// since the last close (record word 0 minus word 3, exact in the fixed-point form) enters the
// running mean and sum of squared deviations (Welford's update), and word 3 takes the sum.
__global__ void batch_fold_kernel(unsigned long long* rec, size_t n, int mixed, double* mv, int k) {
    const double inv_k = 1.0 / double(k);
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        unsigned long long* r = rec + i * 4;
        const unsigned long long cur = r[0], last = r[3];
        const double d = mixed ? double((long long)(cur - last)) / kFxEnergy
                               : __longlong_as_double((long long)cur) - __longlong_as_double((long long)last);
        r[3] = cur;
        const double mean = mv[2 * i], delta = d - mean, m = mean + delta * inv_k;
        mv[2 * i] = m;
        mv[2 * i + 1] += delta * (d - m);
    }
}

// Launches the fold of the next batch of `t` on `s`.
midsx_status close_batch(midsx_gpu_tallies* t, int sm_count, cudaStream_t s) {
    if (!t->batch || t->n_voxels == 0) return MIDSX_OK;
    ++t->batches_closed;
    batch_fold_kernel<<<std::max(1, sm_count) * 8, 256, 0, s>>>(t->dose, t->n_voxels,
                                                               t->precision == MIDSX_PREC_MIXED, t->batch,
                                                               t->batches_closed);
    CUDA_TRY(cudaGetLastError());
    return MIDSX_OK;
}

midsx_status launch_run(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                        midsx_tallies_h tallies, const midsx_run_config* cfg, void* stream,
                        double* trace = nullptr) {
    if (!tables || !phantom || !source || !tallies || !cfg) return MIDSX_INVALID_ARG;
    if (cfg->precision != MIDSX_PREC_FP64 && cfg->precision != MIDSX_PREC_MIXED) {
        set_last_error("unknown precision");
        return MIDSX_INVALID_ARG;
    }
    if (tallies->precision >= 0 && tallies->precision != cfg->precision) {
        set_last_error("tallies hold results of the other precision; reset them first");
        return MIDSX_INVALID_ARG;
    }
    if (tallies->dose && tallies->n_voxels != phantom->n_voxels) {
        set_last_error("dose tally size differs from the phantom");
        return MIDSX_INVALID_ARG;
    }
    if (phantom->tables != tables) {
        set_last_error("the phantom was created with other tables");
        return MIDSX_INVALID_ARG;
    }
    if (source->max_energy > tables->T.e_max) {
        set_last_error("source energy above the tables' e_max");
        return MIDSX_TABLE_RANGE;
    }
    if (cfg->precision == MIDSX_PREC_MIXED && source->max_energy > kMixedMaxEnergy) {
        set_last_error("the mixed form's fixed-point tallies take source energies up to 262144 eV");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->variance_batches < 0 || cfg->variance_batches > 1024 ||
        (cfg->variance_batches > 1 && !tallies->batch)) {
        set_last_error("variance_batches: 0..1024, and 2 or more only into MIDSX_DOSE_BATCHES tallies");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->n_histories == 0) return MIDSX_OK;
    // a per-history trace runs the lane-parking kernel, which has reference tracking only:
    // refuse other tracking before anything is built for it (macro cells allocate)
    if (trace && cfg->tracking != MIDSX_TRACK_REFERENCE) {
        set_last_error("a per-history trace runs reference tracking only");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->tracking == MIDSX_TRACK_MACRO_CELL) {
        const midsx_status cs = ensure_cells(phantom);
        if (cs != MIDSX_OK) return cs;
    }
    RunParams P;
    std::memset(&P, 0, sizeof(P));
    P.T = tables->T;
    fill_job(P.job0, phantom, source, tallies, cfg->seed, cfg->first_history, cfg->n_histories);
    philox_round_keys(cfg->seed, P.round_keys);
    P.geo_f = make_geo<float>(P.job0.G);
    P.geo_d = make_geo<double>(P.job0.G);
    P.n_jobs = 1;
    P.max_steps = int(P.job0.step_cap);
    P.counter = tallies->stats + kStCount;
    P.total = cfg->n_histories;
    P.trace = trace;
    P.spectra = tallies->spectra;
    if (!tallies->batch) {
        midsx_status st = launch_kernel(tables, P, *cfg, false, stream);
        if (st == MIDSX_OK) tallies->precision = cfg->precision;
        return st;
    }
    // MIDSX_DOSE_BATCHES: one launch per batch over consecutive history ranges, each closed
    const uint64_t nb = uint64_t(std::max(1, cfg->variance_batches));
    if (nb > cfg->n_histories) {
        set_last_error("variance_batches exceeds the run's histories");
        return MIDSX_INVALID_ARG;
    }
    uint64_t first = cfg->first_history;
    for (uint64_t b = 0; b < nb; ++b) {
        const uint64_t n = cfg->n_histories / nb + (b < cfg->n_histories % nb ? 1 : 0);
        P.job0.first = first;
        P.job0.n = n;
        P.total = n;
        first += n;
        midsx_status st = launch_kernel(tables, P, *cfg, false, stream);
        if (st != MIDSX_OK) return st;
        tallies->precision = cfg->precision;
        st = close_batch(tallies, tables->sm_count, static_cast<cudaStream_t>(stream));
        if (st != MIDSX_OK) return st;
    }
    return MIDSX_OK;
}

double fx_signed(unsigned long long v, double scale) { return double((long long)v) / scale; }

}  // namespace

extern "C" midsx_status midsx_gpu_run(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                                      midsx_tallies_h tallies, const midsx_run_config* cfg, void* stream) {
    return launch_run(tables, phantom, source, tallies, cfg, stream);
}

extern "C" midsx_status midsx_gpu_fetch_stats(midsx_tallies_h t, midsx_run_stats* out, void* stream) {
    if (!t || !out) return MIDSX_INVALID_ARG;
    unsigned long long h[kStCount];
    CUDA_TRY(cudaMemcpyAsync(h, t->stats, sizeof(h), cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
    midsx_status st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    out->histories = h[kStHistories];
    out->steps = h[kStSteps];
    out->voxel_fetches = h[kStFetches];
    out->photo = h[kStPhoto];
    out->coherent = h[kStCoh];
    out->incoherent = h[kStIncoh];
    out->compton_trials = h[kStTrials];
    out->step_cap_hits = h[kStStepCap];
    out->compton_cap_hits = h[kStTrialCap];
    out->edge_clamps = h[kStEdge];
    out->tally_words = h[kStWords];
    out->source_energy = double(h[kStSourceE]) / kFxStat;
    out->deposited_grid = double(h[kStDepGrid]) / kFxStat;
    out->deposited_background = double(h[kStDepBg]) / kFxStat;
    out->escaped_energy = double(h[kStEscE]) / kFxStat;
    if (h[kStRangeErr]) {
        set_last_error("an energy left the RITA tables during transport");
        return MIDSX_TABLE_RANGE;
    }
    if (h[kStStepCap] || h[kStTrialCap]) {
        set_last_error("a history reached the step or Compton-trial cap");
        return MIDSX_STEP_CAP;
    }
    return MIDSX_OK;
}

namespace {
// Voxel dose records to doubles on the device (the host conversion of fx_signed, term for
// term): one output array per requested quantity, written with coalesced stores.
__global__ void dose_convert_kernel(const unsigned long long* rec, int stride, size_t n, int mixed, double* sum,
                                    double* sumsq, double* count) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const unsigned long long* r = rec + i * size_t(stride);
        if (sum) sum[i] = mixed ? double((long long)r[0]) / kFxEnergy : __longlong_as_double((long long)r[0]);
        if (sumsq) sumsq[i] = mixed ? double(r[1]) / kFxEnergy2 : __longlong_as_double((long long)r[1]);
        if (count) count[i] = double(r[2]);
    }
}
}  // namespace

// The conversion runs on the device into stream-ordered scratch, and the doubles go straight
// into the caller's arrays (a DMA into pinned memory; no host pass over the voxels).
extern "C" midsx_status midsx_gpu_fetch_dose(midsx_tallies_h t, double* sum, double* sumsq, double* count,
                                             void* stream) {
    if (!t || !t->dose) return MIDSX_INVALID_ARG;
    if ((sumsq || count) && t->dose_stride < 4) return MIDSX_INVALID_ARG;
    const size_t n = t->n_voxels;
    if (n == 0 || (!sum && !sumsq && !count)) return MIDSX_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* outs[3] = {sum, sumsq, count};
    double* dev[3] = {nullptr, nullptr, nullptr};
    bool good = true;
    for (int k = 0; k < 3 && good; ++k)
        if (outs[k]) good = cuda_ok(cudaMallocAsync(&dev[k], n * 8, s), "cudaMallocAsync");
    if (good) {
        int sms = 0, device = 0;
        cudaGetDevice(&device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        dose_convert_kernel<<<std::max(1, sms) * 8, 256, 0, s>>>(t->dose, t->dose_stride, n,
                                                                t->precision == MIDSX_PREC_MIXED, dev[0], dev[1],
                                                                dev[2]);
        good = cuda_ok(cudaGetLastError(), "dose_convert_kernel");
    }
    for (int k = 0; k < 3 && good; ++k)
        if (outs[k]) good = cuda_ok(cudaMemcpyAsync(outs[k], dev[k], n * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    for (int k = 0; k < 3; ++k)
        if (dev[k]) cudaFreeAsync(dev[k], s);
    if (!good) return MIDSX_CUDA_ERROR;
    return wait_stream(stream);
}

namespace {
__global__ void batch_variance_kernel(const double* mv, size_t n, double scale, double* var) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        var[i] = mv[2 * i + 1] * scale;
}
}  // namespace

// B s^2 with s^2 = M2 / (B - 1), the Welford sum of squared deviations of the batch sums.
extern "C" midsx_status midsx_gpu_fetch_dose_variance(midsx_tallies_h t, double* var, int32_t* n_batches,
                                                      void* stream) {
    if (!t || !var || !t->batch) {
        set_last_error("midsx_gpu_fetch_dose_variance: tallies without MIDSX_DOSE_BATCHES");
        return MIDSX_INVALID_ARG;
    }
    if (t->batches_closed < 2) {
        set_last_error("midsx_gpu_fetch_dose_variance: fewer than two batches closed");
        return MIDSX_INVALID_ARG;
    }
    const size_t n = t->n_voxels;
    if (n_batches) *n_batches = t->batches_closed;
    if (n == 0) return MIDSX_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* dev = nullptr;
    if (!cuda_ok(cudaMallocAsync(&dev, n * 8, s), "cudaMallocAsync")) return MIDSX_CUDA_ERROR;
    const double B = double(t->batches_closed);
    int sms = 0, device = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    batch_variance_kernel<<<std::max(1, sms) * 8, 256, 0, s>>>(t->batch, n, B / (B - 1.0), dev);
    bool good = cuda_ok(cudaGetLastError(), "batch_variance_kernel") &&
                cuda_ok(cudaMemcpyAsync(var, dev, n * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    cudaFreeAsync(dev, s);
    if (!good) return MIDSX_CUDA_ERROR;
    return wait_stream(stream);
}

extern "C" midsx_status midsx_gpu_fetch_scalar(midsx_tallies_h t, int32_t index, double* out, void* stream) {
    if (!t || !out || index < 0 || index >= int32_t(t->host_specs.size())) return MIDSX_INVALID_ARG;
    const DevTally& d = t->host_specs[index];
    if (d.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) return MIDSX_INVALID_ARG;
    unsigned long long h[kScalarWords];
    CUDA_TRY(cudaMemcpyAsync(h, d.acc, sizeof(h), cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
    midsx_status st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    const bool mixed = t->precision == MIDSX_PREC_MIXED;
    const bool surface = d.kind != MIDSX_TALLY_VOLUME_AACUBOID;
    for (int i = 0; i < kScalarWords; ++i) out[i] = 0;
    for (int q = 0; q < 2; ++q) {
        const bool is_cos = surface && q == 1;
        for (int c = 0; c < 4; ++c) {
            int b = q * 12 + c * 3;
            out[b] = double(h[b]);
            if (mixed) {
                out[b + 1] = fx_signed(h[b + 1], is_cos ? kFxCosine : kFxEnergy);
                out[b + 2] = double(h[b + 2]) / (is_cos ? kFxCosine : kFxEnergy2);
            } else {
                std::memcpy(&out[b + 1], &h[b + 1], 8);
                std::memcpy(&out[b + 2], &h[b + 2], 8);
            }
        }
    }
    for (int i = 24; i < 32; ++i) out[i] = double(h[i]);
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_fetch_binned(midsx_tallies_h t, int32_t index, double* energy, double* count,
                                               void* stream) {
    if (!t || index < 0 || index >= int32_t(t->host_specs.size())) return MIDSX_INVALID_ARG;
    const DevTally& d = t->host_specs[index];
    if (d.kind != MIDSX_TALLY_SURFACE_BINNED_RECT) return MIDSX_INVALID_ARG;
    size_t bins = size_t(d.nu) * d.nv;
    std::vector<unsigned long long> h(bins * 8);
    CUDA_TRY(cudaMemcpyAsync(h.data(), d.acc, h.size() * 8, cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
    midsx_status st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    const bool mixed = t->precision == MIDSX_PREC_MIXED;
    for (size_t i = 0; i < bins * 4; ++i) {
        if (energy) {
            if (mixed) {
                energy[i] = fx_signed(h[2 * i], kFxEnergy);
            } else {
                std::memcpy(&energy[i], &h[2 * i], 8);
            }
        }
        if (count) count[i] = double(h[2 * i + 1]);
    }
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_fetch_spectrum(midsx_tallies_h t, int32_t index, double* count, double* cosine,
                                                 void* stream) {
    if (!t || index < 0 || index >= int32_t(t->host_specs.size())) return MIDSX_INVALID_ARG;
    const DevTally& d = t->host_specs[index];
    if (d.n_energy <= 0) return MIDSX_INVALID_ARG;
    const size_t cells = size_t(d.n_energy) * 4;
    std::vector<unsigned long long> h(cells * 2);
    CUDA_TRY(cudaMemcpyAsync(h.data(), d.acc + kScalarWords, h.size() * 8, cudaMemcpyDeviceToHost,
                             static_cast<cudaStream_t>(stream)));
    midsx_status st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    const bool mixed = t->precision == MIDSX_PREC_MIXED;
    for (size_t i = 0; i < cells; ++i) {
        if (count) count[i] = double(h[2 * i]);
        if (cosine) {
            if (mixed)
                cosine[i] = fx_signed(h[2 * i + 1], kFxCosine);
            else
                std::memcpy(&cosine[i], &h[2 * i + 1], 8);
        }
    }
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_run_host(midsx_tables_h tables, const midsx_geometry_spec* geom,
                                           const uint8_t* ids, const midsx_source_spec* source,
                                           const midsx_tally_spec* specs, int32_t n_specs, int32_t dose_mode,
                                           const midsx_run_config* cfg, double* dose_sum_out,
                                           midsx_run_stats* stats_out) {
    midsx_phantom_h ph = nullptr;
    midsx_source_h src = nullptr;
    midsx_tallies_h tl = nullptr;
    midsx_status st = midsx_gpu_phantom_create(tables, geom, ids, &ph);
    if (st == MIDSX_OK) st = midsx_gpu_source_create(source, &src);
    if (st == MIDSX_OK) st = midsx_gpu_tallies_create(ph, specs, n_specs, dose_mode, &tl);
    if (st == MIDSX_OK) st = midsx_gpu_run(tables, ph, src, tl, cfg, nullptr);
    if (st == MIDSX_OK && stats_out) {
        midsx_status s2 = midsx_gpu_fetch_stats(tl, stats_out, nullptr);
        if (s2 != MIDSX_OK && s2 != MIDSX_STEP_CAP) st = s2;
    }
    if (st == MIDSX_OK && dose_sum_out && dose_mode > 0) st = midsx_gpu_fetch_dose(tl, dose_sum_out, nullptr, nullptr, nullptr);
    if (tl) midsx_gpu_tallies_destroy(tl);
    if (src) midsx_gpu_source_destroy(src);
    if (ph) midsx_gpu_phantom_destroy(ph);
    return st;
}

extern "C" midsx_status midsx_gpu_trace_deposits(midsx_tables_h tables, midsx_phantom_h phantom,
                                                 midsx_source_h source, const midsx_run_config* cfg,
                                                 double* hist_dep) {
    if (!tables || !phantom || !source || !cfg || !hist_dep) {
        set_last_error("midsx_gpu_trace_deposits: missing handle or output");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->n_histories == 0 || cfg->n_histories > (uint64_t(1) << 28)) {
        set_last_error("midsx_gpu_trace_deposits: n_histories must be in [1, 2^28]");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->tracking != MIDSX_TRACK_REFERENCE) {
        set_last_error("midsx_gpu_trace_deposits: a per-history trace runs reference tracking only");
        return MIDSX_INVALID_ARG;
    }
    midsx_tallies_h tl = nullptr;
    midsx_status st = midsx_gpu_tallies_create(nullptr, nullptr, 0, 0, &tl);
    if (st != MIDSX_OK) return st;
    double* d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, cfg->n_histories * sizeof(double)), "cudaMalloc")) {
        midsx_gpu_tallies_destroy(tl);
        return MIDSX_OOM;
    }
    st = launch_run(tables, phantom, source, tl, cfg, nullptr, d);
    if (st == MIDSX_OK) {
        midsx_run_stats rs;
        st = midsx_gpu_fetch_stats(tl, &rs, nullptr);
        if (st == MIDSX_STEP_CAP) st = MIDSX_OK;
    }
    if (st == MIDSX_OK && !cuda_ok(cudaMemcpy(hist_dep, d, cfg->n_histories * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy"))
        st = MIDSX_CUDA_ERROR;
    cudaFree(d);
    midsx_gpu_tallies_destroy(tl);
    return st;
}

// ------------------------------------------------- allocation-free per-history trace ---
// Device scratch of midsx_gpu_trace_deposits_noalloc, reserved when the library's device code
// is loaded onto a GPU and held until the process exits: the run's statistics counters in
// the first 256 bytes, then one double per history (at most kNoAllocMaxHistories).  Every
// call on a device reuses the same array.
namespace {
constexpr uint64_t kNoAllocMaxHistories = uint64_t(1) << 20;  // 1,048,576 histories, 8 MiB
constexpr size_t kNoAllocStatsBytes = 256;
static_assert((kStCount + 1) * sizeof(unsigned long long) <= kNoAllocStatsBytes,
              "statistics and the history counter fit the scratch header");
}  // namespace

static __device__ __align__(256) unsigned char midsx_noalloc_scratch[kNoAllocStatsBytes +
                                                                      kNoAllocMaxHistories * sizeof(double)];

namespace {
// Device address of midsx_noalloc_scratch on the current device.  Host code sees only a
// host-side stand-in under that name, so every call asks the runtime for the address with the
// caller's device current.  Nothing is cached: after a cudaDeviceReset the library's device
// code is loaded again, possibly at another address.  The lookup allocates nothing.
midsx_status noalloc_scratch(void** out) {
    void* p = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&p, midsx_noalloc_scratch), "cudaGetSymbolAddress")) return MIDSX_CUDA_ERROR;
    *out = p;
    return MIDSX_OK;
}
}  // namespace

extern "C" midsx_status midsx_gpu_trace_deposits_noalloc(midsx_tables_h tables, midsx_phantom_h phantom,
                                                         midsx_source_h source, const midsx_run_config* cfg,
                                                         double* hist_dep, void* stream) {
    if (!tables || !phantom || !source || !cfg || !hist_dep || cfg->n_histories == 0) {
        set_last_error("midsx_gpu_trace_deposits_noalloc: invalid argument");
        return MIDSX_INVALID_ARG;
    }
    if (cfg->n_histories > kNoAllocMaxHistories) {
        set_last_error("midsx_gpu_trace_deposits_noalloc: n_histories exceeds its fixed scratch of 1048576 histories");
        return MIDSX_INVALID_ARG;
    }
    // the trace runs reference tracking only; other modes would build macro cells (cudaMalloc)
    if (cfg->tracking != MIDSX_TRACK_REFERENCE) {
        set_last_error("midsx_gpu_trace_deposits_noalloc: reference tracking only (other modes allocate)");
        return MIDSX_INVALID_ARG;
    }
    void* base = nullptr;
    midsx_status st = noalloc_scratch(&base);
    if (st != MIDSX_OK) return st;
    unsigned long long* stats = static_cast<unsigned long long*>(base);
    double* dep = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kNoAllocStatsBytes);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the counters keep the previous call's values: clear them; every history of this call
    // writes its own deposit slot, so the deposit area needs no clearing
    CUDA_TRY(cudaMemsetAsync(stats, 0, kNoAllocStatsBytes, s));
    midsx_gpu_tallies view;  // statistics only: no tallies, no dose, nothing allocated
    view.stats = stats;
    st = launch_run(tables, phantom, source, &view, cfg, stream, dep);
    view.stats = nullptr;
    if (st != MIDSX_OK) return st;
    unsigned long long h[kStCount];
    CUDA_TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(hist_dep, dep, cfg->n_histories * sizeof(double), cudaMemcpyDeviceToHost, s));
    st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    if (h[kStRangeErr]) {
        set_last_error("an energy left the RITA tables during transport");
        return MIDSX_TABLE_RANGE;
    }
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_sample(midsx_tables_h tables, int32_t precision, int32_t kind, int32_t material,
                                         double energy, uint64_t seed, uint64_t first, int64_t n, double* out0,
                                         double* out1) {
    if (!tables || kind < 0 || kind > 2 || material < 0 || material >= tables->T.n_materials || n <= 0 || !out0 ||
        (kind == 1 && !out1) || n > (int64_t(1) << 30))
        return MIDSX_INVALID_ARG;
    if (kind == 0 && energy > tables->T.e_max) return MIDSX_TABLE_RANGE;
    double *d0 = nullptr, *d1 = nullptr;
    auto guard = scope_exit([&] {
        cudaFree(d0);
        cudaFree(d1);
    });
    CUDA_TRY(cudaMalloc(&d0, n * sizeof(double)));
    CUDA_TRY(cudaMalloc(&d1, n * sizeof(double)));
    unsigned grid = unsigned((n + 255) / 256);
    if (precision == MIDSX_PREC_MIXED)
        sample_kernel<float><<<grid, 256>>>(tables->T, kind, material, energy, seed, first, n, d0, d1);
    else
        sample_kernel<double><<<grid, 256>>>(tables->T, kind, material, energy, seed, first, n, d0, d1);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpy(out0, d0, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (out1) CUDA_TRY(cudaMemcpy(out1, d1, n * sizeof(double), cudaMemcpyDeviceToHost));
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_table_index(midsx_tables_h tables, int32_t material, const double* e, int64_t n,
                                              int64_t* idx) {
    if (!tables || !e || !idx || n <= 0 || material < 0 || material >= tables->T.n_materials || n > (int64_t(1) << 28))
        return MIDSX_INVALID_ARG;
    double* de = nullptr;
    int64_t* di = nullptr;
    auto guard = scope_exit([&] {
        cudaFree(de);
        cudaFree(di);
    });
    CUDA_TRY(cudaMalloc(&de, n * sizeof(double)));
    CUDA_TRY(cudaMalloc(&di, 6 * n * sizeof(int64_t)));
    CUDA_TRY(cudaMemcpy(de, e, n * sizeof(double), cudaMemcpyHostToDevice));
    index_kernel<<<unsigned((n + 255) / 256), 256>>>(tables->T, material, de, n, di);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpy(idx, di, 6 * n * sizeof(int64_t), cudaMemcpyDeviceToHost));
    return MIDSX_OK;
}

// ================================================================== batched launches ===
struct midsx_gpu_batch {
    midsx_tables_h tables = nullptr;
    int n_jobs = 0;
    std::vector<DevJob> host_jobs;
    std::vector<unsigned long long> host_prefix;
    std::vector<midsx_tallies_h> tallies;
    DevJob* jobs = nullptr;
    unsigned long long* prefix = nullptr;
    unsigned long long* words = nullptr;  // [0] epoch, [1] history counter, [2 ...] the jobs' counters
    cudaGraphExec_t graph = nullptr;
    int graph_precision = -1;
    double max_energy = 0;
    // large jobs in launches of their own (midsx_gpu_batch_set_own_launch); the persistent
    // launch takes the others, through their own record and prefix arrays
    uint64_t own_min = 0;
    std::vector<int> own;
    std::vector<unsigned long long> host_rest_prefix;
    int n_rest = 0;
    DevJob* rest_jobs = nullptr;
    unsigned long long* rest_prefix = nullptr;
};

namespace {

void batch_params(const midsx_gpu_batch* b, RunParams& P, const unsigned long long* prefix, unsigned long long total) {
    std::memset(&P, 0, sizeof(P));
    P.T = b->tables->T;
    P.jobs = b->jobs;
    P.n_jobs = b->n_jobs;
    P.prefix = prefix;
    P.counter = b->words + 1;
    P.total = total;
    P.epoch = b->words;
    for (auto* t : b->tallies) P.spectra |= t->spectra;
    for (const DevJob& j : b->host_jobs) P.max_steps = std::max(P.max_steps, int(j.step_cap));
}

// Splits the jobs into those with a launch of their own (n >= min) and the rest, whose
// records and history prefix go to device arrays of their own.  Synchronous.
midsx_status batch_split(midsx_gpu_batch* b, uint64_t min_histories) {
    // default: 16 loads of the GPU's resident photon slots (7 blocks x 4 warps x 64 slots per
    // SM); 4, 8, 16, 32 and 64 loads measured 8.05 / 8.06 / 8.05 / 8.02 / 7.98e8 histories/s
    // on the 64-job batch
    if (min_histories == 0) min_histories = uint64_t(28672) * uint64_t(std::max(1, b->tables->sm_count));
    std::vector<int> own;
    std::vector<DevJob> rest;
    std::vector<unsigned long long> rest_prefix(1, 0);
    for (int i = 0; i < b->n_jobs; ++i) {
        const DevJob& d = b->host_jobs[size_t(i)];
        if (d.n >= min_histories) {
            own.push_back(i);
        } else {
            rest.push_back(d);
            rest_prefix.push_back(rest_prefix.back() + d.n);
        }
    }
    if (!rest.empty()) {
        CUDA_TRY(cudaMemcpy(b->rest_jobs, rest.data(), rest.size() * sizeof(DevJob), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(b->rest_prefix, rest_prefix.data(), rest_prefix.size() * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice));
    }
    b->own_min = min_histories;
    b->own = own;
    b->n_rest = int(rest.size());
    b->host_rest_prefix = rest_prefix;
    return MIDSX_OK;
}

midsx_status batch_check_precision(midsx_gpu_batch* b, int precision) {
    if (precision != MIDSX_PREC_FP64 && precision != MIDSX_PREC_MIXED) {
        set_last_error("unknown precision");
        return MIDSX_INVALID_ARG;
    }
    if (precision == MIDSX_PREC_MIXED && b->max_energy > kMixedMaxEnergy) {
        set_last_error("the mixed form's fixed-point tallies take source energies up to 262144 eV");
        return MIDSX_INVALID_ARG;
    }
    for (auto* t : b->tallies) {
        if (t->precision >= 0 && t->precision != precision) {
            set_last_error("a job's tallies hold results of the other precision; reset them first");
            return MIDSX_INVALID_ARG;
        }
    }
    return MIDSX_OK;
}

// One run of the batch on `s`: the large jobs' own launches (single-job kernel, default
// launch shape, the batch's epoch and history counter words), the persistent launch over the
// rest, then the epoch advance.
midsx_status batch_enqueue(midsx_gpu_batch* b, const midsx_run_config& cfg, cudaStream_t s) {
    if (b->host_prefix.back() == 0) return MIDSX_OK;
    midsx_run_config single = cfg;
    single.block_size = single.blocks_per_sm = single.regroup = single.chunk = 0;
    single.scheduler = MIDSX_SCHED_DEFAULT;
    single.steps_per_pass = single.pass_repeats = 0;
    for (int j : b->own) {
        RunParams Q;
        std::memset(&Q, 0, sizeof(Q));
        Q.T = b->tables->T;
        Q.job0 = b->host_jobs[size_t(j)];
        philox_round_keys(Q.job0.seed, Q.round_keys);
        Q.geo_f = make_geo<float>(Q.job0.G);
        Q.geo_d = make_geo<double>(Q.job0.G);
        Q.n_jobs = 1;
        Q.max_steps = int(Q.job0.step_cap);
        Q.counter = b->words + 1;
        Q.total = Q.job0.n;
        Q.epoch = b->words;  // history ids first + epoch * n + i, as in the persistent launch
        Q.spectra = b->tallies[size_t(j)]->spectra;
        midsx_status st = launch_kernel(b->tables, Q, single, false, s);
        if (st != MIDSX_OK) return st;
    }
    if (b->host_rest_prefix.back() > 0) {
        RunParams P;
        batch_params(b, P, b->rest_prefix, b->host_rest_prefix.back());
        P.jobs = b->rest_jobs;
        P.n_jobs = b->n_rest;
        midsx_status st = launch_kernel(b->tables, P, cfg, true, s);
        if (st != MIDSX_OK) return st;
    }
    advance_epoch_kernel<<<1, 1, 0, s>>>(b->words);
    CUDA_TRY(cudaGetLastError());
    return MIDSX_OK;
}

}  // namespace

extern "C" midsx_status midsx_gpu_batch_create(midsx_tables_h tables, const midsx_batch_job* jobs, int32_t n_jobs,
                                               midsx_batch_h* out) {
    if (!tables || !jobs || !out || n_jobs < 1 || n_jobs > MIDSX_MAX_BATCH_JOBS) {
        set_last_error("midsx_gpu_batch_create: invalid argument (1..64 jobs)");
        return MIDSX_INVALID_ARG;
    }
    auto* b = new midsx_gpu_batch();
    auto guard = scope_exit([b] { midsx_gpu_batch_destroy(b); });
    b->tables = tables;
    b->n_jobs = n_jobs;
    b->host_prefix.push_back(0);
    for (int i = 0; i < n_jobs; ++i) {
        const midsx_batch_job& j = jobs[i];
        midsx_status cst = check_job(tables, j.phantom, j.source, j.tallies, "batch job " + std::to_string(i));
        if (cst != MIDSX_OK) return cst;
        // the tracking of the batch's launches is not known yet: the cells exist for any
        cst = ensure_cells(j.phantom);
        if (cst != MIDSX_OK) return cst;
        DevJob d;
        std::memset(&d, 0, sizeof(d));
        fill_job(d, j.phantom, j.source, j.tallies, j.seed, j.first_history, j.n_histories);
        b->host_jobs.push_back(d);
        b->tallies.push_back(j.tallies);
        b->host_prefix.push_back(b->host_prefix.back() + j.n_histories);
        b->max_energy = std::max(b->max_energy, j.source->max_energy);
    }
    if (!cuda_ok(cudaMalloc(&b->jobs, n_jobs * sizeof(DevJob)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&b->prefix, (n_jobs + 1) * sizeof(unsigned long long)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&b->words, (2 + kMaxBatchJobs) * sizeof(unsigned long long)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&b->rest_jobs, n_jobs * sizeof(DevJob)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&b->rest_prefix, (n_jobs + 1) * sizeof(unsigned long long)), "cudaMalloc"))
        return MIDSX_OOM;
    CUDA_TRY(cudaMemcpy(b->jobs, b->host_jobs.data(), n_jobs * sizeof(DevJob), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b->prefix, b->host_prefix.data(), (n_jobs + 1) * sizeof(unsigned long long),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(b->words, 0, (2 + kMaxBatchJobs) * sizeof(unsigned long long)));
    midsx_status sst = batch_split(b, 0);
    if (sst != MIDSX_OK) return sst;
    guard.release();
    *out = b;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_batch_set_own_launch(midsx_batch_h b, uint64_t min_histories) {
    if (!b) return MIDSX_INVALID_ARG;
    return batch_split(b, min_histories);
}

extern "C" midsx_status midsx_gpu_batch_destroy(midsx_batch_h b) {
    if (!b) return MIDSX_INVALID_ARG;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->jobs);
    cudaFree(b->prefix);
    cudaFree(b->words);
    cudaFree(b->rest_jobs);
    cudaFree(b->rest_prefix);
    delete b;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_batch_run(midsx_batch_h b, const midsx_run_config* cfg, void* stream) {
    if (!b || !cfg) return MIDSX_INVALID_ARG;
    midsx_status st = batch_check_precision(b, cfg->precision);
    if (st != MIDSX_OK) return st;
    st = batch_enqueue(b, *cfg, static_cast<cudaStream_t>(stream));
    if (st == MIDSX_OK)
        for (auto* t : b->tallies) t->precision = cfg->precision;
    return st;
}

extern "C" midsx_status midsx_gpu_batch_capture(midsx_batch_h b, const midsx_run_config* cfg, void* stream) {
    if (!b || !cfg || !stream) {
        set_last_error("midsx_gpu_batch_capture needs a non-default stream");
        return MIDSX_INVALID_ARG;
    }
    midsx_status st = batch_check_precision(b, cfg->precision);
    if (st != MIDSX_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // attributes and occupancy are resolved outside the capture
    RunParams P;
    batch_params(b, P, b->prefix, b->host_prefix.back());
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    midsx_status enq = batch_enqueue(b, *cfg, s);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (enq != MIDSX_OK) {
        if (graph) cudaGraphDestroy(graph);
        return enq;
    }
    if (!cuda_ok(e, "cudaStreamEndCapture")) return MIDSX_CUDA_ERROR;
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (!cuda_ok(e, "cudaGraphInstantiate")) return MIDSX_CUDA_ERROR;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = exec;
    b->graph_precision = cfg->precision;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_batch_replay(midsx_batch_h b, void* stream) {
    if (!b || !b->graph) {
        set_last_error("no captured graph");
        return MIDSX_INVALID_ARG;
    }
    midsx_status st = batch_check_precision(b, b->graph_precision);
    if (st != MIDSX_OK) return st;
    CUDA_TRY(cudaGraphLaunch(b->graph, static_cast<cudaStream_t>(stream)));
    for (auto* t : b->tallies) t->precision = b->graph_precision;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_batch_autotune(midsx_batch_h b, int32_t precision, uint64_t trial_histories,
                                                 midsx_run_config* best, double* best_rate, void* stream) {
    if (!b || !best || trial_histories < 1000) return MIDSX_INVALID_ARG;
    midsx_status st = batch_check_precision(b, precision);
    if (st != MIDSX_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // trial prefix: every job contributes in proportion to its size (at least one history)
    const double total = double(b->host_prefix.back());
    std::vector<unsigned long long> tp(1, 0);
    for (int i = 0; i < b->n_jobs; ++i) {
        double share = total > 0 ? double(b->host_jobs[size_t(i)].n) / total : 1.0 / b->n_jobs;
        unsigned long long k = std::max<unsigned long long>(1, (unsigned long long)(share * double(trial_histories)));
        tp.push_back(tp.back() + k);
    }
    unsigned long long* dprefix = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto guard = scope_exit([&] {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(dprefix);
    });
    CUDA_TRY(cudaMalloc(&dprefix, tp.size() * sizeof(unsigned long long)));
    CUDA_TRY(cudaMemcpy(dprefix, tp.data(), tp.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    // candidate launch shapes: both schedulers, their block sizes, occupancy and regroup
    // thresholds (the pool's blocks hold at most 128 threads)
    std::vector<midsx_run_config> cands;
    {
        midsx_run_config c;
        std::memset(&c, 0, sizeof(c));
        c.precision = precision;
        c.scheduler = MIDSX_SCHED_LANES;
        for (int bs : {128, 256})
            for (int ps : {0, 2, 4})
                for (int rg : {12, 16, 20, 24, 28})
                    for (int ch : {1, 4}) {
                        c.block_size = bs;
                        c.blocks_per_sm = ps;
                        c.regroup = rg;
                        c.chunk = ch;
                        cands.push_back(c);
                    }
        c.scheduler = MIDSX_SCHED_POOL;
        c.chunk = 0;
        bool spectra = false;
        for (auto* t : b->tallies) spectra |= t->spectra;
        if (!spectra)
            for (int bs : {64, 128})
                for (int sp : {1, 2})
                    for (int pr : {1, 8})
                        for (int rg : {24, 28, 32}) {
                            c.block_size = bs;
                            c.blocks_per_sm = 0;
                            c.steps_per_pass = sp;
                            c.pass_repeats = pr;
                            c.regroup = rg;
                            cands.push_back(c);
                        }
    }
    double best_r = -1;
    RunParams P;
    batch_params(b, P, dprefix, tp.back());
    for (int pass = 0; pass < 2 && st == MIDSX_OK; ++pass) {  // pass 0 warms the caches
        int last_sched = -1, last_block = -1;
        for (const midsx_run_config& cand : cands) {
            if (st != MIDSX_OK) break;
            if (launch_smem(P.n_jobs, true, precision == MIDSX_PREC_MIXED, cand.scheduler == MIDSX_SCHED_POOL,
                            b->tables->T.n_materials, cand.block_size) > b->tables->max_smem)
                continue;  // too many materials for this block size
            // one warm-up launch per scheduler and block size is enough
            if (pass == 0 && cand.scheduler == last_sched && cand.block_size == last_block) continue;
            last_sched = cand.scheduler;
            last_block = cand.block_size;
            if (!cuda_ok(cudaEventRecord(e0, s), "cudaEventRecord")) st = MIDSX_CUDA_ERROR;
            if (st == MIDSX_OK) st = launch_kernel(b->tables, P, cand, true, s);
            if (st == MIDSX_OK && !cuda_ok(cudaEventRecord(e1, s), "cudaEventRecord")) st = MIDSX_CUDA_ERROR;
            if (st == MIDSX_OK) st = wait_stream(stream);
            float ms = 0;
            if (st == MIDSX_OK && !cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime"))
                st = MIDSX_CUDA_ERROR;
            if (st == MIDSX_OK && pass == 1 && ms > 0) {
                double r = double(tp.back()) / (ms * 1e-3);
                if (r > best_r) {
                    best_r = r;
                    *best = cand;
                }
            }
        }
    }
    if (st != MIDSX_OK) return st;
    for (auto* t : b->tallies) {
        st = midsx_gpu_tallies_reset(t, stream);
        if (st != MIDSX_OK) return st;
    }
    if (best_rate) *best_rate = best_r;
    return wait_stream(stream);
}

// ==================================================================== stream helpers ===
extern "C" midsx_status midsx_gpu_stream_create(void** stream_out) {
    if (!stream_out) return MIDSX_INVALID_ARG;
    cudaStream_t s = nullptr;
    CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream_out = s;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_stream_destroy(void* stream) {
    if (!stream) return MIDSX_INVALID_ARG;
    CUDA_TRY(cudaStreamDestroy(static_cast<cudaStream_t>(stream)));
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_stream_synchronize(void* stream) { return wait_stream(stream); }

// ============================================== internal runtime for the request server ===
#include "runtime.h"

namespace midsx {
namespace rt {

size_t job_record_bytes() { return sizeof(DevJob); }

midsx_status pack_job(midsx_tables_h tables, midsx_phantom_h phantom, midsx_source_h source,
                      midsx_tallies_h tallies, uint64_t seed, uint64_t first, uint64_t n, int precision,
                      void* dst, uint32_t* step_cap) {
    if (!tables || !phantom || !source || !tallies || !dst) return MIDSX_INVALID_ARG;
    midsx_status st = check_job(tables, phantom, source, tallies, "job");
    if (st != MIDSX_OK) return st;
    if (precision != MIDSX_PREC_FP64 && precision != MIDSX_PREC_MIXED) {
        set_last_error("unknown precision");
        return MIDSX_INVALID_ARG;
    }
    if (precision == MIDSX_PREC_MIXED && source->max_energy > kMixedMaxEnergy) {
        set_last_error("the mixed form's fixed-point tallies take source energies up to 262144 eV");
        return MIDSX_INVALID_ARG;
    }
    if (tallies->precision >= 0 && tallies->precision != precision) {
        set_last_error("tallies hold results of the other precision");
        return MIDSX_INVALID_ARG;
    }
    if (!phantom->ids) {
        set_last_error("phantom not resident on the device");
        return MIDSX_INVALID_ARG;
    }
    const midsx_status cs = ensure_cells(phantom);  // the launch's tracking is not known here
    if (cs != MIDSX_OK) return cs;
    DevJob d;
    std::memset(&d, 0, sizeof(d));
    fill_job(d, phantom, source, tallies, seed, first, n);
    std::memcpy(dst, &d, sizeof(d));
    if (step_cap) *step_cap = d.step_cap;
    return MIDSX_OK;
}

bool tallies_spectra(midsx_tallies_h t) { return t && t->spectra; }

midsx_status launch_packed(midsx_tables_h tables, const void* dev_jobs, int n_jobs,
                           const unsigned long long* dev_prefix, unsigned long long total,
                           unsigned long long* dev_counter, const midsx_run_config& cfg, cudaStream_t s,
                           bool spectra, uint32_t step_cap) {
    if (!tables || !dev_jobs || !dev_prefix || !dev_counter || n_jobs < 1 || n_jobs > kMaxBatchJobs)
        return MIDSX_INVALID_ARG;
    if (cfg.precision != MIDSX_PREC_FP64 && cfg.precision != MIDSX_PREC_MIXED) {
        set_last_error("unknown precision");
        return MIDSX_INVALID_ARG;
    }
    if (total == 0) return MIDSX_OK;
    RunParams P;
    std::memset(&P, 0, sizeof(P));
    P.T = tables->T;
    P.jobs = static_cast<const DevJob*>(dev_jobs);
    P.n_jobs = n_jobs;
    P.prefix = dev_prefix;
    P.counter = dev_counter;
    P.total = total;
    P.spectra = spectra;
    P.server = 1;
    P.max_steps = int(std::min<uint32_t>(step_cap, 2147483647u));
    return launch_kernel(tables, P, cfg, true, s);
}

size_t tallies_footprint(size_t n_voxels, const midsx_tally_spec* specs, int n_specs, int dose_mode) {
    midsx_gpu_tallies t;
    if (tallies_layout(n_voxels, specs, n_specs, dose_mode, &t) != MIDSX_OK) return 0;
    return tallies_bytes(&t);
}

midsx_status tallies_create_async(midsx_phantom_h phantom, const midsx_tally_spec* specs, int n_specs,
                                  int dose_mode, cudaMemPool_t pool, cudaStream_t s, midsx_tallies_h* out) {
    if (!out || !pool || (dose_mode > 0 && !phantom)) return MIDSX_INVALID_ARG;
    auto* t = new midsx_gpu_tallies();
    midsx_status st = tallies_layout(phantom ? phantom->n_voxels : 0, specs, n_specs, dose_mode, t);
    if (st != MIDSX_OK) {
        delete t;
        return st;
    }
    // one allocation: statistics, accumulators, tally records, dose grid (8-byte words each)
    const size_t bytes = tallies_bytes(t);
    unsigned char* base = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&base), bytes, pool, s);
    if (e != cudaSuccess) {
        delete t;
        cuda_ok(e, "cudaMallocFromPoolAsync");
        return e == cudaErrorMemoryAllocation ? MIDSX_OOM : MIDSX_CUDA_ERROR;
    }
    size_t off = 0;
    t->stats = reinterpret_cast<unsigned long long*>(base + off);
    off += (kStCount + 1) * 8;
    if (t->acc_words) t->acc = reinterpret_cast<unsigned long long*>(base + off);
    off += t->acc_words * 8;
    if (!t->host_specs.empty()) t->specs = reinterpret_cast<DevTally*>(base + off);
    off += t->host_specs.size() * sizeof(DevTally);
    if (t->dose_stride) t->dose = reinterpret_cast<unsigned long long*>(base + off);
    off += t->n_voxels * size_t(t->dose_stride) * 8;
    if (dose_mode == MIDSX_DOSE_BATCHES) t->batch = reinterpret_cast<double*>(base + off);
    for (auto& d : t->host_specs) d.acc = t->acc + reinterpret_cast<size_t>(d.acc);
    bool ok = cuda_ok(cudaMemsetAsync(base, 0, bytes, s), "cudaMemsetAsync");
    // the records are copied from the handle's own host vector, which outlives the copy
    if (ok && !t->host_specs.empty())
        ok = cuda_ok(cudaMemcpyAsync(t->specs, t->host_specs.data(), t->host_specs.size() * sizeof(DevTally),
                                     cudaMemcpyHostToDevice, s),
                     "cudaMemcpyAsync");
    if (!ok) {
        cudaFreeAsync(base, s);
        delete t;
        return MIDSX_CUDA_ERROR;
    }
    t->pooled = true;
    *out = t;
    return MIDSX_OK;
}

void tallies_destroy_async(midsx_tallies_h t, cudaStream_t s) {
    if (!t) return;
    if (t->pooled)
        cudaFreeAsync(t->stats, s);  // the block starts at the statistics
    delete t;
}

void set_tallies_precision(midsx_tallies_h t, int precision) {
    if (t) t->precision = precision;
}

size_t phantom_voxels(midsx_phantom_h p) { return p ? p->n_voxels : 0; }

midsx_status phantom_download(midsx_phantom_h p, std::vector<uint8_t>& dense) {
    if (!p || !p->ids) return MIDSX_INVALID_ARG;
    dense.resize(p->n_voxels);
    CUDA_TRY(cudaMemcpy(dense.data(), p->ids, p->n_voxels, cudaMemcpyDeviceToHost));
    return MIDSX_OK;
}

uint8_t* phantom_storage(midsx_phantom_h p) { return p ? p->ids : nullptr; }

void phantom_bind(midsx_phantom_h p, uint8_t* dense_ids) {
    p->ids = dense_ids;
    p->G.ids = dense_ids;
}

void phantom_drop_storage(midsx_phantom_h p) {
    if (p && p->ids) cudaFree(p->ids);
    phantom_bind(p, nullptr);
}

void phantom_delete_handle(midsx_phantom_h p) { delete p; }

int tables_device(midsx_tables_h t) { return t ? t->device : 0; }

}  // namespace rt
}  // namespace midsx
