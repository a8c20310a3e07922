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
};

struct DevGeom {
    double domain[3], origin[3], spacing[3], ext[3];
    int dims[3];
    int background;
    const uint8_t* ids;
};

struct RunParams {
    DevTables T;
    DevGeom G;
    DevSource S;
    const DevTally* tallies;
    int n_tallies;
    int dose_stride;  // 0 = no dose tally, 1 = sum, 4 = count/sum/sumsq record
    unsigned long long* dose;
    unsigned long long* stats;
    uint64_t seed, first, n;
    int max_steps, max_trials;
    int regroup;    // lanes of a warp that wait for a real collision before the warp runs them
    double* trace;  // optional: energy deposited in grid voxels per history
};

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

template <>
struct Acc<true> {  // 64-bit fixed point, exact and order independent
    __device__ static void energy(unsigned long long* p, double v) {
        atomicAdd(p, (unsigned long long)__double2ll_rn(v * kFxEnergy));
    }
    __device__ static void energy2(unsigned long long* p, double v) {
        atomicAdd(p, (unsigned long long)__double2ll_rn(v * v * kFxEnergy2));
    }
    __device__ static void cosine(unsigned long long* p, double v) {
        atomicAdd(p, (unsigned long long)__double2ll_rn(v * kFxCosine));
    }
    __device__ static void cosine2(unsigned long long* p, double v) {
        atomicAdd(p, (unsigned long long)__double2ll_rn(v * v * kFxCosine));
    }
};

__device__ __forceinline__ void count1(unsigned long long* p) { atomicAdd(p, 1ull); }

// ------------------------------------------------------------------ tally scoring ---
// VectorVolumeQuantity / VectorSurfaceQuantity::measure: skip zero values, else add
// (count, sum, sum of squares) to the class.
template <bool MX>
__device__ __forceinline__ void vec_energy(unsigned long long* acc, int q, int cls, double v, uint32_t& words) {
    if (v == 0.0) return;
    unsigned long long* s = acc + q * 12 + cls * 3;
    count1(s);
    Acc<MX>::energy(s + 1, v);
    Acc<MX>::energy2(s + 2, v);
    ++words;  // one accumulator record (count, sum, sum of squares) updated
}

template <bool MX>
__device__ __forceinline__ void vec_cosine(unsigned long long* acc, int q, int cls, double v, uint32_t& words) {
    if (v == 0.0) return;
    unsigned long long* s = acc + q * 12 + cls * 3;
    count1(s);
    Acc<MX>::cosine(s + 1, v);
    Acc<MX>::cosine2(s + 2, v);
    ++words;
}

// One step segment [p0, p0 + s d) against every scalar/binned tally.
// cls0: class of the photon at the step start (surface quantities use initial_photon);
// cls1: class of final_photon (post-interaction counts if the step interacted, else
// a default Photon = primary), used by volume quantities.
template <typename R, bool MX>
__device__ __noinline__ void score_tallies(const RunParams& P, const V3<R>& p0, const V3<R>& d, R s, R E, int cls0,
                              int cls1, bool interact, R dep, uint32_t& words) {
    for (int ti = 0; ti < P.n_tallies; ++ti) {
        const DevTally& T = P.tallies[ti];
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
                lo[i] = (R(T.a[i]) - pp[i]) / dd[i];
                hi[i] = (R(T.b[i]) - pp[i]) / dd[i];
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
            vec_energy<MX>(acc, 0, cls1, double(e_dep), words);
            if (!counted) {
                vec_energy<MX>(acc, 1, cls1, double(E), words);
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
        V3<R> nrm = {R(T.norm[0]), R(T.norm[1]), R(T.norm[2])};
        R ec = dot(d, nrm);
        if (fabs_(ec) < R(kEps) || ec < R(0)) continue;
        V3<R> a = {R(T.a[0]), R(T.a[1]), R(T.a[2])};
        V3<R> w = {a.x - p0.x, a.y - p0.y, a.z - p0.z};
        R t = dot(w, nrm) / ec;
        if (t > s || t < R(0)) continue;
        V3<R> ip = {p0.x + t * d.x, p0.y + t * d.y, p0.z + t * d.z};
        V3<R> rel = {ip.x - a.x, ip.y - a.y, ip.z - a.z};
        if (kind == MIDSX_TALLY_SURFACE_DISC) {
            if (sqrt_(dot(rel, rel)) > R(T.radius)) continue;
        } else {
            V3<R> e1 = {R(T.b[0]), R(T.b[1]), R(T.b[2])};
            V3<R> e2 = {R(T.c[0]), R(T.c[1]), R(T.c[2])};
            R u = dot(e1, rel), v = dot(e2, rel);
            if (u < R(0) || u > R(T.e1e1) || v < R(0) || v > R(T.e2e2)) continue;
            if (kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
                int iu = int(u / R(T.e1e1) * R(T.nu));
                int iv = int(v / R(T.e2e2) * R(T.nv));
                iu = iu >= T.nu ? T.nu - 1 : iu;
                iv = iv >= T.nv ? T.nv - 1 : iv;
                unsigned long long* bin = T.acc + (size_t(iv) * T.nu + iu) * 8 + cls0 * 2;
                Acc<MX>::energy(bin, double(E));
                count1(bin + 1);
                ++words;
                continue;
            }
        }
        unsigned long long* acc = T.acc;
        vec_energy<MX>(acc, 0, cls0, double(E), words);
        vec_cosine<MX>(acc, 1, cls0, double(ec), words);
        count1(acc + 24 + cls0);
        ++words;
    }
}

// ------------------------------------------------------------------ source sampling ---
// PhotonSource::generatePhoton: position (PointGeometry), direction, energy, in that order.
template <typename R>
__device__ void sample_source(const DevSource& S, HistoryRng& rng, V3<R>& pos, V3<R>& dir, R& E) {
    pos = {R(S.pos[0]), R(S.pos[1]), R(S.pos[2])};
    V3<R> d;
    switch (S.dir_kind) {
        case MIDSX_DIR_BEAM:
            d = {R(S.a[0]) - pos.x, R(S.a[1]) - pos.y, R(S.a[2]) - pos.z};
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
            d = {R(S.a[0]) + a1 * R(S.b[0]) + a2 * R(S.c[0]) - pos.x,
                 R(S.a[1]) + a1 * R(S.b[1]) + a2 * R(S.c[1]) - pos.y,
                 R(S.a[2]) + a1 * R(S.b[2]) + a2 * R(S.c[2]) - pos.z};
            break;
        }
        default: {  // DISC
            R theta = R(2 * kPi) * uniform<R>(rng);
            R r = R(S.radius) * uniform<R>(rng);
            R st, ct;
            sincos_(theta, &st, &ct);
            d = {R(S.a[0]) + r * (R(S.b[0]) * ct + R(S.c[0]) * st) - pos.x,
                 R(S.a[1]) + r * (R(S.b[1]) * ct + R(S.c[1]) * st) - pos.y,
                 R(S.a[2]) + r * (R(S.b[2]) * ct + R(S.c[2]) * st) - pos.z};
            break;
        }
    }
    R nd = sqrt_(dot(d, d));
    dir = {d.x / nd, d.y / nd, d.z / nd};
    if (S.spec_kind == MIDSX_SPEC_MONO) {
        E = R(S.mono);
    } else {
        // DiscreteInversion::sample: energy[lower_bound(cdf, U)], clamped to the last bin
        double u = double(uniform<R>(rng));
        int idx = lower_index(S.cdf, 0, S.n_bins, u);
        if (idx >= S.n_bins) idx = S.n_bins - 1;
        E = R(S.energy[idx]);
    }
}

// -------------------------------------------------------------------- the kernel ---
#include "kernel_body.cuh"
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
    int* rows = nullptr;
    int* bk = nullptr;
    int32_t ids[MIDSX_MAX_MATERIALS];
    int device = 0;
    int sm_count = 0;
};

struct midsx_gpu_phantom {
    DevGeom G;
    uint8_t* ids = nullptr;
    size_t n_voxels = 0;
};

struct midsx_gpu_source {
    DevSource S;
    double* buf = nullptr;
    double max_energy = 0;
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
    int precision = -1;  // precision of the accumulated contents, -1 = empty
};

namespace {

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
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
    CUDA_TRY(cudaGetDevice(&h->device));
    CUDA_TRY(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device));
    size_t nd = size_t(blob->n_data), ni = size_t(blob->n_idata);
    if (!cuda_ok(cudaMalloc(&h->d, nd * sizeof(double)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&h->f, nd * sizeof(float)), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&h->rows, ni * sizeof(int)), "cudaMalloc")) {
        cudaFree(h->d);
        cudaFree(h->f);
        cudaFree(h->rows);
        delete h;
        return MIDSX_OOM;
    }
    std::vector<int> rows(ni);
    for (size_t i = 0; i < ni; ++i) rows[i] = int(blob->idata[i]);
    CUDA_TRY(cudaMemcpy(h->d, blob->data, nd * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->rows, rows.data(), ni * sizeof(int), cudaMemcpyHostToDevice));
    f64_to_f32_kernel<<<unsigned((nd + 255) / 256), 256>>>(h->d, h->f, nd);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    DevTables& T = h->T;
    T.d = h->d;
    T.f = h->f;
    T.rows = h->rows;
    T.n_materials = blob->n_materials;
    T.alpha = kMec2 / (std::sqrt(2.0) * 4.135667662e-15 * 299792458E2 * 1E8);
    T.e_max = blob->e_max;
    fill_lin(T.majorant, blob->majorant);
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
    if (!cuda_ok(cudaMalloc(&h->bk, bb.data.size() * sizeof(int)), "cudaMalloc")) {
        midsx_gpu_tables_destroy(h);
        return MIDSX_OOM;
    }
    CUDA_TRY(cudaMemcpy(h->bk, bb.data.data(), bb.data.size() * sizeof(int), cudaMemcpyHostToDevice));
    T.bk = h->bk;
    *out = h;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tables_destroy(midsx_tables_h t) {
    if (!t) return MIDSX_INVALID_ARG;
    cudaFree(t->d);
    cudaFree(t->f);
    cudaFree(t->rows);
    cudaFree(t->bk);
    delete t;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_phantom_create(midsx_tables_h tables, const midsx_geometry_spec* g,
                                                 const uint8_t* ids, midsx_phantom_h* out) {
    if (!tables || !g || !ids || !out) return MIDSX_INVALID_ARG;
    for (int i = 0; i < 3; ++i) {
        if (g->dims[i] < 1 || !(g->spacing[i] > 0) || !(g->domain[i] > 0)) {
            set_last_error("midsx_gpu_phantom_create: bad geometry");
            return MIDSX_INVALID_ARG;
        }
    }
    uint8_t lut[256];
    std::memset(lut, 0xFF, sizeof(lut));
    int bg = -1;
    for (int m = 0; m < tables->T.n_materials; ++m) {
        lut[tables->ids[m] & 0xFF] = uint8_t(m);
        if (tables->ids[m] == g->background_id) bg = m;
    }
    if (bg < 0) {
        set_last_error("background material not in tables");
        return MIDSX_NOT_FOUND;
    }
    auto* p = new midsx_gpu_phantom();
    p->n_voxels = size_t(g->dims[0]) * g->dims[1] * g->dims[2];
    uint8_t *raw = nullptr, *dlut = nullptr;
    int* bad = nullptr;
    if (!cuda_ok(cudaMalloc(&p->ids, p->n_voxels), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&raw, p->n_voxels), "cudaMalloc") || !cuda_ok(cudaMalloc(&dlut, 256), "cudaMalloc") ||
        !cuda_ok(cudaMalloc(&bad, sizeof(int)), "cudaMalloc")) {
        cudaFree(p->ids);
        cudaFree(raw);
        cudaFree(dlut);
        cudaFree(bad);
        delete p;
        return MIDSX_OOM;
    }
    CUDA_TRY(cudaMemcpy(raw, ids, p->n_voxels, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dlut, lut, 256, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(bad, 0, sizeof(int)));
    remap_kernel<<<tables->sm_count * 8, 256>>>(raw, p->ids, dlut, p->n_voxels, bad);
    CUDA_TRY(cudaGetLastError());
    int hbad = 0;
    CUDA_TRY(cudaMemcpy(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(raw);
    cudaFree(dlut);
    cudaFree(bad);
    if (hbad) {
        cudaFree(p->ids);
        delete p;
        set_last_error("voxel material id not among the tables' materials");
        return MIDSX_NOT_FOUND;
    }
    DevGeom& G = p->G;
    for (int i = 0; i < 3; ++i) {
        G.domain[i] = g->domain[i];
        G.origin[i] = g->origin[i];
        G.spacing[i] = g->spacing[i];
        G.dims[i] = g->dims[i];
        G.ext[i] = double(g->dims[i]) * g->spacing[i];  // VoxelGrid::setDimSpace
    }
    G.background = bg;
    G.ids = p->ids;
    *out = p;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_phantom_destroy(midsx_phantom_h p) {
    if (!p) return MIDSX_INVALID_ARG;
    cudaFree(p->ids);
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
            delete s;
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
            delete s;
            set_last_error("bad spectrum");
            return MIDSX_INVALID_ARG;
        }
        // DiscreteInversion: normalise (if the sum differs from 1) then cumulative sum
        std::vector<double> h(2 * size_t(nb));
        double sum = 0;
        for (int i = 0; i < nb; ++i) sum += spec->bin_prob[i];
        double acc = 0;
        for (int i = 0; i < nb; ++i) {
            double p = (sum != 1.0) ? spec->bin_prob[i] / sum : spec->bin_prob[i];
            acc = (i == 0) ? p : acc + p;
            h[i] = spec->bin_energy[i];
            h[nb + i] = acc;
            s->max_energy = std::max(s->max_energy, spec->bin_energy[i]);
        }
        CUDA_TRY(cudaMalloc(&s->buf, h.size() * sizeof(double)));
        CUDA_TRY(cudaMemcpy(s->buf, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        S.n_bins = nb;
        S.energy = s->buf;
        S.cdf = s->buf + nb;
    } else {
        if (!(spec->mono_energy > 0)) {
            delete s;
            set_last_error("bad mono energy");
            return MIDSX_INVALID_ARG;
        }
        s->max_energy = spec->mono_energy;
    }
    *out = s;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_source_destroy(midsx_source_h s) {
    if (!s) return MIDSX_INVALID_ARG;
    cudaFree(s->buf);
    delete s;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tallies_create(midsx_phantom_h phantom, const midsx_tally_spec* specs,
                                                 int32_t n_specs, int32_t dose_mode, midsx_tallies_h* out) {
    if (!out || n_specs < 0 || n_specs > MIDSX_MAX_TALLIES || (n_specs > 0 && !specs) || dose_mode < 0 ||
        dose_mode > 2 || (dose_mode > 0 && !phantom)) {
        set_last_error("midsx_gpu_tallies_create: invalid argument");
        return MIDSX_INVALID_ARG;
    }
    auto* t = new midsx_gpu_tallies();
    t->dose_mode = dose_mode;
    t->dose_stride = dose_mode == 0 ? 0 : (dose_mode == 1 ? 1 : 4);
    t->n_voxels = phantom ? phantom->n_voxels : 0;
    size_t words = 0;
    for (int i = 0; i < n_specs; ++i) {
        const midsx_tally_spec& s = specs[i];
        DevTally d;
        std::memset(&d, 0, sizeof(d));
        d.kind = s.kind;
        d.nu = s.nu;
        d.nv = s.nv;
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
                delete t;
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
                delete t;
                set_last_error("binned tally needs nu, nv >= 1");
                return MIDSX_INVALID_ARG;
            }
        } else if (s.kind != MIDSX_TALLY_VOLUME_AACUBOID) {
            delete t;
            set_last_error("unknown tally kind");
            return MIDSX_INVALID_ARG;
        }
        d.acc = reinterpret_cast<unsigned long long*>(words);  // offset, fixed below
        words += (s.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) ? size_t(s.nu) * s.nv * 8 : kScalarWords;
        t->host_specs.push_back(d);
    }
    t->acc_words = words;
    if (!cuda_ok(cudaMalloc(&t->stats, kStCount * sizeof(unsigned long long)), "cudaMalloc") ||
        (words && !cuda_ok(cudaMalloc(&t->acc, words * 8), "cudaMalloc")) ||
        (n_specs && !cuda_ok(cudaMalloc(&t->specs, n_specs * sizeof(DevTally)), "cudaMalloc")) ||
        (t->dose_stride &&
         !cuda_ok(cudaMalloc(&t->dose, t->n_voxels * t->dose_stride * sizeof(unsigned long long)), "cudaMalloc"))) {
        midsx_gpu_tallies_destroy(t);
        return MIDSX_OOM;
    }
    for (auto& d : t->host_specs) d.acc = t->acc + reinterpret_cast<size_t>(d.acc);
    if (n_specs)
        CUDA_TRY(cudaMemcpy(t->specs, t->host_specs.data(), n_specs * sizeof(DevTally), cudaMemcpyHostToDevice));
    midsx_status st = midsx_gpu_tallies_reset(t, nullptr);
    if (st != MIDSX_OK) return st;
    CUDA_TRY(cudaDeviceSynchronize());
    *out = t;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_tallies_destroy(midsx_tallies_h t) {
    if (!t) return MIDSX_INVALID_ARG;
    cudaFree(t->dose);
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
    t->precision = -1;
    return MIDSX_OK;
}

namespace {

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
    if (source->max_energy > tables->T.e_max) {
        set_last_error("source energy above the tables' e_max");
        return MIDSX_TABLE_RANGE;
    }
    if (cfg->n_histories == 0) return MIDSX_OK;
    RunParams P;
    std::memset(&P, 0, sizeof(P));
    P.T = tables->T;
    P.G = phantom->G;
    P.S = source->S;
    P.tallies = tallies->specs;
    P.n_tallies = int(tallies->host_specs.size());
    P.dose_stride = tallies->dose_stride;
    P.dose = tallies->dose;
    P.stats = tallies->stats;
    P.seed = cfg->seed;
    P.first = cfg->first_history;
    P.n = cfg->n_histories;
    P.max_steps = cfg->max_steps > 0 ? cfg->max_steps : 100000;
    P.max_trials = cfg->max_compton_trials > 0 ? cfg->max_compton_trials : 100000;
    P.trace = trace;
    P.regroup = cfg->regroup > 0 ? std::min(cfg->regroup, 32) : 16;
    const bool mixed = cfg->precision == MIDSX_PREC_MIXED;
    int block = cfg->block_size > 0 ? cfg->block_size : 256;
    if (block > 256 || block % 32) {
        set_last_error("block_size must be a multiple of 32 up to 256");
        return MIDSX_INVALID_ARG;
    }
    size_t smem = size_t(2) * tables->T.n_materials * block * (mixed ? 4 : 8);
    if (smem > 48 * 1024) {
        if (mixed)
            CUDA_TRY(cudaFuncSetAttribute(transport_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        else
            CUDA_TRY(cudaFuncSetAttribute(transport_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    }
    int per_sm = cfg->blocks_per_sm;
    if (per_sm <= 0) {
        if (mixed)
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<float>, block, smem));
        else
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<double>, block, smem));
        per_sm = std::max(per_sm, 1);
    }
    uint64_t want = (P.n + block - 1) / block;
    uint64_t grid = std::min<uint64_t>(want, uint64_t(tables->sm_count) * per_sm);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mixed)
        transport_kernel<float><<<unsigned(grid), block, smem, s>>>(P);
    else
        transport_kernel<double><<<unsigned(grid), block, smem, s>>>(P);
    CUDA_TRY(cudaGetLastError());
    tallies->precision = cfg->precision;
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

extern "C" midsx_status midsx_gpu_fetch_dose(midsx_tallies_h t, double* sum, double* sumsq, double* count,
                                             void* stream) {
    if (!t || !t->dose) return MIDSX_INVALID_ARG;
    if ((sumsq || count) && t->dose_stride < 4) return MIDSX_INVALID_ARG;
    size_t n = t->n_voxels, w = size_t(t->dose_stride);
    std::vector<unsigned long long> h(n * w);
    CUDA_TRY(cudaMemcpyAsync(h.data(), t->dose, n * w * 8, cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
    midsx_status st = wait_stream(stream);
    if (st != MIDSX_OK) return st;
    const bool mixed = t->precision == MIDSX_PREC_MIXED;
    for (size_t i = 0; i < n; ++i) {
        const unsigned long long* r = &h[i * w];
        if (sum) {
            if (mixed) {
                sum[i] = fx_signed(r[0], kFxEnergy);
            } else {
                double d;
                std::memcpy(&d, &r[0], 8);
                sum[i] = d;
            }
        }
        if (sumsq) {
            if (mixed) {
                sumsq[i] = double(r[1]) / kFxEnergy2;
            } else {
                double d;
                std::memcpy(&d, &r[1], 8);
                sumsq[i] = d;
            }
        }
        if (count) count[i] = double(r[2]);
    }
    return MIDSX_OK;
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
    if (!tables || !phantom || !source || !cfg || !hist_dep || cfg->n_histories == 0 ||
        cfg->n_histories > (uint64_t(1) << 28))
        return MIDSX_INVALID_ARG;
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
static_assert(kStCount * sizeof(unsigned long long) <= kNoAllocStatsBytes, "statistics fit the scratch header");
}  // namespace

static __device__ __align__(256) unsigned char midsx_noalloc_scratch[kNoAllocStatsBytes +
                                                                      kNoAllocMaxHistories * sizeof(double)];

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_address[256] = {};

// Device address of midsx_noalloc_scratch on the current device.  Host code sees only a
// host-side stand-in under that name, so the address is asked from the runtime once per
// device, with that device current, and kept.
midsx_status noalloc_scratch(void** out) {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_last_error("device ordinal out of range");
        return MIDSX_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_address[dev]) {
        void* p = nullptr;
        if (!cuda_ok(cudaGetSymbolAddress(&p, midsx_noalloc_scratch), "cudaGetSymbolAddress")) return MIDSX_CUDA_ERROR;
        g_noalloc_address[dev] = p;
    }
    *out = g_noalloc_address[dev];
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
    cudaFree(d0);
    cudaFree(d1);
    return MIDSX_OK;
}

extern "C" midsx_status midsx_gpu_table_index(midsx_tables_h tables, int32_t material, const double* e, int64_t n,
                                              int64_t* idx) {
    if (!tables || !e || !idx || n <= 0 || material < 0 || material >= tables->T.n_materials || n > (int64_t(1) << 28))
        return MIDSX_INVALID_ARG;
    double* de = nullptr;
    int64_t* di = nullptr;
    CUDA_TRY(cudaMalloc(&de, n * sizeof(double)));
    CUDA_TRY(cudaMalloc(&di, 6 * n * sizeof(int64_t)));
    CUDA_TRY(cudaMemcpy(de, e, n * sizeof(double), cudaMemcpyHostToDevice));
    index_kernel<<<unsigned((n + 255) / 256), 256>>>(tables->T, material, de, n, di);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpy(idx, di, 6 * n * sizeof(int64_t), cudaMemcpyDeviceToHost));
    cudaFree(de);
    cudaFree(di);
    return MIDSX_OK;
}
