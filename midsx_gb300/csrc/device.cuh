// device.cuh - device functions of the photon-history transport kernels.
//
// Every function states the reference code it restates (paths inside MIDSX):
//   free path, delta test            src/MIDSX/Core/physics_engine.cpp:170-183
//   interaction type                 src/MIDSX/Core/physics_engine.cpp:82-109
//   photoelectric / Rayleigh / Compton
//                                    src/MIDSX/Core/photon_interactions.cpp:43-141
//   direction rotation               src/MIDSX/Core/particle.cpp:7-45
//   source sampling                  src/MIDSX/Core/source.cpp:44-155,
//                                    src/MIDSX/Core/probability_dist.cpp:18-28
//   surface / volume tallies         src/MIDSX/Core/surface_tally.cpp:5-112,
//                                    src/MIDSX/Core/volume_tally.cpp:5-91
//   quantity classification          src/MIDSX/Core/volume_quantity.cpp:53-67,
//                                    src/MIDSX/Core/surface_quantity.cpp:49-63
#pragma once
#include <stdint.h>

#include "../../include/midsx_gpu.h"
#include "lookup.h"

namespace midsx {

// -------------------------------------------------------------------- constants ---
// include/MIDSX/Core/constants.h:13-23
constexpr double kPi = 3.14159265358979323846;
constexpr double kMec2 = 0.51099895000E6;  // eV
constexpr double kEps = 1e-9;
// ALPHA = mec2 / (sqrt(2) h c 1e8), 1/Angstrom; evaluated on the host in FP64 and
// passed to the kernels.

// ----------------------------------------------------------------- Philox4x32-10 ---
// Counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
// as easy as 1, 2, 3" (SC'11): 10 rounds of the Philox S-box with multipliers
// 0xD2511F53 / 0xCD9E8D57 and Weyl key increments 0x9E3779B9 / 0xBB67AE85.
struct Philox4 {
    uint32_t v[4];
};

MIDSX_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
    lo = a * b;
    hi = __umulhi(a, b);
#else
    uint64_t p = uint64_t(a) * uint64_t(b);
    lo = uint32_t(p);
    hi = uint32_t(p >> 32);
#endif
}

// Out of line: the event code draws from many call sites, and one copy of the ten rounds
// instead of one per site measured +1.2 % (instruction fetch is the kernel's largest stall).
// The photon-pool kernel's Woodcock steps draw through philox4x32_10_rk, inlined.
__host__ __device__ __noinline__ inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                             uint32_t k0, uint32_t k1) {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, x0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, x2, hi1, lo1);
        uint32_t y0 = hi1 ^ x1 ^ k0;
        uint32_t y2 = hi0 ^ x3 ^ k1;
        x0 = y0;
        x1 = lo1;
        x2 = y2;
        x3 = lo0;
    }
    Philox4 o;
    o.v[0] = x0;
    o.v[1] = x1;
    o.v[2] = x2;
    o.v[3] = x3;
    return o;
}

// The same generator with the key schedule precomputed: rk[2r], rk[2r + 1] are round r's
// keys (philox_round_keys).  A launch of one seed passes them as kernel parameters, so the
// rounds read them from the constant bank instead of adding the Weyl increments per block.
MIDSX_HD void philox_round_keys(uint64_t seed, uint32_t* rk) {
    uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        rk[2 * r] = k0;
        rk[2 * r + 1] = k1;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

MIDSX_HD Philox4 philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const uint32_t (&rk)[20]) {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, x0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, x2, hi1, lo1);
        uint32_t y0 = hi1 ^ x1 ^ rk[2 * r];
        uint32_t y2 = hi0 ^ x3 ^ rk[2 * r + 1];
        x0 = y0;
        x1 = lo1;
        x2 = y2;
        x3 = lo0;
    }
    Philox4 o;
    o.v[0] = x0;
    o.v[1] = x1;
    o.v[2] = x2;
    o.v[3] = x3;
    return o;
}

// One random stream per history h, key (seed_lo, seed_hi), with two kinds of draws:
//   * event draws (source, interaction type, samplers, azimuths): draw n is the 32-bit word
//     (n & 3) of Philox block (n >> 2, h_lo, h_hi, 0); every interaction starts a new block
//     (align_event: n rounded up to a multiple of 4), so its draws never need words cached
//     by an earlier event (a parked photon's lane holds another photon's in between);
//   * Woodcock-step draws: the step's free-path and delta-test uniforms are the 32-bit word
//     pair (2 (i & 1), 2 (i & 1) + 1) of block (i >> 1, h_lo, h_hi, 1 + n), n the event
//     draws so far (constant along a flight segment - the steps between two interactions -
//     and different for every segment), i = (the history's Woodcock steps so far) + p, p the
//     parity of that count at the segment's start, so that a segment starts on a block
//     boundary and two steps share one block.  The photon-pool kernel's passes of two steps
//     compute one block per pass.
// A draw is handed out as the 64-bit value word << 32: the FP64 path takes its top 53 bits
// (32 random, so a free path is cut at -ln 2^-32 = 22.2 mean free paths, which a step passes
// with probability 2.3e-10), the FP32 path its top 24 bits, so both precisions consume
// identical streams.  Four event draws per block instead of two, and two steps per block
// instead of one: +3.0 % and +2.6 % on the cone-beam dose workload.
struct HistoryRng {
    uint32_t k0, k1, h0, h1;
    uint32_t n;
    uint32_t b1, b2, b3;  // words 1-3 of the current event block

    MIDSX_HD void init(uint64_t seed, uint64_t history) {
        k0 = uint32_t(seed);
        k1 = uint32_t(seed >> 32);
        h0 = uint32_t(history);
        h1 = uint32_t(history >> 32);
        n = 0;
        b1 = b2 = b3 = 0;
    }
    MIDSX_HD uint64_t next64() {
        uint32_t r;
        const uint32_t k = n & 3u;
        if (k == 0u) {
            const Philox4 w = philox4x32_10(n >> 2, h0, h1, 0u, k0, k1);
            r = w.v[0];
            b1 = w.v[1];
            b2 = w.v[2];
            b3 = w.v[3];
        } else {
            r = k == 1u ? b1 : (k == 2u ? b2 : b3);
        }
        ++n;
        return uint64_t(r) << 32;
    }
    // The Philox block of Woodcock step index i (the step stream above), with the key
    // schedule precomputed (philox_round_keys of the seed) or computed as it goes.
    MIDSX_HD Philox4 step_block_rk(uint32_t i, const uint32_t (&rk)[20]) const {
        return philox4x32_10_rk(i >> 1, h0, h1, 1u + n, rk);
    }
    MIDSX_HD Philox4 step_block(uint32_t i) const { return philox4x32_10(i >> 1, h0, h1, 1u + n, k0, k1); }
    // An interaction's first event draw starts a new block.
    MIDSX_HD void align_event() { n = (n + 3u) & ~3u; }
};

// Uniform in (0, 1].
MIDSX_HD double to_uniform(uint64_t r, double) { return double((r >> 11) + 1) * 0x1.0p-53; }
MIDSX_HD float to_uniform(uint64_t r, float) { return float(uint32_t(r >> 40) + 1u) * 0x1.0p-24f; }

template <typename R>
MIDSX_HD R uniform(HistoryRng& rng) {
    return to_uniform(rng.next64(), R(0));
}

// ------------------------------------------------------------------------ vectors ---
template <typename R>
struct V3 {
    R x, y, z;
};

template <typename R>
MIDSX_HD R dot(const V3<R>& a, const V3<R>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

MIDSX_HD double acos_(double v) { return acos(v); }
MIDSX_HD float acos_(float v) { return acosf(v); }
MIDSX_HD void sincos_(double v, double* s, double* c) {
#if defined(__CUDA_ARCH__)
    sincos(v, s, c);
#else
    *s = sin(v);
    *c = cos(v);
#endif
}
MIDSX_HD void sincos_(float v, float* s, float* c) {
#if defined(__CUDA_ARCH__)
    sincosf(v, s, c);
#else
    *s = sinf(v);
    *c = cosf(v);
#endif
}
MIDSX_HD double fabs_(double v) { return fabs(v); }
MIDSX_HD float fabs_(float v) { return fabsf(v); }

// ParticleHelpers::rotateDirection: rotate v by theta about the unit vector perpendicular
// to v built from its smallest component, then by phi about v, as the quaternion product
// q = q_phi * q_theta applied as q v q^-1 (particle.cpp:7-45).
template <typename R>
MIDSX_HD V3<R> rotate_half(const V3<R>& v, R st, R ct, R sp, R cp);

template <typename R>
MIDSX_HD V3<R> rotate_direction(const V3<R>& v, R theta, R phi) {
    R st, ct, sp, cp;
    sincos_(theta / R(2), &st, &ct);
    sincos_(phi / R(2), &sp, &cp);
    return rotate_half(v, st, ct, sp, cp);
}

// New direction at polar cosine mu and azimuth 2 pi u: rotateDirection with theta = acos mu
// and phi = 2 pi u.  The FP64 form evaluates acos and the half-angle sincos as the reference
// does; the FP32 form takes the half angles from mu and u directly - cos(theta/2) =
// sqrt((1 + mu) / 2), sin(theta/2) = sqrt((1 - mu) / 2), (sin, cos)(phi/2) = sincospi(u) -
// with no acos and no trigonometric range reduction.  A mu outside [-1, 1] gives a NaN
// direction in both forms.
template <typename R>
MIDSX_HD V3<R> scatter_direction(const V3<R>& v, R mu, R u) {
    if constexpr (sizeof(R) == 8) {
        return rotate_direction(v, acos_(mu), R(2 * kPi) * u);
    } else {
        const R st = sqrt_((R(1) - mu) * R(0.5)), ct = sqrt_((R(1) + mu) * R(0.5));
        R sp, cp;
#if defined(__CUDA_ARCH__)
        sincospif(u, &sp, &cp);
#else
        sp = std::sin(R(kPi) * u);
        cp = std::cos(R(kPi) * u);
#endif
        return rotate_half(v, st, ct, sp, cp);
    }
}

// rotateDirection from the half-angle sines and cosines of theta and phi.
template <typename R>
MIDSX_HD V3<R> rotate_half(const V3<R>& v, R st, R ct, R sp, R cp) {
    V3<R> p;
    R ax = fabs_(v.x), ay = fabs_(v.y), az = fabs_(v.z);
    if (ax <= ay && ax <= az) {
        p = {R(0), -v.z, v.y};
    } else if (ay <= az) {
        p = {v.z, R(0), -v.x};
    } else {
        p = {-v.y, v.x, R(0)};
    }
    R pn = sqrt_(dot(p, p));
    if (pn > R(0)) {  // one division
        const R ipn = R(1) / pn;
        p.x *= ipn;
        p.y *= ipn;
        p.z *= ipn;
    }
    // q_theta = (ct, p st), q_phi = (cp, v sp)
    R tw = ct, tx = p.x * st, ty = p.y * st, tz = p.z * st;
    R fw = cp, fx = v.x * sp, fy = v.y * sp, fz = v.z * sp;
    // q = q_phi * q_theta
    R qw = fw * tw - fx * tx - fy * ty - fz * tz;
    R qx = fw * tx + fx * tw + fy * tz - fz * ty;
    R qy = fw * ty - fx * tz + fy * tw + fz * tx;
    R qz = fw * tz + fx * ty - fy * tx + fz * tw;
    // r = q * (0, v)
    R rw = -qx * v.x - qy * v.y - qz * v.z;
    R rx = qw * v.x + qy * v.z - qz * v.y;
    R ry = qw * v.y - qx * v.z + qz * v.x;
    R rz = qw * v.z + qx * v.y - qy * v.x;
    // q^-1 = conj(q) / |q|^2
    R n2 = qw * qw + qx * qx + qy * qy + qz * qz;
    const R in2 = R(1) / n2;  // one division
    const R iw = qw * in2, ix = -qx * in2, iy = -qy * in2, iz = -qz * in2;
    // out = r * q^-1 (vector part)
    V3<R> o;
    o.x = rw * ix + rx * iw + ry * iz - rz * iy;
    o.y = rw * iy - rx * iz + ry * iw + rz * ix;
    o.z = rw * iz + rx * iy - ry * ix + rz * iw;
    return o;
}

// ----------------------------------------------------------------- device tables ---
// Each searched node array carries two bucket tables (lookup.h, BucketSpec): one for FP64
// queries against the FP64 nodes (bk_d) and one for FP32 queries against the FP32 nodes
// (bk_f), offsets into DevTables::bk.  kind 0 = energy (eV), 1 = momentum transfer (1/A).
struct DevLin {
    int x, lx, ly, n;
    int bk_d, bk_f, kind;
};
struct DevSpline {
    int knot_e, knot_u, ctrl, n_ctrl, degree;
    int bk_d, bk_f;
    double lx_min, lx_max;
    float f_lx_min, f_lx_max;  // FP32 copies for the mixed form
};
struct DevRita {
    int energy, log_energy, row_start, x, y, a, b, n_energy;
    int bk_d, bk_f;
};
struct DevMaterial {
    DevLin total, sfunc;
    DevSpline coh, incoh;
    DevRita rita;
};
struct DevTables {
    const double* d;     // FP64 data (blob layout)
    const float* f;      // FP32 copy, same offsets
    const float* fs;     // FP32 LogLogLinear slopes at the ly offsets (lin_eval_slope_at_log)
    const double* ds;    // the same slopes in FP64: the quotient the FP64 lookup would compute
    const int* rows;     // RITA row starts
    const int* bk;       // bucket tables of every searched node array
    BucketSpec bs[2][2];  // [kind][0 = FP64 query, 1 = FP32 query]
    int n_materials;
    double alpha;        // 1/Angstrom per unit k
    float alpha_f;       // FP32 copy
    double e_max;
    DevLin majorant;
    DevMaterial mat[MIDSX_MAX_MATERIALS];
};

template <typename R>
MIDSX_HD const R* tab(const DevTables& t);
template <>
MIDSX_HD const double* tab<double>(const DevTables& t) {
    return t.d;
}
template <>
MIDSX_HD const float* tab<float>(const DevTables& t) {
    return t.f;
}
// LogLogLinear slopes of the working precision (tables_create: FP64 quotients, and their
// FP32 roundings)
template <typename R>
MIDSX_HD const R* slopes(const DevTables& t);
template <>
MIDSX_HD const double* slopes<double>(const DevTables& t) {
    return t.ds;
}
template <>
MIDSX_HD const float* slopes<float>(const DevTables& t) {
    return t.fs;
}

template <typename R>
MIDSX_HD const int* buckets(const DevTables& t, int bk_d, int bk_f) {
    return t.bk + (sizeof(R) == 8 ? bk_d : bk_f);
}
template <typename R>
MIDSX_HD const BucketSpec& bspec(const DevTables& t, int kind) {
    return t.bs[kind][sizeof(R) == 8 ? 0 : 1];
}

// LogLogLinear interval index with the bucketed search (same result as lin_index).
template <typename R>
MIDSX_HD int lin_index_bk(const DevTables& t, const DevLin& L, R q) {
    const R* x = tab<R>(t) + L.x;
    if (q <= x[0]) return 0;
    if (q >= x[L.n - 1]) return L.n;
    const int* st = buckets<R>(t, L.bk_d, L.bk_f);
    int b = bucket_of(q, bspec<R>(t, L.kind));
    return upper_index(x, st[b], st[b + 1], q);
}

template <typename R>
MIDSX_HD R lin_lookup(const DevTables& t, const DevLin& L, R q) {
    const R* D = tab<R>(t);
    const int idx = lin_index_bk<R>(t, L, q);
    // slopes from the host: FP32 rounded once from FP64; FP64 the same quotient the device
    // would divide out per lookup, bit for bit (one division less per FP64 lookup)
    if (idx == 0 || idx >= L.n) return lin_eval_slope_at_log(D + L.lx, D + L.ly, slopes<R>(t) + L.ly, L.n, idx, R(0));
    return lin_eval_slope_at_log(D + L.lx, D + L.ly, slopes<R>(t) + L.ly, L.n, idx, log10_(q));
}

// Knot span with the bucketed search (same result as spline_span).
template <typename R>
MIDSX_HD int spline_span_bk(const DevTables& t, const DevSpline& S, R e) {
    const R* ke = tab<R>(t) + S.knot_e;
    if (e <= ke[0]) return S.degree;
    const int* st = buckets<R>(t, S.bk_d, S.bk_f);
    int b = bucket_of(e, bspec<R>(t, 0));
    return upper_index(ke, st[b], st[b + 1], e) - 1;
}

template <typename R>
MIDSX_HD R spline_lookup(const DevTables& t, const DevSpline& S, R e) {
    const R* D = tab<R>(t);
    int span = spline_span_bk<R>(t, S, e);
    R lo, hi;
    if constexpr (sizeof(R) == 8) {
        lo = S.lx_min;
        hi = S.lx_max;
    } else {
        lo = S.f_lx_min;
        hi = S.f_lx_max;
    }
    return spline_eval_at(D + S.knot_u, D + S.ctrl, S.degree, span, lo, hi, e);
}

// An energy query shared by several energy tables: the energy, its log10 and its bucket
// (every energy table uses the same slice parametrisation), computed once.
template <typename R>
struct EnergyKey {
    R q, lq;
    int b;
};

template <typename R>
MIDSX_HD EnergyKey<R> energy_key(const DevTables& t, R q) {
    return {q, log10_(q), bucket_of(q, bspec<R>(t, 0))};
}

// lin_lookup of an energy table (kind 0) with a precomputed key: same index, same value.
template <typename R>
MIDSX_HD R lin_lookup_key(const DevTables& t, const DevLin& L, const EnergyKey<R>& k) {
    const R* D = tab<R>(t);
    const R* x = D + L.x;
    int idx;
    if (k.q <= x[0]) {
        idx = 0;
    } else if (k.q >= x[L.n - 1]) {
        idx = L.n;
    } else {
        const int* st = buckets<R>(t, L.bk_d, L.bk_f);
        idx = upper_index(x, st[k.b], st[k.b + 1], k.q);
    }
    return lin_eval_slope_at_log(D + L.lx, D + L.ly, slopes<R>(t) + L.ly, L.n, idx, k.lq);
}

// spline_lookup with a precomputed key: same span, same value.
template <typename R>
MIDSX_HD R spline_lookup_key(const DevTables& t, const DevSpline& S, const EnergyKey<R>& k) {
    const R* D = tab<R>(t);
    const R* ke = D + S.knot_e;
    int span;
    if (k.q <= ke[0]) {
        span = S.degree;
    } else {
        const int* st = buckets<R>(t, S.bk_d, S.bk_f);
        span = upper_index(ke, st[k.b], st[k.b + 1], k.q) - 1;
    }
    R lo, hi;
    if constexpr (sizeof(R) == 8) {
        lo = S.lx_min;
        hi = S.lx_max;
    } else {
        lo = S.f_lx_min;
        hi = S.f_lx_max;
    }
    return spline_eval_at_log(D + S.knot_u, D + S.ctrl, S.degree, span, lo, hi, k.lq);
}

// Lower RITA energy row (lower_bound - 1) with the bucketed search.
template <typename R>
MIDSX_HD int rita_row_bk(const DevTables& t, const DevRita& T, R E) {
    const R* en = tab<R>(t) + T.energy;
    const int* st = buckets<R>(t, T.bk_d, T.bk_f);
    int b = bucket_of(E, bspec<R>(t, 0));
    return lower_index(en, st[b], st[b + 1], E) - 1;
}

// ContinuousInversion::sample (probability_dist.cpp:73-88).  Returns false if E has no
// bracketing energy pair (outside the built tables).
template <typename R>
MIDSX_HD bool rita_sample(const DevTables& t, const DevRita& T, R E, R y, R& mu) {
    const R* D = tab<R>(t);
    int lower = rita_row_bk<R>(t, T, E);
    int upper = lower + 1;
    if (lower < 0 || upper >= T.n_energy) return false;
    const R* X = D + T.x;
    const R* Y = D + T.y;
    const R* A = D + T.a;
    const R* B = D + T.b;
    const int* rs = t.rows + T.row_start;
    R xl = rita_x_from_y(X, Y, A, B, rs[lower], rs[lower + 1], y);
    R xu = rita_x_from_y(X, Y, A, B, rs[upper], rs[upper + 1], y);
    const R* LE = D + T.log_energy;
    R ll = log_(xl + R(1));
    mu = exp_(ll + (log_(xu + R(1)) - ll) * (log_(E) - LE[lower]) / (LE[upper] - LE[lower])) - R(1);
    return true;
}

// -------------------------------------------------------------------- tally specs ---
struct DevTally {
    int kind, nu, nv, n_energy;  // n_energy: incident-energy spectrum bins of a DISC / RECT
    double a[3], b[3], c[3];
    double radius;
    double norm[3];      // plane normal used for the entrance cosine
    double e1e1, e2e2;   // rectangle basis dot products
    double e_min, e_width;  // spectrum bins [e_min + k e_width, e_min + (k+1) e_width)
    unsigned long long* acc;
    // FP32 copies for the mixed form
    float fa[3], fb[3], fc[3], fnorm[3];
    float fradius, fe1e1, fe2e2, fe_min, fe_width;
};


// The working-precision value of a field stored in FP64 with an FP32 copy.
template <typename R>
MIDSX_HD R pickr(double d, float f) {
    if constexpr (sizeof(R) == 8)
        return d;
    else
        return f;
}

// Spectrum bin of incident energy E, -1 outside the tally's n_energy bins: floor((E - e_min) /
// e_width) in the working precision (IEEE division, as the oracle computes it in FP64).
template <typename R>
__device__ __forceinline__ int energy_bin(const DevTally& T, R E) {
    const R k = (E - pickr<R>(T.e_min, T.fe_min)) / pickr<R>(T.e_width, T.fe_width);
    if (!(k >= R(0)) || k >= R(T.n_energy)) return -1;
    return int(k);
}

// fixed-point scales of the mixed path (per eV, per eV^2, per unit cosine)
constexpr double kFxEnergy = 4096.0;
constexpr double kFxEnergy2 = 1.0 / 16.0;
constexpr double kFxCosine = 1073741824.0;

// Scatter class: 0 primary, 1 single coherent, 2 single incoherent, 3 multiple.
MIDSX_HD int scatter_class(int n_coh, int n_incoh) {
    int total = n_coh + n_incoh;
    if (total > 1) return 3;
    if (n_coh == 1) return 1;
    if (n_incoh == 1) return 2;
    return 0;
}

}  // namespace midsx
