// lookup.h - table lookups of the transport path, shared by the CUDA kernels and the
// host-side evaluator (midsx_tables_eval).  Each function restates one reference lookup:
//
//   LogLogLinear::operator()     src/MIDSX/Core/interpolators.cpp:37-76
//   LogLogSpline::operator()     src/MIDSX/Core/interpolators.cpp:14-31 (Eigen Spline:
//                                span search and basis functions of Piegl & Tiller,
//                                "The NURBS Book", algorithms A2.1 and A2.2)
//   ContinuousInversion::sample  src/MIDSX/Core/probability_dist.cpp:73-119
//
// Index searches compare raw energies against raw node arrays.  The reference compares
// log10 values; log10 is monotone, so the index is the same except where a query lies
// within rounding of a node, and the raw comparison makes the index a pure function of
// the stored tables (the CPU oracle and the device agree bit for bit).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MIDSX_HD __host__ __device__ __forceinline__
#else
#define MIDSX_HD inline
#include <cmath>
#endif

namespace midsx {

// Division in the flights of the opt-in tracking modes (slab tests, macro-cell walks).
// FP64: the IEEE quotient.  FP32 on the device: the approximate quotient (__fdividef, within
// 2 ulp for divisors up to 2^126), below the FP32 rounding the mixed form already carries:
// +3 to +7 % for macro-cell and background fast tracking.  The reference tracking path keeps
// IEEE division (there the approximate form measured -1.2 %).
MIDSX_HD double adiv(double a, double b) { return a / b; }
MIDSX_HD float adiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdividef(a, b);
#else
    return a / b;
#endif
}

// First index i in [lo, hi) with a[i] > q (std::upper_bound), hi if none.
template <typename R>
MIDSX_HD int upper_index(const R* a, int lo, int hi, R q) {
    int n = hi - lo;
    while (n > 0) {
        int half = n >> 1;
        if (!(q < a[lo + half])) {  // a[mid] <= q
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// First index i in [lo, hi) with a[i] >= q (std::lower_bound), hi if none.
template <typename R>
MIDSX_HD int lower_index(const R* a, int lo, int hi, R q) {
    int n = hi - lo;
    while (n > 0) {
        int half = n >> 1;
        if (a[lo + half] < q) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// ------------------------------------------------------------ bucketed search ------
// A node array x[0..n) is paired with a bucket table over the floating-point bit pattern of
// the query: bucket b holds every query whose top bits (sign, exponent, top K mantissa bits)
// equal base + b, i.e. an exact binade slice [lo(b), lo(b + 1)).  starts[b] is the search
// result for lo(b), computed on the host with the same comparison, so for any query in the
// slice the result lies in [starts[b], starts[b + 1]] and a search over that range gives
// exactly the full-array answer.  Queries below the first slice use slice 0 (starts[0] is the
// range start), queries above the last use the last slice (starts[nb] is the range end).
struct BucketSpec {
    int kbits;       // mantissa bits per binade slice
    long long base;  // key of the first slice
    int nb;          // number of slices
};

MIDSX_HD long long bucket_key(double q, int kbits) {
#if defined(__CUDA_ARCH__)
    unsigned long long bits = (unsigned long long)__double_as_longlong(q);
#else
    unsigned long long bits;
    __builtin_memcpy(&bits, &q, 8);
#endif
    return (long long)(bits >> (52 - kbits));
}

MIDSX_HD long long bucket_key(float q, int kbits) {
#if defined(__CUDA_ARCH__)
    unsigned int bits = __float_as_uint(q);
#else
    unsigned int bits;
    __builtin_memcpy(&bits, &q, 4);
#endif
    return (long long)(bits >> (23 - kbits));
}

template <typename R>
MIDSX_HD int bucket_of(R q, const BucketSpec& s) {
    long long b = bucket_key(q, s.kbits) - s.base;
    if (!(q > R(0))) b = 0;  // zero, negative or NaN queries: first slice
    return b < 0 ? 0 : (b >= s.nb ? s.nb - 1 : int(b));
}

MIDSX_HD double exp10_(double y) { return pow(10.0, y); }
#if defined(__CUDA_ARCH__)
MIDSX_HD float exp10_(float y) { return exp10f(y); }
#else
MIDSX_HD float exp10_(float y) { return powf(10.0f, y); }
#endif
MIDSX_HD double log10_(double y) { return log10(y); }
MIDSX_HD float log10_(float y) { return log10f(y); }
MIDSX_HD double log_(double y) { return log(y); }
MIDSX_HD float log_(float y) { return logf(y); }
MIDSX_HD double exp_(double y) { return exp(y); }
MIDSX_HD float exp_(float y) { return expf(y); }
MIDSX_HD double sqrt_(double y) { return sqrt(y); }
MIDSX_HD float sqrt_(float y) { return sqrtf(y); }

// Interval index of a LogLogLinear table: 0 = below/at first node (clamp), n = at/above the
// last node (clamp), else the std::upper_bound position (1..n-1).
template <typename R>
MIDSX_HD int lin_index(const R* x, int n, R q) {
    if (q <= x[0]) return 0;
    if (q >= x[n - 1]) return n;
    return upper_index(x, 0, n, q);
}

// LogLogLinear value on interval idx, given lq = log10(q).  Tables queried at one energy
// share the logarithm.
template <typename R>
MIDSX_HD R lin_eval_at_log(const R* lx, const R* ly, int n, int idx, R lq) {
    if (idx == 0) return exp10_(ly[0]);
    if (idx >= n) return exp10_(ly[n - 1]);
    R x1 = lx[idx - 1], x2 = lx[idx];
    R y1 = ly[idx - 1], y2 = ly[idx];
    R slope = (y2 - y1) / (x2 - x1);
    return exp10_(y1 + slope * (lq - x1));
}

// LogLogLinear value on interval idx with the interval's slope given (sl[idx] for the interval
// [idx - 1, idx]).  The slopes are computed in FP64 on the host: the FP64 lookups take them as
// they are (the quotient lin_eval_at_log divides out, bit for bit), the FP32 lookups rounded
// once.  Grid nodes closer than FP32 resolves in log10 (merged grids hold node pairs a
// few meV apart) share one float log10 energy, a zero-width interval whose slope recomputed in
// FP32 would be infinite; the stored slope stays finite, and no division is left on the device.
template <typename R>
MIDSX_HD R lin_eval_slope_at_log(const R* lx, const R* ly, const R* sl, int n, int idx, R lq) {
    if (idx == 0) return exp10_(ly[0]);
    if (idx >= n) return exp10_(ly[n - 1]);
    return exp10_(ly[idx - 1] + sl[idx] * (lq - lx[idx - 1]));
}

template <typename R>
MIDSX_HD R lin_eval_at(const R* lx, const R* ly, int n, int idx, R q) {
    if (idx == 0 || idx >= n) return lin_eval_at_log(lx, ly, n, idx, R(0));
    return lin_eval_at_log(lx, ly, n, idx, log10_(q));
}

template <typename R>
MIDSX_HD R lin_eval(const R* x, const R* lx, const R* ly, int n, R q) {
    return lin_eval_at(lx, ly, n, lin_index(x, n, q), q);
}

// Knot span of a B-spline (NURBS Book A2.1 with clamping as in Eigen's Spline::Span):
// degree if q <= first knot, else upper_bound over knots[degree-1, n_knots-degree-1) - 1.
template <typename R>
MIDSX_HD int spline_span(const R* knot_e, int n_ctrl, int degree, R e) {
    int n_knots = n_ctrl + degree + 1;
    if (e <= knot_e[0]) return degree;
    return upper_index(knot_e, degree - 1, n_knots - degree - 1, e) - 1;
}

// B-spline value at parameter u = (log10 e - lx_min) / (lx_max - lx_min), given le = log10 e.
template <typename R>
MIDSX_HD R spline_eval_at_log(const R* knot_u, const R* ctrl, int degree, int span, R lx_min,
                              R lx_max, R le) {
    R u = (le - lx_min) / (lx_max - lx_min);
    R N[4], left[4], right[4];
    N[0] = R(1);
    for (int j = 1; j <= degree; ++j) {
        left[j] = u - knot_u[span + 1 - j];
        right[j] = knot_u[span + j] - u;
        R saved = R(0);
        for (int r = 0; r < j; ++r) {
            R temp = N[r] / (right[r + 1] + left[j - r]);
            N[r] = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        N[j] = saved;
    }
    R v = R(0);
    for (int i = 0; i <= degree; ++i) v += ctrl[span - degree + i] * N[i];
    return exp10_(v);
}

template <typename R>
MIDSX_HD R spline_eval_at(const R* knot_u, const R* ctrl, int degree, int span, R lx_min,
                          R lx_max, R e) {
    return spline_eval_at_log(knot_u, ctrl, degree, span, lx_min, lx_max, log10_(e));
}

// RITA inverse of one energy row: x(y) from the rational interpolation (PENELOPE eq. 1.54
// as coded in getXFromY).  rows [r0, r1) hold x, y, a, b.
template <typename R>
MIDSX_HD R rita_x_from_y(const R* X, const R* Y, const R* A, const R* B, int r0, int r1, R y) {
    int j = lower_index(Y, r0, r1, y) - 1;  // findIndexOfNextSmallestValue
    if (j == r1 - 1) return R(1);           // y above the last CDF value: x_max
    if (j < r0) return R(-1);               // y below the first: x_min
    R yi = Y[j], yi1 = Y[j + 1], xi = X[j], xi1 = X[j + 1];
    R a = A[j], b = B[j];
    R nu = y - yi;
    R delta = yi1 - yi;
    return xi + (R(1) + a + b) * delta * nu / (delta * delta + a * delta * nu + b * nu * nu) * (xi1 - xi);
}

}  // namespace midsx
