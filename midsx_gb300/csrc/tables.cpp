// tables.cpp - host construction of the FP64 interaction tables of the transport path.
//
// Restates the reference's table set-up (run once per simulation, not on the hot path):
//   MaterialProperties (number densities)   src/MIDSX/Core/material_properties.cpp:10-77
//   MaterialData (weighted sums, merged
//     grids, interpolator choice, total)    src/MIDSX/Core/material_data.cpp:9-170
//   InteractionData majorant                src/MIDSX/Core/interaction_data.cpp:42-73
//   ContinuousInversion (RITA build)        src/MIDSX/Core/probability_dist.cpp:121-287
//   Interpolator::Spline / LogLogSpline     src/MIDSX/Core/interpolators.cpp:3-31
// The reference's LogLogSpline is Eigen's SplineFitting::Interpolate (knot averaging +
// collocation, The NURBS Book section 9.2.1); it is rewritten here from that published
// method with a banded elimination in place of Eigen's dense QR solve.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/midsx_gpu.h"
#include "lookup.h"
#include "tables_internal.h"

namespace midsx {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string& s) { g_last_error = s; }
const char* last_error() { return g_last_error.c_str(); }

// ------------------------------------------------------------------ data files ------
namespace {

struct XY {
    std::vector<double> x, y;
};

struct ElementData {
    int Z = 0;
    double awr = 0;
    XY coh, incoh, photo, ffactor, sfunc;
};

struct MaterialDef {
    int id = 0;
    std::string name;
    double density = 0;
    std::vector<std::pair<int, double>> comp;  // (Z, weight fraction), ascending Z
};

struct DataLibrary {
    std::map<int, ElementData> elements;
    std::map<int, double> atomic_weight;
    std::vector<MaterialDef> materials;
};

std::mutex g_lib_mutex;
std::map<std::string, std::shared_ptr<DataLibrary>> g_libs;

template <typename T>
bool read_pod(std::ifstream& f, T& v) {
    return bool(f.read(reinterpret_cast<char*>(&v), sizeof(T)));
}

void read_xy(std::ifstream& f, XY& t) {
    uint32_t n = 0;
    if (!read_pod(f, n)) throw std::runtime_error("truncated epdl_photon.bin");
    t.x.resize(n);
    t.y.resize(n);
    f.read(reinterpret_cast<char*>(t.x.data()), sizeof(double) * n);
    f.read(reinterpret_cast<char*>(t.y.data()), sizeof(double) * n);
    if (!f) throw std::runtime_error("truncated epdl_photon.bin");
}

std::vector<std::string> split(const std::string& s, char sep) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == sep) {
            out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(c);
        }
    }
    out.push_back(cur);
    return out;
}

std::shared_ptr<DataLibrary> load_library(const std::string& dir) {
    std::lock_guard<std::mutex> lock(g_lib_mutex);
    auto it = g_libs.find(dir);
    if (it != g_libs.end()) return it->second;
    auto lib = std::make_shared<DataLibrary>();
    {
        std::ifstream f(dir + "/epdl_photon.bin", std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + dir + "/epdl_photon.bin");
        char magic[8];
        f.read(magic, 8);
        uint32_t version = 0, n = 0;
        read_pod(f, version);
        read_pod(f, n);
        if (std::memcmp(magic, "MIDSXEPD", 8) != 0 || version != 1)
            throw std::runtime_error("bad epdl_photon.bin header");
        for (uint32_t i = 0; i < n; ++i) {
            ElementData e;
            uint32_t z = 0;
            read_pod(f, z);
            read_pod(f, e.awr);
            e.Z = int(z);
            read_xy(f, e.coh);
            read_xy(f, e.incoh);
            read_xy(f, e.photo);
            read_xy(f, e.ffactor);
            read_xy(f, e.sfunc);
            lib->elements[e.Z] = std::move(e);
        }
    }
    {
        std::ifstream f(dir + "/elements.txt");
        if (!f) throw std::runtime_error("cannot open " + dir + "/elements.txt");
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            auto p = split(line, '|');
            if (p.size() != 3) throw std::runtime_error("bad elements.txt line: " + line);
            lib->atomic_weight[std::stoi(p[0])] = std::stod(p[2]);
        }
    }
    {
        std::ifstream f(dir + "/materials.txt");
        if (!f) throw std::runtime_error("cannot open " + dir + "/materials.txt");
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            auto p = split(line, '|');
            if (p.size() != 4) throw std::runtime_error("bad materials.txt line: " + line);
            MaterialDef m;
            m.id = std::stoi(p[0]);
            m.name = p[1];
            m.density = std::stod(p[2]);
            for (auto& c : split(p[3], ',')) {
                auto zw = split(c, ':');
                m.comp.emplace_back(std::stoi(zw[0]), std::stod(zw[1]));
            }
            std::sort(m.comp.begin(), m.comp.end());
            lib->materials.push_back(std::move(m));
        }
    }
    g_libs[dir] = lib;
    return lib;
}

const MaterialDef* find_material(const DataLibrary& lib, int id) {
    for (auto& m : lib.materials)
        if (m.id == id) return &m;
    return nullptr;
}

// ------------------------------------------------------------- interpolators ------

// Interpolator::LogLogLinear with the reference's own search on log10 values.
struct LogLin {
    std::vector<double> x, lx, ly;
    LogLin() = default;
    LogLin(const std::vector<double>& xs, const std::vector<double>& ys) : x(xs) {
        lx.resize(xs.size());
        ly.resize(ys.size());
        for (size_t i = 0; i < xs.size(); ++i) {
            lx[i] = std::log10(xs[i]);
            ly[i] = std::log10(ys[i]);
        }
    }
    double operator()(double q) const {
        double lq = std::log10(q);
        size_t n = lx.size();
        if (lq <= lx[0]) return std::pow(10.0, ly[0]);
        if (lq >= lx[n - 1]) return std::pow(10.0, ly[n - 1]);
        size_t idx = std::upper_bound(lx.begin(), lx.end(), lq) - lx.begin();
        double slope = (ly[idx] - ly[idx - 1]) / (lx[idx] - lx[idx - 1]);
        return std::pow(10.0, ly[idx - 1] + slope * (lq - lx[idx - 1]));
    }
};

// Interpolator::LogLogSpline: global B-spline interpolation of (log10 x, log10 y) with
// parameters u = (log10 x - min) / (max - min), degree min(n - 1, 3), averaged knots.
struct LogSpline {
    int degree = 0;
    double lx_min = 0, lx_max = 0;
    std::vector<double> knots, ctrl;

    LogSpline() = default;
    LogSpline(const std::vector<double>& xs, const std::vector<double>& ys) {
        const int n = int(xs.size());
        if (n < 2) throw std::runtime_error("spline needs at least two points");
        std::vector<double> lx(n), ly(n), u(n);
        for (int i = 0; i < n; ++i) {
            lx[i] = std::log10(xs[i]);
            ly[i] = std::log10(ys[i]);
        }
        lx_min = *std::min_element(lx.begin(), lx.end());
        lx_max = *std::max_element(lx.begin(), lx.end());
        for (int i = 0; i < n; ++i) u[i] = (lx[i] - lx_min) / (lx_max - lx_min);
        degree = std::min(n - 1, 3);
        const int p = degree;
        // knot averaging (The NURBS Book eq. 9.8)
        knots.assign(n + p + 1, 0.0);
        for (int j = 1; j < n - p; ++j) {
            double s = 0;
            for (int k = 0; k < p; ++k) s += u[j + k];
            knots[j + p] = s / p;
        }
        for (int k = 0; k <= p; ++k) {
            knots[k] = 0.0;
            knots[n + k] = 1.0;
        }
        // collocation matrix in band storage: row i, columns i-p .. i+p
        const int w = 2 * p + 1;
        std::vector<double> band(size_t(n) * w, 0.0);
        auto at = [&](int i, int j) -> double& { return band[size_t(i) * w + (j - i + p)]; };
        at(0, 0) = 1.0;
        at(n - 1, n - 1) = 1.0;
        for (int i = 1; i < n - 1; ++i) {
            int span = find_span(u[i]);
            double N[4];
            basis(span, u[i], N);
            for (int k = 0; k <= p; ++k) {
                int j = span - p + k;
                if (j < i - p || j > i + p) throw std::runtime_error("spline band overflow");
                at(i, j) = N[k];
            }
        }
        // Gaussian elimination without pivoting (collocation matrices of B-splines are
        // totally positive, de Boor 1976), then back substitution.
        std::vector<double> rhs = ly;
        for (int k = 0; k < n; ++k) {
            double piv = at(k, k);
            if (piv == 0.0) throw std::runtime_error("singular spline system");
            for (int i = k + 1; i <= std::min(n - 1, k + p); ++i) {
                double f = at(i, k) / piv;
                if (f == 0.0) continue;
                for (int j = k; j <= std::min(n - 1, k + p); ++j) at(i, j) -= f * at(k, j);
                rhs[i] -= f * rhs[k];
            }
        }
        ctrl.assign(n, 0.0);
        for (int i = n - 1; i >= 0; --i) {
            double s = rhs[i];
            for (int j = i + 1; j <= std::min(n - 1, i + p); ++j) s -= at(i, j) * ctrl[j];
            ctrl[i] = s / at(i, i);
        }
    }

    int find_span(double u) const {
        const int nk = int(knots.size());
        if (u <= knots[0]) return degree;
        auto pos = std::upper_bound(knots.begin() + (degree - 1), knots.begin() + (nk - degree - 1), u);
        return int(pos - knots.begin()) - 1;
    }

    void basis(int span, double u, double* N) const {
        double left[4], right[4];
        N[0] = 1.0;
        for (int j = 1; j <= degree; ++j) {
            left[j] = u - knots[span + 1 - j];
            right[j] = knots[span + j] - u;
            double saved = 0.0;
            for (int r = 0; r < j; ++r) {
                double temp = N[r] / (right[r + 1] + left[j - r]);
                N[r] = saved + right[r + 1] * temp;
                saved = left[j - r] * temp;
            }
            N[j] = saved;
        }
    }

    double operator()(double e) const {
        double u = (std::log10(e) - lx_min) / (lx_max - lx_min);
        int span = find_span(u);
        double N[4];
        basis(span, u, N);
        double v = 0;
        for (int i = 0; i <= degree; ++i) v += ctrl[span - degree + i] * N[i];
        return std::pow(10.0, v);
    }
};

std::vector<double> merge_grids(const std::vector<const std::vector<double>*>& grids) {
    std::vector<double> m;
    for (auto* g : grids) m.insert(m.end(), g->begin(), g->end());
    std::sort(m.begin(), m.end());
    m.erase(std::unique(m.begin(), m.end()), m.end());
    return m;
}

// ---------------------------------------------------------------- RITA build ------
struct RitaRow {
    std::vector<double> x, y, a, b;
};

constexpr double kElectronRestMass = 0.51099895000E6;  // eV, include/MIDSX/Core/constants.h:16
constexpr double kPlanck = 4.135667662e-15;            // eV s
constexpr double kSpeedOfLight = 299792458E2;          // cm/s
constexpr double kAvogadro = 6.022140857e23;           // 1/mol
inline double alpha_inv_angstrom() {
    return kElectronRestMass / (std::sqrt(2.0) * kPlanck * kSpeedOfLight * 1E8);
}

struct RitaBuilder {
    const LogLin& ff;
    double E = 0;
    double norm = 1;  // integral of the PDF over [-1, 1] at E (normalizePDF)

    double pdf(double mu) const {
        double k = E / kElectronRestMass;
        double x = alpha_inv_angstrom() * k * std::sqrt(1 - mu);
        return (1 + mu * mu) * std::pow(ff(x), 2);
    }
    double npdf(double mu) const { return pdf(mu) / norm; }

    void normalize() {
        const int N = 1001;
        const double lo = -1, hi = 1;
        double h = (hi - lo) / (N - 1), sum = 0;
        for (int k = 0; k < N; ++k) {
            double f = pdf(lo + k * h);
            sum += (k == 0 || k == N - 1) ? f : (k % 2 == 0 ? 2 * f : 4 * f);
        }
        norm = h / 3 * sum;
    }

    // generateCDFPerEnergy: cumulative Simpson integral with 51 points per interval.
    void cdf(const std::vector<double>& xg, std::vector<double>& y) const {
        const int NP = 51;
        y.assign(xg.size(), 0.0);
        for (size_t j = 0; j + 1 < xg.size(); ++j) {
            double x0 = xg[j], x1 = xg[j + 1];
            double h = (x1 - x0) / (NP - 1), sum = 0;
            for (int k = 0; k < NP; ++k) {
                double f = npdf(x0 + k * h);
                sum += (k == 0 || k == NP - 1) ? f : (k % 2 == 0 ? 2 * f : 4 * f);
            }
            y[j + 1] = y[j] + h / 3 * sum;
        }
    }

    void params(const std::vector<double>& xg, const std::vector<double>& y, std::vector<double>& a,
                std::vector<double>& b) const {
        size_t n = xg.size();
        a.assign(n, 0.0);
        b.assign(n, 0.0);
        for (size_t i = 0; i + 1 < n; ++i) {
            double s = (y[i + 1] - y[i]) / (xg[i + 1] - xg[i]);
            double bi = 1 - std::pow(s, 2) * (1 / (npdf(xg[i]) * npdf(xg[i + 1])));
            double ai = s * (1 / npdf(xg[i])) - bi - 1;
            a[i] = ai;
            b[i] = bi;
        }
    }

    static double eta(double x, double xi, double xi1, double ai, double bi) {
        double tau = (x - xi) / (xi1 - xi);
        if (tau == 0) return 0;
        double c = 1 + ai + bi - ai * tau;
        return c / (2 * bi * tau) * (1 - std::sqrt(1 - 4 * bi * tau * tau / std::pow(c, 2)));
    }

    static double pnum(double x, double xi, double xi1, double yi, double yi1, double ai, double bi) {
        double e = eta(x, xi, xi1, ai, bi);
        return std::pow(1 + ai * e + bi * e * e, 2) / ((1 + ai + bi) * (1 - bi * e * e)) * (yi1 - yi) /
               (xi1 - xi);
    }

    // getInterpErrorOverInterval (PENELOPE eq. 1.57 as coded: 51 sub-steps of width
    // (x_{i+1}-x_i)/51 and a trapezoid end correction; |.| is the floating-point abs).
    double interval_error(double xi, double xi1, double yi, double yi1, double ai, double bi) const {
        const int N = 51;
        double dx = (xi1 - xi) / N, sum = 0;
        for (int i = 1; i < N; ++i) {
            double xk = xi + i * dx;
            sum += std::fabs(npdf(xk) - pnum(xk, xi, xi1, yi, yi1, ai, bi));
        }
        return dx * (sum + (std::fabs(npdf(xi1) - pnum(xi1, xi, xi1, yi, yi1, ai, bi)) +
                            std::fabs(npdf(xi) - pnum(xi, xi, xi1, yi, yi1, ai, bi))) /
                               2);
    }

    RitaRow build(double energy, double err_thresh) {
        E = energy;
        normalize();
        // Eigen::VectorXd::LinSpaced(10, -1, 1)
        std::vector<double> xg(10);
        const double step = 2.0 / 9.0;
        for (int i = 0; i < 10; ++i) xg[i] = (i == 9) ? 1.0 : -1.0 + i * step;
        std::vector<double> y, a, b;
        bool met = false;
        int guard = 0;
        while (!met) {
            if (++guard > 64) throw std::runtime_error("RITA grid refinement did not converge");
            cdf(xg, y);
            params(xg, y, a, b);
            std::vector<double> nx;
            met = true;
            for (size_t i = 0; i + 1 < xg.size(); ++i) {
                nx.push_back(xg[i]);
                double eps = interval_error(xg[i], xg[i + 1], y[i], y[i + 1], a[i], b[i]);
                if (eps > err_thresh) {
                    nx.push_back((xg[i] + xg[i + 1]) / 2);
                    met = false;
                }
            }
            nx.push_back(xg.back());
            xg.swap(nx);
        }
        RitaRow r;
        r.x = xg;
        cdf(xg, r.y);
        params(xg, r.y, r.a, r.b);
        return r;
    }
};

// ----------------------------------------------------------- material tables ------
struct MaterialTables {
    int id = 0;
    double density = 0;
    std::vector<double> incoh_x, incoh_y, coh_x, coh_y, photo_x, photo_y, total_x, total_y;
    std::vector<double> sf_x, sf_y, ff_x, ff_y;
    LogSpline incoh, coh;
    LogLin photo, total, sf, ff;
    std::vector<double> rita_e;
    std::vector<RitaRow> rita;
};

enum Table { kCoh, kIncoh, kPhoto, kFF, kSF };

const XY& element_table(const ElementData& e, Table t) {
    switch (t) {
        case kCoh: return e.coh;
        case kIncoh: return e.incoh;
        case kPhoto: return e.photo;
        case kFF: return e.ffactor;
        default: return e.sfunc;
    }
}

// MaterialData::calculateWeightedAverageOfColumns (material_data.cpp:87-114).
void weighted_average(const DataLibrary& lib, const MaterialDef& m, Table t, bool macroscopic,
                      std::vector<double>& gx, std::vector<double>& gy) {
    std::vector<const std::vector<double>*> grids;
    for (auto& zw : m.comp) grids.push_back(&element_table(lib.elements.at(zw.first), t).x);
    gx = merge_grids(grids);
    gy.assign(gx.size(), 0.0);
    for (auto& zw : m.comp) {
        const XY& d = element_table(lib.elements.at(zw.first), t);
        double weight = zw.second;
        if (macroscopic) {
            // MaterialProperties::setNumberDensity (material_properties.cpp:66-73)
            weight = kAvogadro * m.density * zw.second / lib.atomic_weight.at(zw.first);
        }
        if (t == kCoh || t == kIncoh) {
            LogSpline s(d.x, d.y);
            for (size_t i = 0; i < gx.size(); ++i) gy[i] += weight * s(gx[i]);
        } else {
            LogLin l(d.x, d.y);
            for (size_t i = 0; i < gx.size(); ++i) gy[i] += weight * l(gx[i]);
        }
    }
}

MaterialTables build_material(const DataLibrary& lib, const MaterialDef& m, double e_max) {
    MaterialTables mt;
    mt.id = m.id;
    mt.density = m.density;
    for (auto& zw : m.comp) {
        if (!lib.elements.count(zw.first) || !lib.atomic_weight.count(zw.first))
            throw std::runtime_error("element " + std::to_string(zw.first) + " missing from data");
    }
    weighted_average(lib, m, kIncoh, true, mt.incoh_x, mt.incoh_y);
    for (auto& v : mt.incoh_y) v *= 1E-24;
    mt.incoh = LogSpline(mt.incoh_x, mt.incoh_y);
    weighted_average(lib, m, kCoh, true, mt.coh_x, mt.coh_y);
    for (auto& v : mt.coh_y) v *= 1E-24;
    mt.coh = LogSpline(mt.coh_x, mt.coh_y);
    weighted_average(lib, m, kPhoto, true, mt.photo_x, mt.photo_y);
    for (auto& v : mt.photo_y) v *= 1E-24;
    mt.photo = LogLin(mt.photo_x, mt.photo_y);
    // total on the merged grid (material_data.cpp:24-27,75-85,125-134)
    mt.total_x = merge_grids({&mt.incoh_x, &mt.coh_x, &mt.photo_x});
    mt.total_y.resize(mt.total_x.size());
    for (size_t i = 0; i < mt.total_x.size(); ++i) {
        double e = mt.total_x[i];
        mt.total_y[i] = mt.incoh(e) + mt.coh(e) + mt.photo(e);
    }
    mt.total = LogLin(mt.total_x, mt.total_y);
    weighted_average(lib, m, kSF, false, mt.sf_x, mt.sf_y);
    mt.sf = LogLin(mt.sf_x, mt.sf_y);
    weighted_average(lib, m, kFF, false, mt.ff_x, mt.ff_y);
    mt.ff = LogLin(mt.ff_x, mt.ff_y);
    // RITA tables on the incoherent energy grid (material_data.cpp:62-73), energies up to
    // the first node >= e_max so that every energy <= e_max has a bracketing pair.
    size_t n_e = 0;
    while (n_e < mt.incoh_x.size() && (n_e == 0 || mt.incoh_x[n_e - 1] < e_max)) ++n_e;
    if (n_e < 2 || mt.incoh_x[n_e - 1] < e_max)
        throw std::runtime_error("e_max beyond the incoherent energy grid");
    mt.rita_e.assign(mt.incoh_x.begin(), mt.incoh_x.begin() + n_e);
    mt.rita.resize(n_e);
    std::string err;
#pragma omp parallel for schedule(dynamic, 1)
    for (long i = 0; i < long(n_e); ++i) {
        try {
            RitaBuilder rb{mt.ff};
            mt.rita[i] = rb.build(mt.rita_e[i], 1E-4);
        } catch (const std::exception& ex) {
#pragma omp critical
            err = ex.what();
        }
    }
    if (!err.empty()) throw std::runtime_error(err);
    return mt;
}

// ----------------------------------------------------------------- flattening ------
struct Flat {
    std::vector<double> d;
    std::vector<int64_t> id;
    int64_t push(const std::vector<double>& v) {
        int64_t off = int64_t(d.size());
        d.insert(d.end(), v.begin(), v.end());
        return off;
    }
    midsx_lin_table lin(const std::vector<double>& x, const LogLin& l) {
        midsx_lin_table t;
        t.x = push(x);
        t.lx = push(l.lx);
        t.ly = push(l.ly);
        t.n = int32_t(x.size());
        t.reserved = 0;
        return t;
    }
    midsx_spline_table spline(const LogSpline& s) {
        midsx_spline_table t;
        std::vector<double> ke(s.knots.size());
        for (size_t i = 0; i < ke.size(); ++i)
            ke[i] = std::pow(10.0, s.lx_min + s.knots[i] * (s.lx_max - s.lx_min));
        t.knot_e = push(ke);
        t.knot_u = push(s.knots);
        t.ctrl = push(s.ctrl);
        t.n_ctrl = int32_t(s.ctrl.size());
        t.degree = s.degree;
        t.lx_min = s.lx_min;
        t.lx_max = s.lx_max;
        return t;
    }
};

}  // namespace

midsx_table_blob* build_blob(const std::string& dir, const int32_t* ids, int n, double e_max) {
    auto lib = load_library(dir);
    if (n < 1 || n > MIDSX_MAX_MATERIALS) throw std::invalid_argument("material count out of range");
    std::vector<MaterialTables> mats;
    for (int i = 0; i < n; ++i) {
        const MaterialDef* def = find_material(*lib, ids[i]);
        if (!def) throw std::out_of_range("unknown material id " + std::to_string(ids[i]));
        for (int j = 0; j < i; ++j)
            if (ids[j] == ids[i]) throw std::invalid_argument("duplicate material id");
        mats.push_back(build_material(*lib, *def, e_max));
    }
    // majorant (interaction_data.cpp:42-73)
    std::vector<const std::vector<double>*> grids;
    for (auto& m : mats) grids.push_back(&m.total_x);
    std::vector<double> mx = merge_grids(grids), my(mx.size());
    for (size_t i = 0; i < mx.size(); ++i) {
        double best = -1;
        for (auto& m : mats) best = std::max(best, m.total(mx[i]));
        my[i] = best;
    }
    LogLin maj(mx, my);

    Flat fl;
    auto* blob = new midsx_table_blob();
    std::memset(blob, 0, sizeof(*blob));
    blob->version = 1;
    blob->n_materials = n;
    blob->e_max = e_max;
    blob->majorant = fl.lin(mx, maj);
    for (int i = 0; i < n; ++i) {
        MaterialTables& m = mats[i];
        midsx_material_table& t = blob->mat[i];
        t.id = m.id;
        t.density = m.density;
        t.total = fl.lin(m.total_x, m.total);
        t.photo = fl.lin(m.photo_x, m.photo);
        t.sfunc = fl.lin(m.sf_x, m.sf);
        t.ffactor = fl.lin(m.ff_x, m.ff);
        t.coh = fl.spline(m.coh);
        t.incoh = fl.spline(m.incoh);
        midsx_rita_table& r = t.rita;
        r.n_energy = int32_t(m.rita_e.size());
        r.energy = fl.push(m.rita_e);
        std::vector<double> le(m.rita_e.size());
        for (size_t k = 0; k < le.size(); ++k) le[k] = std::log(m.rita_e[k]);
        r.log_energy = fl.push(le);
        std::vector<double> X, Y, A, B;
        r.row_start = int64_t(fl.id.size());
        int64_t rows = 0;
        for (auto& row : m.rita) {
            fl.id.push_back(rows);
            X.insert(X.end(), row.x.begin(), row.x.end());
            Y.insert(Y.end(), row.y.begin(), row.y.end());
            A.insert(A.end(), row.a.begin(), row.a.end());
            B.insert(B.end(), row.b.begin(), row.b.end());
            rows += int64_t(row.x.size());
        }
        fl.id.push_back(rows);
        r.n_rows = int32_t(rows);
        r.x = fl.push(X);
        r.y = fl.push(Y);
        r.a = fl.push(A);
        r.b = fl.push(B);
    }
    blob->n_data = int64_t(fl.d.size());
    blob->data = new double[fl.d.size()];
    std::memcpy(blob->data, fl.d.data(), sizeof(double) * fl.d.size());
    blob->n_idata = int64_t(fl.id.size());
    blob->idata = new int64_t[fl.id.size()];
    std::memcpy(blob->idata, fl.id.data(), sizeof(int64_t) * fl.id.size());
    return blob;
}

std::shared_ptr<DataLibrary> load_library_public(const std::string& dir) { return load_library(dir); }
const MaterialDef* find_material_public(const DataLibrary& lib, int id) { return find_material(lib, id); }

int catalog_id(const std::string& dir, const std::string& name) {
    auto lib = load_library(dir);
    for (auto& m : lib->materials)
        if (m.name == name) return m.id;
    return -1;
}

std::string catalog_name(const std::string& dir, int id) {
    auto lib = load_library(dir);
    const MaterialDef* m = find_material(*lib, id);
    return m ? m->name : std::string();
}

}  // namespace midsx

// ------------------------------------------------------------------------ C ABI ---
using midsx::set_last_error;

#define MIDSX_GUARD(body)                                      \
    try {                                                      \
        body                                                   \
    } catch (const std::invalid_argument& e) {                 \
        set_last_error(e.what());                              \
        return MIDSX_INVALID_ARG;                              \
    } catch (const std::out_of_range& e) {                     \
        set_last_error(e.what());                              \
        return MIDSX_NOT_FOUND;                                \
    } catch (const std::bad_alloc& e) {                        \
        set_last_error("host allocation failed");              \
        return MIDSX_OOM;                                      \
    } catch (const std::exception& e) {                        \
        set_last_error(e.what());                              \
        return MIDSX_IO_ERROR;                                 \
    }

extern "C" midsx_status midsx_tables_build(const char* data_dir, const int32_t* material_ids,
                                           int32_t n, double e_max, midsx_table_blob** out) {
    if (!data_dir || !material_ids || !out || n < 1 || n > MIDSX_MAX_MATERIALS || !(e_max > 0)) {
        set_last_error("midsx_tables_build: invalid argument");
        return MIDSX_INVALID_ARG;
    }
    MIDSX_GUARD({
        *out = midsx::build_blob(data_dir, material_ids, n, e_max);
        return MIDSX_OK;
    })
}

extern "C" void midsx_tables_free(midsx_table_blob* blob) {
    if (!blob) return;
    delete[] blob->data;
    delete[] blob->idata;
    delete blob;
}

extern "C" midsx_status midsx_catalog_id(const char* data_dir, const char* name, int32_t* id_out) {
    if (!data_dir || !name || !id_out) return MIDSX_INVALID_ARG;
    MIDSX_GUARD({
        int id = midsx::catalog_id(data_dir, name);
        if (id < 0) {
            set_last_error(std::string("unknown material name: ") + name);
            return MIDSX_NOT_FOUND;
        }
        *id_out = id;
        return MIDSX_OK;
    })
}

extern "C" midsx_status midsx_catalog_name(const char* data_dir, int32_t id, char* name_out,
                                           int32_t cap) {
    if (!data_dir || !name_out || cap < 1) return MIDSX_INVALID_ARG;
    MIDSX_GUARD({
        std::string s = midsx::catalog_name(data_dir, id);
        if (s.empty()) {
            set_last_error("unknown material id " + std::to_string(id));
            return MIDSX_NOT_FOUND;
        }
        std::snprintf(name_out, size_t(cap), "%s", s.c_str());
        return MIDSX_OK;
    })
}

extern "C" midsx_status midsx_catalog_material(const char* data_dir, int32_t id, double* density, int32_t* n,
                                               int32_t* z, double* weight, double* atomic_weight, int32_t cap) {
    if (!data_dir || !density || !n) return MIDSX_INVALID_ARG;
    MIDSX_GUARD({
        auto lib = midsx::load_library_public(data_dir);
        const auto* m = midsx::find_material_public(*lib, id);
        if (!m) {
            set_last_error("unknown material id " + std::to_string(id));
            return MIDSX_NOT_FOUND;
        }
        *density = m->density;
        *n = int32_t(m->comp.size());
        for (int32_t i = 0; i < *n && i < cap; ++i) {
            if (z) z[i] = m->comp[size_t(i)].first;
            if (weight) weight[i] = m->comp[size_t(i)].second;
            if (atomic_weight) atomic_weight[i] = lib->atomic_weight.at(m->comp[size_t(i)].first);
        }
        return MIDSX_OK;
    })
}

extern "C" midsx_status midsx_tables_rita(const midsx_table_blob* blob, int32_t material, double energy, double y,
                                          double* mu) {
    if (!blob || !mu || material < 0 || material >= blob->n_materials) return MIDSX_INVALID_ARG;
    const midsx_rita_table& r = blob->mat[material].rita;
    const double* D = blob->data;
    const int64_t* rows = blob->idata + r.row_start;
    int lower = midsx::lower_index(D + r.energy, 0, r.n_energy, energy) - 1;
    if (lower < 0 || lower + 1 >= r.n_energy) return MIDSX_TABLE_RANGE;
    const double *X = D + r.x, *Y = D + r.y, *A = D + r.a, *B = D + r.b, *LE = D + r.log_energy;
    double xl = midsx::rita_x_from_y(X, Y, A, B, int(rows[lower]), int(rows[lower + 1]), y);
    double xu = midsx::rita_x_from_y(X, Y, A, B, int(rows[lower + 1]), int(rows[lower + 2]), y);
    double ll = std::log(xl + 1);
    *mu = std::exp(ll + (std::log(xu + 1) - ll) * (std::log(energy) - LE[lower]) / (LE[lower + 1] - LE[lower])) - 1;
    return MIDSX_OK;
}

extern "C" midsx_status midsx_tables_eval(const midsx_table_blob* blob, int32_t material,
                                          int32_t which, const double* x, double* y, int64_t n) {
    if (!blob || !x || !y || n < 0 || which < 0 || which > 6) return MIDSX_INVALID_ARG;
    if (which != 6 && (material < 0 || material >= blob->n_materials)) return MIDSX_INVALID_ARG;
    const double* D = blob->data;
    const midsx_material_table* m = (which == 6) ? nullptr : &blob->mat[material];
    for (int64_t i = 0; i < n; ++i) {
        double q = x[i], v = 0;
        const midsx_lin_table* lt = nullptr;
        const midsx_spline_table* st = nullptr;
        switch (which) {
            case 0: lt = &m->total; break;
            case 1: lt = &m->photo; break;
            case 2: st = &m->coh; break;
            case 3: st = &m->incoh; break;
            case 4: lt = &m->sfunc; break;
            case 5: lt = &m->ffactor; break;
            default: lt = &blob->majorant; break;
        }
        if (lt) {
            v = midsx::lin_eval(D + lt->x, D + lt->lx, D + lt->ly, lt->n, q);
        } else {
            int span = midsx::spline_span(D + st->knot_e, st->n_ctrl, st->degree, q);
            v = midsx::spline_eval_at(D + st->knot_u, D + st->ctrl, st->degree, span, st->lx_min,
                                      st->lx_max, q);
        }
        y[i] = v;
    }
    return MIDSX_OK;
}

namespace {

// Mean fraction of the photon energy given to the electron in one incoherent scatter at
// k = E / mec2, under the transport's sampling density KN(mu) * S(alpha k sqrt(1 - mu))
// (photon_interactions.cpp:62-141).  Substituting t = sqrt(1 - mu) makes the S(x) argument
// linear in t; composite 8-point Gauss-Legendre over 256 panels of t in [0, sqrt 2].
double incoherent_transfer_fraction(const double* D, const midsx_lin_table& sf, double k) {
    static const double gx[8] = {-0.9602898564975363, -0.7966664774136267, -0.5255324099163290,
                                 -0.1834346424956498, 0.1834346424956498,  0.5255324099163290,
                                 0.7966664774136267,  0.9602898564975363};
    static const double gw[8] = {0.1012285362903763, 0.2223810344533745, 0.3137066678687174,
                                 0.3626837833783620, 0.3626837833783620, 0.3137066678687174,
                                 0.2223810344533745, 0.1012285362903763};
    const int panels = 256;
    const double t_hi = std::sqrt(2.0), h = t_hi / panels;
    const double alpha = midsx::alpha_inv_angstrom();
    double num = 0, den = 0;
    for (int p = 0; p < panels; ++p) {
        const double c = (p + 0.5) * h;
        for (int q = 0; q < 8; ++q) {
            const double t = c + 0.5 * h * gx[q];
            const double mu = 1 - t * t;
            const double r = 1 / (1 + k * (1 - mu));  // k'/k
            const double kn = r * r * (r + 1 / r - (1 - mu * mu));
            const double s = midsx::lin_eval(D + sf.x, D + sf.lx, D + sf.ly, sf.n, alpha * k * t);
            const double w = gw[q] * 2 * t * kn * s;  // d(mu) = 2 t dt
            num += w * (1 - r);
            den += w;
        }
    }
    return den > 0 ? num / den : 0.0;
}

}  // namespace

extern "C" midsx_status midsx_tables_mu_en(const midsx_table_blob* blob, int32_t material, const double* x,
                                           double* y, int64_t n) {
    if (!blob || !x || !y || n < 0 || material < 0 || material >= blob->n_materials) return MIDSX_INVALID_ARG;
    const double* D = blob->data;
    const midsx_material_table& m = blob->mat[material];
    if (!(m.density > 0)) return MIDSX_INVALID_ARG;
    for (int64_t i = 0; i < n; ++i) {
        const double E = x[i];
        if (!(E > 0) || E > blob->e_max) return MIDSX_TABLE_RANGE;
        const double photo = midsx::lin_eval(D + m.photo.x, D + m.photo.lx, D + m.photo.ly, m.photo.n, E);
        const midsx_spline_table& st = m.incoh;
        const int span = midsx::spline_span(D + st.knot_e, st.n_ctrl, st.degree, E);
        const double incoh = midsx::spline_eval_at(D + st.knot_u, D + st.ctrl, st.degree, span, st.lx_min,
                                                   st.lx_max, E);
        const double f = incoherent_transfer_fraction(D, m.sfunc, E / midsx::kElectronRestMass);
        y[i] = (photo + incoh * f) / m.density;
    }
    return MIDSX_OK;
}

extern "C" const char* midsx_status_string(midsx_status s) {
    switch (s) {
        case MIDSX_OK: return "ok";
        case MIDSX_INVALID_ARG: return "invalid argument";
        case MIDSX_OOM: return "out of memory";
        case MIDSX_TIMEOUT: return "timeout";
        case MIDSX_STEP_CAP: return "step or trial cap reached";
        case MIDSX_TABLE_RANGE: return "energy outside tables";
        case MIDSX_CUDA_ERROR: return "CUDA error";
        case MIDSX_NOT_FOUND: return "not found";
        case MIDSX_IO_ERROR: return "data file error";
    }
    return "unknown status";
}

extern "C" const char* midsx_last_error(void) { return midsx::last_error(); }
