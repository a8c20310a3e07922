// oracle.cpp - CPU restatement of MIDSX's photon-history transport loop.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU baseline:
// it may be used by tests/, __graft_entry__.smoke() and bench.py's CPU legs, never by the
// product path.  It restates the reference's own hot path and keeps its data structures
// and loop shape (per-step Photon copies held in TempSurface/TempVolumeTallyData vectors,
// tallies processed after each history, per-thread tally replicas, per-thread lists of
// (voxel, deposit) events, a per-photon critical section), so that it times like the
// reference as well as computing like it.  The reference itself cannot be compiled here
// (Eigen and pybind11 are not available), so it cannot be linked in instead.
//
// Restated reference code (paths inside MIDSX):
//   runSimulation                       src/MIDSX/Core/run_simulation.cpp:6-41
//   PhysicsEngine::transportPhoton*,
//     setInteractionType, getFreePath,
//     isDeltaScatter, processTallies    src/MIDSX/Core/physics_engine.cpp:17-210
//   Photoelectric / Coherent / Incoherent
//     interact (Kahn + S(x))            src/MIDSX/Core/photon_interactions.cpp:43-141
//   rotateDirection (quaternions)       src/MIDSX/Core/particle.cpp:7-45
//   LogLogLinear / LogLogSpline eval    src/MIDSX/Core/interpolators.cpp:14-76
//   ContinuousInversion::sample         src/MIDSX/Core/probability_dist.cpp:73-119
//   DiscreteInversion::sample           src/MIDSX/Core/probability_dist.cpp:18-28
//   PhotonSource and its parts          src/MIDSX/Core/source.cpp:44-155
//   isInComputationalDomain / getVoxel  src/MIDSX/Core/computational_domain.cpp:16-31
//   VoxelGrid index / withinGrid        src/MIDSX/Core/voxel_grid.cpp:43-59,119-128
//   AACuboidVolumeTally                 src/MIDSX/Core/volume_tally.cpp:5-91
//   Disc/RectangularSurfaceTally        src/MIDSX/Core/surface_tally.cpp:5-112
//   Vector/Count quantities             src/MIDSX/Core/volume_quantity.cpp,
//                                       src/MIDSX/Core/surface_quantity.cpp, quantity.cpp
//
// Deliberate differences from the reference, each forced by testing needs:
//   * a seed: RNG_PHILOX gives every history its own Philox4x32-10 stream (the device's
//     stream definition, so trajectories can be compared history by history);
//     RNG_MT19937 gives every thread a std::mt19937 seeded from (seed, thread), the
//     reference's generator;
//   * uniforms in the Philox mode are in (0, 1]; the reference's are in [0, 1);
//   * a voxel index equal to the grid size (a position exactly on the far face, where
//     the reference's vector::at throws) is clamped and counted;
//   * bounded loops: per-history step cap (by default far above any real history: 16
//     crossings of the domain at the largest majorant from 1 keV up) and Compton trial cap,
//     counted;
//   * table indices are found by comparing raw energies with the node arrays (the
//     reference compares their log10; the index agrees except at rounding ties).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include <omp.h>

#include "../include/midsx_gpu.h"

namespace ref {

const double PI = 3.14159265358979323846;
const double EPSILON = 1e-9;
const double INF = std::numeric_limits<double>::infinity();
const double ELECTRON_REST_MASS = 0.51099895000E6;
const double PLANCK_CONSTANT = 4.135667662e-15;
const double SPEED_OF_LIGHT = 299792458E2;
const double ALPHA = ELECTRON_REST_MASS / (std::sqrt(2.0) * PLANCK_CONSTANT * SPEED_OF_LIGHT * 1E8);

// ----------------------------------------------------------------------- RNG ------
enum RngMode { RNG_PHILOX = 0, RNG_MT19937 = 1 };

// Philox4x32-10 (Salmon et al., SC'11), written out independently of the device code.
static inline void philox_round(uint32_t* c, const uint32_t* k) {
    uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
    uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
    uint32_t n0 = uint32_t(p1 >> 32) ^ c[1] ^ k[0];
    uint32_t n1 = uint32_t(p1);
    uint32_t n2 = uint32_t(p0 >> 32) ^ c[3] ^ k[1];
    uint32_t n3 = uint32_t(p0);
    c[0] = n0;
    c[1] = n1;
    c[2] = n2;
    c[3] = n3;
}

static inline void philox10(uint32_t* c, uint32_t k0, uint32_t k1) {
    uint32_t k[2] = {k0, k1};
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k);
        k[0] += 0x9E3779B9u;
        k[1] += 0xBB67AE85u;
    }
}

// The device's stream definition (Philox mode), restated: a history id h and the run's seed
// (the key) give two kinds of draws.
//   * Event draws (source, interaction type, samplers, azimuths): draw n is the 32-bit word
//     (n & 3) of block (n >> 2, h_lo, h_hi, 0).  Each interaction starts a new block (n
//     rounded up to a multiple of 4).
//   * Woodcock-step draws: the step's two uniforms (free path, delta test) are the 32-bit
//     word pair (2 (i & 1), 2 (i & 1) + 1) of block (i >> 1, h_lo, h_hi, 1 + n), n the event
//     draws made so far - constant along a flight segment (the steps between two
//     interactions), different for every segment - and i = (Woodcock steps of the history
//     so far) + p, p the parity of that count at the segment's start, so that every segment
//     starts on a block boundary.  Two steps thus share one block.
struct Generator {
    int mode = RNG_PHILOX;
    // Philox history stream
    uint64_t seed = 0, history = 0;
    uint64_t draws = 0;
    uint64_t steps = 0;    // Woodcock steps of the history so far
    uint64_t parity = 0;   // of `steps` at the start of the current flight segment
    double step_u[2] = {0, 0};
    int step_left = 0;     // step uniforms not yet handed out by next()
    // mt19937 thread stream
    std::mt19937 mt;
    std::uniform_real_distribution<double> unit{0.0, 1.0};

    void startHistory(uint64_t h) {
        history = h;
        draws = 0;
        steps = 0;
        parity = 0;
        step_left = 0;
    }
    // A Woodcock step: its free-path and delta-test uniforms become the next two next() values.
    void beginStep() {
        if (mode != RNG_PHILOX) return;
        const uint64_t i = steps + parity;
        uint32_t c[4] = {uint32_t(i >> 1), uint32_t(history), uint32_t(history >> 32), uint32_t(1u + draws)};
        philox10(c, uint32_t(seed), uint32_t(seed >> 32));
        const int w = (i & 1) ? 2 : 0;
        for (int k = 0; k < 2; ++k) step_u[k] = double(((uint64_t(c[w + k]) << 32) >> 11) + 1) * (1.0 / 9007199254740992.0);
        step_left = 2;
        ++steps;
    }
    // An interaction: its draws start on a block boundary.
    void beginEvent() {
        if (mode == RNG_PHILOX) draws = (draws + 3) & ~uint64_t(3);
    }
    // A photon that leaves an interaction starts a new flight segment.
    void beginSegment() { parity = steps & 1; }
    double next() {
        if (mode == RNG_MT19937) return unit(mt);
        if (step_left) return step_u[2 - step_left--];
        uint32_t c[4] = {uint32_t(draws >> 2), uint32_t(history), uint32_t(history >> 32), 0u};
        philox10(c, uint32_t(seed), uint32_t(seed >> 32));
        const uint64_t r = uint64_t(c[draws & 3]) << 32;
        ++draws;
        return double((r >> 11) + 1) * (1.0 / 9007199254740992.0);
    }
};

thread_local Generator* tl_gen = nullptr;

// ProbabilityDist::Uniform: a range over the thread's generator.
struct Uniform {
    double lo = 0, hi = 1;
    Uniform() = default;
    Uniform(double a, double b) : lo(a), hi(b) {}
    double sample() const { return lo + (hi - lo) * tl_gen->next(); }
    void setRange(double a, double b) {
        lo = a;
        hi = b;
    }
};

// --------------------------------------------------------------------- vectors ------
struct Vec3 {
    double x = 0, y = 0, z = 0;
    Vec3() = default;
    Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
    Vec3 operator+(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
    Vec3 operator-(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
    Vec3 operator*(double s) const { return {x * s, y * s, z * s}; }
    double dot(const Vec3& o) const { return x * o.x + y * o.y + z * o.z; }
    Vec3 cross(const Vec3& o) const { return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x}; }
    double norm() const { return std::sqrt(dot(*this)); }
    Vec3 normalized() const {
        double n = norm();
        return n > 0 ? Vec3(x / n, y / n, z / n) : *this;
    }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct Quat {
    double w, x, y, z;
    Quat operator*(const Quat& o) const {
        return {w * o.w - x * o.x - y * o.y - z * o.z, w * o.x + x * o.w + y * o.z - z * o.y,
                w * o.y - x * o.z + y * o.w + z * o.x, w * o.z + x * o.y - y * o.x + z * o.w};
    }
    Quat inverse() const {
        double n2 = w * w + x * x + y * y + z * z;
        return {w / n2, -x / n2, -y / n2, -z / n2};
    }
};

Vec3 getPerpendicularVector(const Vec3& v) {
    if (std::abs(v.x) <= std::abs(v.y) && std::abs(v.x) <= std::abs(v.z)) return Vec3(1, 0, 0).cross(v);
    if (std::abs(v.y) <= std::abs(v.z)) return Vec3(0, 1, 0).cross(v);
    return Vec3(0, 0, 1).cross(v);
}

Vec3 rotateDirection(const Vec3& v, double theta, double phi) {
    Vec3 p = getPerpendicularVector(v).normalized();
    Quat qt{std::cos(theta / 2), p.x * std::sin(theta / 2), p.y * std::sin(theta / 2), p.z * std::sin(theta / 2)};
    Quat qp{std::cos(phi / 2), v.x * std::sin(phi / 2), v.y * std::sin(phi / 2), v.z * std::sin(phi / 2)};
    Quat q = qp * qt;
    Quat r = q * Quat{0, v.x, v.y, v.z} * q.inverse();
    return {r.x, r.y, r.z};
}

// --------------------------------------------------------------- interpolation ------
struct LogLogLinear {
    const double *x = nullptr, *lx = nullptr, *ly = nullptr;
    int n = 0;
    double operator()(double q) const {
        if (q <= x[0]) return std::pow(10, ly[0]);
        if (q >= x[n - 1]) return std::pow(10, ly[n - 1]);
        int idx = int(std::upper_bound(x, x + n, q) - x);
        double lq = std::log10(q);
        double slope = (ly[idx] - ly[idx - 1]) / (lx[idx] - lx[idx - 1]);
        return std::pow(10, ly[idx - 1] + slope * (lq - lx[idx - 1]));
    }
    int index(double q) const {
        if (q <= x[0]) return 0;
        if (q >= x[n - 1]) return n;
        return int(std::upper_bound(x, x + n, q) - x);
    }
};

struct LogLogSpline {
    const double *knot_e = nullptr, *knots = nullptr, *ctrl = nullptr;
    int n_ctrl = 0, degree = 0;
    double xmin = 0, xmax = 1;
    int span(double e) const {
        int nk = n_ctrl + degree + 1;
        if (e <= knot_e[0]) return degree;
        return int(std::upper_bound(knot_e + degree - 1, knot_e + nk - degree - 1, e) - knot_e) - 1;
    }
    double operator()(double e) const {
        int s = span(e);
        double u = (std::log10(e) - xmin) / (xmax - xmin);
        double N[4], left[4], right[4];
        N[0] = 1;
        for (int j = 1; j <= degree; ++j) {
            left[j] = u - knots[s + 1 - j];
            right[j] = knots[s + j] - u;
            double saved = 0;
            for (int r = 0; r < j; ++r) {
                double tmp = N[r] / (right[r + 1] + left[j - r]);
                N[r] = saved + right[r + 1] * tmp;
                saved = left[j - r] * tmp;
            }
            N[j] = saved;
        }
        double v = 0;
        for (int i = 0; i <= degree; ++i) v += ctrl[s - degree + i] * N[i];
        return std::pow(10, v);
    }
};

struct ContinuousInversion {
    const double *energies = nullptr, *log_energies = nullptr, *X = nullptr, *Y = nullptr, *A = nullptr,
                 *B = nullptr;
    const int64_t* rows = nullptr;
    int n_energy = 0;
    Uniform uniform_dist_{0.0, 1.0};

    int lowerIndex(double E) const {
        return int(std::lower_bound(energies, energies + n_energy, E) - energies) - 1;
    }
    double getXFromY(int k, double y) const {
        int64_t r0 = rows[k], r1 = rows[k + 1];
        int64_t j = (std::lower_bound(Y + r0, Y + r1, y) - (Y + r0)) - 1;
        int64_t n = r1 - r0;
        if (j == n - 1) return 1.0;
        if (j < 0) return -1.0;
        j += r0;
        double nu = y - Y[j], delta = Y[j + 1] - Y[j];
        return X[j] + (1 + A[j] + B[j]) * delta * nu / (delta * delta + A[j] * delta * nu + B[j] * nu * nu) *
                          (X[j + 1] - X[j]);
    }
    // returns false when E has no bracketing pair of table energies
    bool sample(double E, double& out) const {
        int lo = lowerIndex(E), hi = lo + 1;
        if (lo < 0 || hi >= n_energy) return false;
        double y = uniform_dist_.sample();
        double xl = getXFromY(lo, y), xu = getXFromY(hi, y);
        out = std::exp(std::log(xl + 1) + (std::log(xu + 1) - std::log(xl + 1)) * (std::log(E) - log_energies[lo]) /
                                              (log_energies[hi] - log_energies[lo])) -
              1.0;
        return true;
    }
};

struct MaterialData {
    LogLogLinear total, sfunc;
    LogLogSpline coh, incoh;
    ContinuousInversion rayleigh;
};

struct InteractionData {
    LogLogLinear majorant;
    std::vector<MaterialData> mats;
    std::vector<int> ids;
};

LogLogLinear make_lin(const midsx_table_blob* b, const midsx_lin_table& t) {
    LogLogLinear l;
    l.x = b->data + t.x;
    l.lx = b->data + t.lx;
    l.ly = b->data + t.ly;
    l.n = t.n;
    return l;
}

LogLogSpline make_spline(const midsx_table_blob* b, const midsx_spline_table& t) {
    LogLogSpline s;
    s.knot_e = b->data + t.knot_e;
    s.knots = b->data + t.knot_u;
    s.ctrl = b->data + t.ctrl;
    s.n_ctrl = t.n_ctrl;
    s.degree = t.degree;
    s.xmin = t.lx_min;
    s.xmax = t.lx_max;
    return s;
}

InteractionData make_interaction_data(const midsx_table_blob* b) {
    InteractionData d;
    d.majorant = make_lin(b, b->majorant);
    for (int m = 0; m < b->n_materials; ++m) {
        const midsx_material_table& t = b->mat[m];
        MaterialData md;
        md.total = make_lin(b, t.total);
        md.sfunc = make_lin(b, t.sfunc);
        md.coh = make_spline(b, t.coh);
        md.incoh = make_spline(b, t.incoh);
        md.rayleigh.energies = b->data + t.rita.energy;
        md.rayleigh.log_energies = b->data + t.rita.log_energy;
        md.rayleigh.X = b->data + t.rita.x;
        md.rayleigh.Y = b->data + t.rita.y;
        md.rayleigh.A = b->data + t.rita.a;
        md.rayleigh.B = b->data + t.rita.b;
        md.rayleigh.rows = b->idata + t.rita.row_start;
        md.rayleigh.n_energy = t.rita.n_energy;
        d.mats.push_back(md);
        d.ids.push_back(t.id);
    }
    return d;
}

// ----------------------------------------------------------------------- photon ------
struct Photon;
struct ParticleInteractionBehavior {
    virtual ~ParticleInteractionBehavior() = default;
    virtual double interact(Photon& p, const MaterialData& m) = 0;
};

struct Photon {
    Vec3 position, direction;
    double energy = 0;
    bool terminated = false, isPrimary = true;
    int coherent = 0, incoherent = 0, total = 0;
    bool failed = false;  // table range / trial cap
    std::shared_ptr<ParticleInteractionBehavior> behavior;
    void move(double d) { position = position + direction * d; }
    void rotate(double theta, double phi) { direction = rotateDirection(direction, theta, phi); }
    double interact(const MaterialData& m) { return behavior->interact(*this, m); }
};

struct Counters {
    uint64_t histories = 0, steps = 0, fetches = 0, photo = 0, coh = 0, incoh = 0, trials = 0, step_cap = 0,
             trial_cap = 0, edge = 0, words = 0, range_err = 0, nonfinite = 0;
    double source_e = 0, dep_grid = 0, dep_bg = 0, esc_e = 0;
    int max_trials = 100000;
};
thread_local Counters* tl_cnt = nullptr;

struct PhotoelectricEffect : ParticleInteractionBehavior {
    double interact(Photon& p, const MaterialData&) override {
        p.terminated = true;
        return p.energy;
    }
};

struct CoherentScattering : ParticleInteractionBehavior {
    Uniform uniform_dist_{0.0, 1.0};
    double interact(Photon& p, const MaterialData& m) override {
        double mu;
        if (!m.rayleigh.sample(p.energy, mu)) {
            tl_cnt->range_err++;
            p.failed = true;
            p.terminated = true;
            return 0;
        }
        double theta = std::acos(mu);
        double phi = 2 * PI * uniform_dist_.sample();
        p.rotate(theta, phi);
        return 0;
    }
};

struct IncoherentScattering : ParticleInteractionBehavior {
    Uniform uniform_dist_{0.0, 1.0};
    double interact(Photon& p, const MaterialData& m) override {
        double k = p.energy / ELECTRON_REST_MASS;
        double chi, mu, k_prime;
        for (int trial = 0; trial < tl_cnt->max_trials; ++trial) {
            tl_cnt->trials++;
            double r1 = uniform_dist_.sample(), r2 = uniform_dist_.sample(), r3 = uniform_dist_.sample();
            if (r1 <= (1 + 2 * k) / (9 + 2 * k)) {
                chi = 1 + 2 * k * r2;
                if (!(r3 <= 4 * (1 / chi - 1 / (chi * chi)))) continue;
            } else {
                chi = (1 + 2 * k) / (1 + 2 * k * r2);
                double t = 1 / k - chi / k + 1;
                if (!(2 * r3 <= t * t + 1 / chi)) continue;
            }
            k_prime = k / chi;
            mu = 1 + 1 / k - 1 / k_prime;
            double x = ALPHA * k * std::sqrt(1 - mu);
            double max_x = ALPHA * k * std::sqrt(2.0);
            double accept = m.sfunc(x) / m.sfunc(max_x);
            if (uniform_dist_.sample() <= accept) {
                double theta = std::acos(mu);
                double phi = 2 * PI * uniform_dist_.sample();
                p.rotate(theta, phi);
                p.energy = k_prime * ELECTRON_REST_MASS;
                return ELECTRON_REST_MASS * (k - k_prime);
            }
        }
        tl_cnt->trial_cap++;
        p.failed = true;
        p.terminated = true;
        return 0;
    }
};

// ---------------------------------------------------------------------- source ------
struct PhotonSource {
    Vec3 position;
    int dir_kind = 0, spec_kind = 0;
    Vec3 a, b, c, u, v;
    double radius = 0, mono = 0;
    std::vector<double> energy, cdf;
    Uniform uniform_dist_{0.0, 1.0};
    Uniform iso_dist_{0.0, 2 * PI};

    Photon generatePhoton() {
        Photon p;
        p.position = position;
        Vec3 d;
        switch (dir_kind) {
            case MIDSX_DIR_BEAM: d = (a - position).normalized(); break;
            case MIDSX_DIR_ISOTROPIC: {
                iso_dist_.setRange(0, PI);
                double theta = iso_dist_.sample();
                iso_dist_.setRange(0, 2 * PI);
                double phi = iso_dist_.sample();
                d = Vec3(std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta));
                break;
            }
            case MIDSX_DIR_RECTANGLE: {
                double a1 = uniform_dist_.sample(), a2 = uniform_dist_.sample();
                d = (a + b * a1 + c * a2 - position).normalized();
                break;
            }
            default: {
                Uniform ud(0, 2 * PI);
                double theta = ud.sample();
                ud.setRange(0, radius);
                double r = ud.sample();
                d = (a + (u * std::cos(theta) + v * std::sin(theta)) * r - position).normalized();
                break;
            }
        }
        p.direction = d;
        if (spec_kind == MIDSX_SPEC_MONO) {
            p.energy = mono;
        } else {
            double s = uniform_dist_.sample();
            size_t idx = size_t(std::lower_bound(cdf.begin(), cdf.end(), s) - cdf.begin());
            if (idx >= cdf.size()) idx = cdf.size() - 1;
            p.energy = energy[idx];
        }
        p.behavior = std::make_shared<PhotoelectricEffect>();
        return p;
    }
};

// ---------------------------------------------------------------------- geometry ------
// VoxelGrid at an origin: extent dims * spacing (VoxelGrid::setDimSpace), first voxel number
// `offset` in the domain's grid-after-grid numbering.
struct Grid {
    Vec3 origin, spacing, grid_dim;
    int dims[3] = {0, 0, 0};
    long offset = 0;
};

struct ComputationalDomain {
    Vec3 dim_space;
    std::vector<Grid> grids;   // voxel_grids_, searched in order
    int background = 0;        // dense material index
    std::vector<uint8_t> ids;  // dense material index per voxel, grid after grid

    bool isInComputationalDomain(const Vec3& p) const {
        return p.x >= 0 && p.x <= dim_space.x && p.y >= 0 && p.y <= dim_space.y && p.z >= 0 && p.z <= dim_space.z;
    }
    // the first grid containing p (withinGrid, inclusive bounds) gives the voxel: returns its
    // number, or -1 for the background voxel
    long getVoxel(const Vec3& p, int& mat) const {
        for (const Grid& g : grids) {
            Vec3 q = p - g.origin;
            if (!(q.x >= 0 && q.y >= 0 && q.z >= 0 && q.x <= g.grid_dim.x && q.y <= g.grid_dim.y &&
                  q.z <= g.grid_dim.z))
                continue;
            int i = int(q.x / g.spacing.x), j = int(q.y / g.spacing.y), k = int(q.z / g.spacing.z);
            if (i >= g.dims[0] || j >= g.dims[1] || k >= g.dims[2]) {
                tl_cnt->edge++;
                i = std::min(i, g.dims[0] - 1);
                j = std::min(j, g.dims[1] - 1);
                k = std::min(k, g.dims[2] - 1);
            }
            long n = g.offset + long(i) + long(j) * g.dims[0] + long(k) * g.dims[0] * g.dims[1];
            mat = ids[size_t(n)];
            tl_cnt->fetches++;
            return n;
        }
        mat = background;
        return -1;
    }
};

// ---------------------------------------------------------------------- tallies ------
struct VectorValue {
    std::vector<double> values;
    void addValue(double v) { values.push_back(v); }
};

struct TempSurfaceTallyData {
    double free_path = 0;
    bool isInteract = false;
    double entrance_cosine = 0;
    bool already_counted = false;
    Photon initial_photon;
};

struct TempVolumeTallyData {
    double energy_deposited = 0, free_path = 0;
    bool isInteract = false, already_counted = false;
    Photon initial_photon, final_photon;
};

struct TempVoxelData {
    long voxel;
    double energy_deposited;
};

int classOf(const Photon& p) {
    if (p.total > 1) return 3;
    if (p.coherent == 1) return 1;
    if (p.incoherent == 1) return 2;
    return 0;
}

// Per-thread replica of one tally: vectors of every measured value per quantity and class.
struct TallyReplica {
    midsx_tally_spec spec;
    Vec3 norm;
    double e1e1 = 0, e2e2 = 0;
    VectorValue vec[2][4];
    int64_t cnt[2][4] = {{0}};
    std::vector<double> bin_e;   // binned: [bin][class]
    std::vector<int64_t> bin_n;

    void measureVector(int q, int cls, double value) {
        if (value == 0) return;
        vec[q][cls].addValue(value);
        tl_cnt->words++;
    }

    void processSurface(TempSurfaceTallyData d) {
        Photon& p = d.initial_photon;
        double ec = p.direction.dot(norm);
        if (std::abs(ec) < EPSILON || ec < 0) return;
        Vec3 a(spec.a[0], spec.a[1], spec.a[2]);
        double t = (a - p.position).dot(norm) / ec;
        if (t > d.free_path || t < 0) return;
        Vec3 ip = p.position + p.direction * t;
        int cls = classOf(p);
        if (spec.kind == MIDSX_TALLY_SURFACE_DISC) {
            if ((ip - a).norm() > spec.radius) return;
        } else {
            Vec3 e1(spec.b[0], spec.b[1], spec.b[2]), e2(spec.c[0], spec.c[1], spec.c[2]);
            Vec3 r = ip - a;
            double u = e1.dot(r), v = e2.dot(r);
            if (u < 0 || u > e1e1 || v < 0 || v > e2e2) return;
            if (spec.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
                int iu = std::min(int(u / e1e1 * spec.nu), spec.nu - 1);
                int iv = std::min(int(v / e2e2 * spec.nv), spec.nv - 1);
                size_t bin = (size_t(iv) * spec.nu + iu) * 4 + cls;
                bin_e[bin] += p.energy;
                bin_n[bin] += 1;
                tl_cnt->words++;
                return;
            }
        }
        d.entrance_cosine = ec;
        measureVector(0, cls, p.energy);
        measureVector(1, cls, d.entrance_cosine);
        if (!d.already_counted) {
            cnt[0][cls]++;
            tl_cnt->words++;
        }
    }

    void processVolume(TempVolumeTallyData d) {
        Photon& p = d.initial_photon;
        Vec3 mn(spec.a[0], spec.a[1], spec.a[2]), mx(spec.b[0], spec.b[1], spec.b[2]);
        double lo[3], hi[3];
        for (int i = 0; i < 3; ++i) {
            if (std::abs(p.direction[i]) < EPSILON) {
                lo[i] = -INF;
                hi[i] = INF;
                continue;
            }
            lo[i] = (mn[i] - p.position[i]) / p.direction[i];
            hi[i] = (mx[i] - p.position[i]) / p.direction[i];
            if (lo[i] > hi[i]) std::swap(lo[i], hi[i]);
        }
        double enter = std::max(std::max(lo[0], lo[1]), lo[2]);
        double exit = std::min(std::min(hi[0], hi[1]), hi[2]);
        if (enter > exit || exit < 0 || enter > d.free_path) return;  // MISSES
        if (enter <= 0) {
            if (exit >= d.free_path) {  // STARTS_INSIDE_STAYS
                d.already_counted = true;
            } else {  // STARTS_INSIDE_EXITS
                d.energy_deposited = 0;
                d.already_counted = true;
            }
        } else if (exit < d.free_path) {  // PASSES_THROUGH
            d.energy_deposited = 0;
        }  // else LANDS_INSIDE
        int cls = classOf(d.final_photon);
        measureVector(0, cls, d.energy_deposited);
        measureVector(1, cls, d.already_counted ? 0.0 : d.initial_photon.energy);
        if (!d.already_counted) {
            cnt[0][cls]++;
            tl_cnt->words++;
        }
        if (d.isInteract) {
            cnt[1][cls]++;
            tl_cnt->words++;
        }
    }
};

// ----------------------------------------------------------------- physics engine ------
struct PhysicsEngine {
    const ComputationalDomain& dom;
    const InteractionData& data;
    Uniform uniform_dist_{0.0, 1.0};
    std::shared_ptr<PhotoelectricEffect> photoelectric_effect_ = std::make_shared<PhotoelectricEffect>();
    std::shared_ptr<CoherentScattering> coherent_scattering_ = std::make_shared<CoherentScattering>();
    std::shared_ptr<IncoherentScattering> incoherent_scattering_ = std::make_shared<IncoherentScattering>();
    int max_steps = 1000000;

    PhysicsEngine(const ComputationalDomain& d, const InteractionData& i) : dom(d), data(i) {}

    double getFreePath(double mu_max) {
        tl_gen->beginStep();
        return -std::log(uniform_dist_.sample()) / mu_max;
    }
    bool isDeltaScatter(double mu, double mu_max) {
        double p = 1 - mu / mu_max;
        return uniform_dist_.sample() < p;
    }

    void setInteractionType(Photon& photon, const MaterialData& m, double total) {
        double E = photon.energy;
        double p_coh = m.coh(E) / total;
        double p_incoh = m.incoh(E) / total;
        double r = uniform_dist_.sample();
        if (r < p_coh) {
            photon.coherent++;
            photon.total++;
            photon.behavior = coherent_scattering_;
        } else if (r < p_coh + p_incoh) {
            photon.incoherent++;
            photon.total++;
            photon.behavior = incoherent_scattering_;
        } else {
            photon.behavior = photoelectric_effect_;
        }
    }

    void transportPhotonOneStep(Photon& photon, std::vector<TempSurfaceTallyData>& ts,
                                std::vector<TempVolumeTallyData>& tv, std::vector<TempVoxelData>& tx) {
        TempSurfaceTallyData sd;
        TempVolumeTallyData vd;
        sd.initial_photon = vd.initial_photon = photon;
        tl_cnt->steps++;
        double E = photon.energy;
        double mu_max = data.majorant(E);
        double s = getFreePath(mu_max);
        sd.free_path = vd.free_path = s;
        photon.move(s);
        if (!dom.isInComputationalDomain(photon.position)) {
            ts.push_back(sd);
            tv.push_back(vd);
            tl_cnt->esc_e += photon.energy;
            photon.terminated = true;
            return;
        }
        int mat;
        long voxel = dom.getVoxel(photon.position, mat);
        const MaterialData& m = data.mats[size_t(mat)];
        double mu = m.total(E);
        if (!isDeltaScatter(mu, mu_max)) {
            sd.isInteract = vd.isInteract = true;
            tl_gen->beginEvent();
            setInteractionType(photon, m, mu);
            photon.isPrimary = false;
            auto* beh = photon.behavior.get();
            if (beh == photoelectric_effect_.get()) tl_cnt->photo++;
            else if (beh == coherent_scattering_.get()) tl_cnt->coh++;
            else tl_cnt->incoh++;
            double dep = photon.interact(m);
            if (photon.failed) return;  // table range or trial cap: drop the history's step
            if (!photon.terminated) tl_gen->beginSegment();
            vd.energy_deposited = dep;
            vd.final_photon = photon;
            tx.push_back({voxel, dep});
            if (!photon.terminated &&
                !(std::abs(photon.direction.x) <= 2 && std::abs(photon.direction.y) <= 2 &&
                  std::abs(photon.direction.z) <= 2)) {
                tl_cnt->nonfinite++;
                tl_cnt->esc_e += photon.energy;
                ts.push_back(sd);
                tv.push_back(vd);
                photon.terminated = true;
                return;
            }
        }
        ts.push_back(sd);
        tv.push_back(vd);
    }
};

struct ThreadState {
    std::vector<TallyReplica> tallies;
    std::vector<TempVoxelData> voxel_data;
    std::vector<TempVoxelData> history_voxel;  // per history and voxel: all its deposits there
    Counters cnt;
    Generator gen;
};

}  // namespace ref

// ------------------------------------------------------------------------- C ABI ------
extern "C" {

typedef struct oracle_result {
    double* dose_sum;       /* n_voxels or NULL */
    double* dose_sumsq;     /* n_voxels or NULL */
    double* dose_count;     /* n_voxels or NULL */
    double* scalar;         /* n_specs * MIDSX_SCALAR_SLOTS or NULL */
    double* binned_energy;  /* sum over binned specs of nu*nv*4, in spec order, or NULL */
    double* binned_count;
    double* history_deposit;/* n histories: energy deposited in grid voxels, or NULL */
    midsx_run_stats stats;
    double run_time;        /* seconds in the history loop (the reference's run_time) */
    /* incident-energy spectra of the DISC / RECT specs with n_energy > 0, binned from the
     * raw IncidentEnergy / EntranceCosine vectors: [bin][class] crossings and cosine sums,
     * specs in order, or NULL */
    double* spectrum_count;
    double* spectrum_cosine;
    /* the raw primary IncidentEnergy and EntranceCosine vectors of surface spec raw_spec
     * (-1: none), up to raw_cap values each; raw_n receives the number of values */
    int32_t raw_spec;
    int32_t reserved;
    int64_t raw_cap;
    double* raw_energy;
    double* raw_cosine;
    int64_t raw_n;
    /* per-history variance of each voxel's dose sum, or NULL: N / (N - 1) * (sum_h x_h^2 -
     * S^2 / N), x_h the energy history h deposited in the voxel (all its deposits there
     * together), S the voxel's sum - the estimator the reference's event-based sigma
     * (src/MIDSX/Core/quantity.cpp:37-45) is not */
    double* dose_var_hist;
} oracle_result;

}  // extern "C"

namespace {

// The history loop over an assembled domain; nvox = voxels of all grids.
int run_domain(const midsx_table_blob* blob, ref::ComputationalDomain& dom, size_t nvox, const midsx_source_spec* src,
               const midsx_tally_spec* specs, int n_specs, uint64_t seed, uint64_t first, uint64_t n, int rng_mode,
               int n_threads, int max_steps, int max_trials, oracle_result* out);

// Domain of `n_grids` grids with MIDSX material ids, remapped to the tables' dense indices.
int build_domain(const midsx_table_blob* blob, const double* domain, int background_id, const midsx_grid_spec* grids,
                 int n_grids, ref::ComputationalDomain& dom, size_t& nvox) {
    using namespace ref;
    dom.dim_space = Vec3(domain[0], domain[1], domain[2]);
    int lut[256];
    for (int& v : lut) v = -1;
    for (int m = 0; m < blob->n_materials; ++m) lut[blob->mat[m].id & 0xFF] = m;
    if (lut[background_id & 0xFF] < 0) return 2;
    dom.background = lut[background_id & 0xFF];
    nvox = 0;
    for (int k = 0; k < n_grids; ++k) {
        const midsx_grid_spec& gs = grids[k];
        if (!gs.ids) return 1;
        Grid g;
        g.origin = Vec3(gs.origin[0], gs.origin[1], gs.origin[2]);
        g.spacing = Vec3(gs.spacing[0], gs.spacing[1], gs.spacing[2]);
        for (int i = 0; i < 3; ++i) g.dims[i] = gs.dims[i];
        g.grid_dim = Vec3(g.dims[0] * g.spacing.x, g.dims[1] * g.spacing.y, g.dims[2] * g.spacing.z);
        g.offset = long(nvox);
        const size_t nv = size_t(g.dims[0]) * g.dims[1] * g.dims[2];
        for (size_t i = 0; i < nv; ++i) {
            if (lut[gs.ids[i]] < 0) return 2;
            dom.ids.push_back(uint8_t(lut[gs.ids[i]]));
        }
        nvox += nv;
        dom.grids.push_back(g);
    }
    return 0;
}

}  // namespace

extern "C" {

/* Runs n histories [first, first + n).  ids are MIDSX material ids (uint8 per voxel).
 * Returns 0 on success, 1 bad argument, 2 unknown material id. */
int oracle_run(const midsx_table_blob* blob, const midsx_geometry_spec* geom, const uint8_t* ids,
               const midsx_source_spec* src, const midsx_tally_spec* specs, int n_specs, uint64_t seed,
               uint64_t first, uint64_t n, int rng_mode, int n_threads, int max_steps, int max_trials,
               oracle_result* out) {
    if (!blob || !geom || !ids || !src || !out || n_specs < 0) return 1;
    midsx_grid_spec one;
    std::memset(&one, 0, sizeof(one));
    for (int i = 0; i < 3; ++i) {
        one.spacing[i] = geom->spacing[i];
        one.origin[i] = geom->origin[i];
        one.dims[i] = geom->dims[i];
    }
    one.ids = ids;
    ref::ComputationalDomain dom;
    size_t nvox = 0;
    int rc = build_domain(blob, geom->domain, geom->background_id, &one, 1, dom, nvox);
    if (rc) return rc;
    return run_domain(blob, dom, nvox, src, specs, n_specs, seed, first, n, rng_mode, n_threads, max_steps,
                      max_trials, out);
}

/* Several grids (ComputationalDomain::voxel_grids_, first-hit order); voxels numbered grid
 * after grid in the dose outputs. */
int oracle_run_grids(const midsx_table_blob* blob, const double* domain, int background_id,
                     const midsx_grid_spec* grids, int n_grids, const midsx_source_spec* src,
                     const midsx_tally_spec* specs, int n_specs, uint64_t seed, uint64_t first, uint64_t n,
                     int rng_mode, int n_threads, int max_steps, int max_trials, oracle_result* out) {
    if (!blob || !domain || !grids || n_grids < 1 || !src || !out || n_specs < 0) return 1;
    ref::ComputationalDomain dom;
    size_t nvox = 0;
    int rc = build_domain(blob, domain, background_id, grids, n_grids, dom, nvox);
    if (rc) return rc;
    return run_domain(blob, dom, nvox, src, specs, n_specs, seed, first, n, rng_mode, n_threads, max_steps,
                      max_trials, out);
}

}  // extern "C"

namespace {

int run_domain(const midsx_table_blob* blob, ref::ComputationalDomain& dom, size_t nvox, const midsx_source_spec* src,
               const midsx_tally_spec* specs, int n_specs, uint64_t seed, uint64_t first, uint64_t n, int rng_mode,
               int n_threads, int max_steps, int max_trials, oracle_result* out) {
    using namespace ref;
    InteractionData data = make_interaction_data(blob);
    PhotonSource source;
    source.position = Vec3(src->position[0], src->position[1], src->position[2]);
    source.dir_kind = src->direction_kind;
    source.spec_kind = src->spectrum_kind;
    source.a = Vec3(src->a[0], src->a[1], src->a[2]);
    source.b = Vec3(src->b[0], src->b[1], src->b[2]);
    source.c = Vec3(src->c[0], src->c[1], src->c[2]);
    source.radius = src->radius;
    source.mono = src->mono_energy;
    if (src->direction_kind == MIDSX_DIR_DISC) {
        Vec3 nrm = source.b;
        source.u = (std::abs(nrm.dot(Vec3(1, 0, 0))) < 1e-9 ? nrm.cross(Vec3(0, 1, 0)) : nrm.cross(Vec3(1, 0, 0)))
                       .normalized();
        source.v = nrm.cross(source.u).normalized();
    }
    if (src->spectrum_kind == MIDSX_SPEC_POLY) {
        double sum = 0;
        for (int i = 0; i < src->n_bins; ++i) sum += src->bin_prob[i];
        double acc = 0;
        for (int i = 0; i < src->n_bins; ++i) {
            double p = sum != 1.0 ? src->bin_prob[i] / sum : src->bin_prob[i];
            acc = i == 0 ? p : acc + p;
            source.energy.push_back(src->bin_energy[i]);
            source.cdf.push_back(acc);
        }
    }
    if (n_threads <= 0) n_threads = omp_get_max_threads();
    std::vector<ThreadState> states;
    states.resize(size_t(n_threads));
    for (int t = 0; t < n_threads; ++t) {
        ThreadState& st = states[size_t(t)];
        st.gen.mode = rng_mode;
        st.gen.seed = seed;
        if (rng_mode == RNG_MT19937) st.gen.mt.seed(uint32_t(seed * 1000003u + uint64_t(t) * 7919u + 17u));
        st.cnt.max_trials = max_trials > 0 ? max_trials : 100000;
        for (int i = 0; i < n_specs; ++i) {
            TallyReplica r;
            r.spec = specs[i];
            if (r.spec.kind == MIDSX_TALLY_SURFACE_DISC) {
                r.norm = Vec3(r.spec.b[0], r.spec.b[1], r.spec.b[2]);
            } else if (r.spec.kind != MIDSX_TALLY_VOLUME_AACUBOID) {
                Vec3 e1(r.spec.b[0], r.spec.b[1], r.spec.b[2]), e2(r.spec.c[0], r.spec.c[1], r.spec.c[2]);
                r.norm = e1.cross(e2).normalized();
                r.e1e1 = e1.dot(e1);
                r.e2e2 = e2.dot(e2);
                if (r.spec.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
                    r.bin_e.assign(size_t(r.spec.nu) * r.spec.nv * 4, 0.0);
                    r.bin_n.assign(size_t(r.spec.nu) * r.spec.nv * 4, 0);
                }
            }
            st.tallies.push_back(std::move(r));
        }
    }
    if (out->history_deposit)
        for (uint64_t i = 0; i < n; ++i) out->history_deposit[i] = 0;
    // the reference's loop has no cap; the oracle's default is the device's derived one: 16
    // crossings of the domain diagonal at the largest majorant between min(1 keV, the source's
    // lowest energy) and e_max (at least 100,000), so a hit marks a runaway history, not a cut
    int steps_cap = max_steps;
    if (steps_cap <= 0) {
        double e_lo = src->spectrum_kind == MIDSX_SPEC_POLY ? INF : src->mono_energy;
        for (int i = 0; src->spectrum_kind == MIDSX_SPEC_POLY && i < src->n_bins; ++i)
            if (src->bin_prob[i] > 0) e_lo = std::min(e_lo, src->bin_energy[i]);
        const double e_floor = std::min(1e3, e_lo);
        const midsx_lin_table& mj = blob->majorant;
        double mu_hi = data.majorant(e_floor);
        for (int i = 0; i < mj.n; ++i) {
            const double e = blob->data[mj.x + i];
            if (e >= e_floor && e <= blob->e_max) mu_hi = std::max(mu_hi, std::pow(10.0, blob->data[mj.ly + i]));
        }
        const Vec3& d = dom.dim_space;
        const double cap = std::ceil(16.0 * std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z) * mu_hi);
        steps_cap = !(cap > 1e5) ? 100000 : (cap >= 2147483647.0 ? 2147483647 : int(cap));
    }
    int progress = 0;
    auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(n_threads)
    {
        ThreadState& st = states[size_t(omp_get_thread_num())];
        tl_gen = &st.gen;
        tl_cnt = &st.cnt;
        PhysicsEngine engine(dom, data);
        engine.max_steps = steps_cap;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < int64_t(n); ++i) {
            st.gen.startHistory(first + uint64_t(i));
            Photon photon = source.generatePhoton();
            st.cnt.histories++;
            st.cnt.source_e += photon.energy;
            std::vector<TempSurfaceTallyData> ts;
            std::vector<TempVolumeTallyData> tv;
            std::vector<TempVoxelData> tx;
            int steps = 0;
            while (!photon.terminated) {
                if (steps++ >= steps_cap) {
                    st.cnt.step_cap++;
                    break;
                }
                engine.transportPhotonOneStep(photon, ts, tv, tx);
            }
            // processTallies
            for (auto& tr : st.tallies) {
                if (tr.spec.kind == MIDSX_TALLY_VOLUME_AACUBOID) {
                    for (auto& d : tv) tr.processVolume(d);
                } else {
                    for (auto& d : ts) tr.processSurface(d);
                }
            }
            double hist_dep = 0;
            const size_t hv0 = st.history_voxel.size();
            for (auto& d : tx) {
                if (d.energy_deposited != 0.0) {
                    if (d.voxel >= 0) {
                        st.voxel_data.push_back(d);
                        st.cnt.dep_grid += d.energy_deposited;
                        hist_dep += d.energy_deposited;
                        st.cnt.words++;
                        if (out->dose_var_hist) {  // this history's total in the voxel
                            size_t k = hv0;
                            while (k < st.history_voxel.size() && st.history_voxel[k].voxel != d.voxel) ++k;
                            if (k == st.history_voxel.size()) st.history_voxel.push_back({d.voxel, 0.0});
                            st.history_voxel[k].energy_deposited += d.energy_deposited;
                        }
                    } else {
                        st.cnt.dep_bg += d.energy_deposited;
                    }
                }
            }
            if (out->history_deposit) out->history_deposit[i] = hist_dep;
#pragma omp critical(oracle_progress)
            {
                // runSimulation's per-photon progress section (output suppressed)
                int64_t every = std::max<int64_t>(1, int64_t(n) / 20);
                if (i % every == 0) progress += 5;
            }
        }
    }
    out->run_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // merge replicas (getVolume/SurfaceQuantityContainers, addVoxelDataToComputationalDomain)
    if (out->dose_sum || out->dose_sumsq || out->dose_count || out->dose_var_hist) {
        std::vector<double> s(nvox, 0.0), s2(nvox, 0.0), c(nvox, 0.0);
        for (auto& st : states)
            for (auto& d : st.voxel_data) {
                s[size_t(d.voxel)] += d.energy_deposited;
                s2[size_t(d.voxel)] += d.energy_deposited * d.energy_deposited;
                c[size_t(d.voxel)] += 1;
            }
        if (out->dose_var_hist) {
            std::vector<double> h2(nvox, 0.0);
            for (auto& st : states)
                for (auto& d : st.history_voxel) h2[size_t(d.voxel)] += d.energy_deposited * d.energy_deposited;
            const double N = double(n);
            for (size_t i = 0; i < nvox; ++i)
                out->dose_var_hist[i] = N > 1 ? N / (N - 1) * std::max(0.0, h2[i] - s[i] * s[i] / N) : 0.0;
        }
        if (out->dose_sum) std::memcpy(out->dose_sum, s.data(), nvox * 8);
        if (out->dose_sumsq) std::memcpy(out->dose_sumsq, s2.data(), nvox * 8);
        if (out->dose_count) std::memcpy(out->dose_count, c.data(), nvox * 8);
    }
    // spectra: every raw (IncidentEnergy, EntranceCosine) pair binned by energy; both values
    // of a crossing are non-zero, so the two vectors of a class run in step
    size_t soff = 0;
    for (int i = 0; i < n_specs; ++i) {
        const midsx_tally_spec& sp = specs[i];
        if (sp.n_energy <= 0) continue;
        const size_t cells = size_t(sp.n_energy) * 4;
        std::vector<double> cnt(cells, 0.0), cs(cells, 0.0);
        for (auto& st : states) {
            TallyReplica& r = st.tallies[size_t(i)];
            for (int c = 0; c < 4; ++c) {
                const auto& ev = r.vec[0][c].values;
                const auto& cv = r.vec[1][c].values;
                for (size_t k = 0; k < ev.size() && k < cv.size(); ++k) {
                    const double b = (ev[k] - sp.e_min) / sp.e_width;
                    if (!(b >= 0) || b >= double(sp.n_energy)) continue;
                    const size_t cell = size_t(int(b)) * 4 + size_t(c);
                    cnt[cell] += 1;
                    cs[cell] += cv[k];
                }
            }
        }
        if (out->spectrum_count) std::memcpy(out->spectrum_count + soff, cnt.data(), cells * 8);
        if (out->spectrum_cosine) std::memcpy(out->spectrum_cosine + soff, cs.data(), cells * 8);
        soff += cells;
    }
    out->raw_n = 0;
    if (out->raw_spec >= 0 && out->raw_spec < n_specs) {
        for (auto& st : states) {
            TallyReplica& r = st.tallies[size_t(out->raw_spec)];
            const auto& ev = r.vec[0][0].values;
            const auto& cv = r.vec[1][0].values;
            for (size_t k = 0; k < ev.size() && k < cv.size() && out->raw_n < out->raw_cap; ++k) {
                if (out->raw_energy) out->raw_energy[out->raw_n] = ev[k];
                if (out->raw_cosine) out->raw_cosine[out->raw_n] = cv[k];
                out->raw_n++;
            }
        }
    }
    size_t boff = 0;
    for (int i = 0; i < n_specs; ++i) {
        const bool binned = specs[i].kind == MIDSX_TALLY_SURFACE_BINNED_RECT;
        if (binned) {
            size_t nb = size_t(specs[i].nu) * specs[i].nv * 4;
            for (size_t k = 0; k < nb; ++k) {
                double e = 0, c = 0;
                for (auto& st : states) {
                    e += st.tallies[size_t(i)].bin_e[k];
                    c += double(st.tallies[size_t(i)].bin_n[k]);
                }
                if (out->binned_energy) out->binned_energy[boff + k] = e;
                if (out->binned_count) out->binned_count[boff + k] = c;
            }
            boff += nb;
            continue;
        }
        if (!out->scalar) continue;
        double* o = out->scalar + size_t(i) * MIDSX_SCALAR_SLOTS;
        for (int k = 0; k < MIDSX_SCALAR_SLOTS; ++k) o[k] = 0;
        for (auto& st : states) {
            TallyReplica& r = st.tallies[size_t(i)];
            for (int q = 0; q < 2; ++q)
                for (int c = 0; c < 4; ++c) {
                    double* b = o + q * 12 + c * 3;
                    for (double v : r.vec[q][c].values) {
                        b[0] += 1;
                        b[1] += v;
                        b[2] += v * v;
                    }
                    o[24 + q * 4 + c] += double(r.cnt[q][c]);
                }
        }
    }
    midsx_run_stats& S = out->stats;
    std::memset(&S, 0, sizeof(S));
    for (auto& st : states) {
        const Counters& c = st.cnt;
        S.histories += c.histories;
        S.steps += c.steps;
        S.voxel_fetches += c.fetches;
        S.photo += c.photo;
        S.coherent += c.coh;
        S.incoherent += c.incoh;
        S.compton_trials += c.trials;
        S.step_cap_hits += c.step_cap;
        S.compton_cap_hits += c.trial_cap;
        S.edge_clamps += c.edge;
        S.tally_words += c.words;
        S.source_energy += c.source_e;
        S.deposited_grid += c.dep_grid;
        S.deposited_background += c.dep_bg;
        S.escaped_energy += c.esc_e;
    }
    return 0;
}

}  // namespace

extern "C" {

/* Sampler harness for the KS tests: n draws of one sampler with history streams
 * [first, first + n) (Philox) - kind 0 Rayleigh cosine, 1 Compton (cos, E'/E),
 * 2 free path at E against the majorant. */
int oracle_sample(const midsx_table_blob* blob, int kind, int material, double energy, uint64_t seed,
                  uint64_t first, int64_t n, int rng_mode, double* out0, double* out1) {
    using namespace ref;
    if (!blob || material < 0 || material >= blob->n_materials || n <= 0 || !out0) return 1;
    InteractionData data = make_interaction_data(blob);
    const MaterialData& m = data.mats[size_t(material)];
#pragma omp parallel
    {
        Generator gen;
        gen.mode = rng_mode;
        gen.seed = seed;
        gen.mt.seed(uint32_t(seed * 1000003u + uint64_t(omp_get_thread_num()) * 7919u + 17u));
        Counters cnt;
        tl_gen = &gen;
        tl_cnt = &cnt;
        CoherentScattering coh;
        IncoherentScattering inc;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            gen.startHistory(first + uint64_t(i));
            if (kind == 0) {
                double mu;
                out0[i] = m.rayleigh.sample(energy, mu) ? mu : NAN;
            } else if (kind == 1) {
                // the Compton sampler without the final rotation draw
                double k = energy / ELECTRON_REST_MASS, mu = 1, kp = k;
                Uniform ud(0, 1);
                for (int t = 0; t < 100000; ++t) {
                    double r1 = ud.sample(), r2 = ud.sample(), r3 = ud.sample(), chi;
                    if (r1 <= (1 + 2 * k) / (9 + 2 * k)) {
                        chi = 1 + 2 * k * r2;
                        if (!(r3 <= 4 * (1 / chi - 1 / (chi * chi)))) continue;
                    } else {
                        chi = (1 + 2 * k) / (1 + 2 * k * r2);
                        double tt = 1 / k - chi / k + 1;
                        if (!(2 * r3 <= tt * tt + 1 / chi)) continue;
                    }
                    kp = k / chi;
                    mu = 1 + 1 / k - 1 / kp;
                    double x = ALPHA * k * std::sqrt(1 - mu);
                    if (ud.sample() <= m.sfunc(x) / m.sfunc(ALPHA * k * std::sqrt(2.0))) break;
                }
                out0[i] = mu;
                if (out1) out1[i] = kp / k;
            } else {
                Uniform ud(0, 1);
                out0[i] = -std::log(ud.sample()) / data.majorant(energy);
            }
        }
    }
    return 0;
}

/* Table indices of the oracle's lookups (same layout as midsx_gpu_table_index). */
int oracle_table_index(const midsx_table_blob* blob, int material, const double* e, int64_t n, int64_t* idx) {
    using namespace ref;
    if (!blob || material < 0 || material >= blob->n_materials || !e || !idx) return 1;
    InteractionData data = make_interaction_data(blob);
    const MaterialData& m = data.mats[size_t(material)];
    for (int64_t i = 0; i < n; ++i) {
        idx[6 * i + 0] = data.majorant.index(e[i]);
        idx[6 * i + 1] = m.total.index(e[i]);
        idx[6 * i + 2] = m.sfunc.index(e[i]);
        idx[6 * i + 3] = m.coh.span(e[i]);
        idx[6 * i + 4] = m.incoh.span(e[i]);
        idx[6 * i + 5] = m.rayleigh.lowerIndex(e[i]);
    }
    return 0;
}

/* Philox4x32-10 block for known-answer tests. */
void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    ref::philox10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}

/* The Philox-mode generator of one history driven by a script, for tests of its draw
 * layout: op 0 = one draw (event draw, or the next step uniform after op 2), 1 =
 * beginEvent, 2 = beginStep, 3 = beginSegment.  out receives every draw's value. */
int oracle_generator_script(uint64_t seed, uint64_t history, const int32_t* ops, int64_t n_ops, double* out) {
    ref::Generator g;
    g.mode = ref::RNG_PHILOX;
    g.seed = seed;
    g.startHistory(history);
    int64_t k = 0;
    for (int64_t i = 0; i < n_ops; ++i) {
        switch (ops[i]) {
            case 0: out[k++] = g.next(); break;
            case 1: g.beginEvent(); break;
            case 2: g.beginStep(); break;
            case 3: g.beginSegment(); break;
            default: return 1;
        }
    }
    return 0;
}

}  // extern "C"
