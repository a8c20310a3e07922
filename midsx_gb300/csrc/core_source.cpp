// core_source.cpp - PhotonSource and its parts (reference: src/MIDSX/Core/source.cpp:5-155,
// src/MIDSX/Core/probability_dist.cpp:11-60).  Host sampling uses a thread-local mt19937 as
// the reference does; device sampling uses the description returned by describe().
#include <cmath>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <stdexcept>

#include "MIDSX/Core/constants.h"
#include "MIDSX/Core/source.h"

namespace {
double uni() {
    thread_local std::mt19937 gen{std::random_device{}()};
    thread_local std::uniform_real_distribution<double> unit(0.0, 1.0);
    return unit(gen);
}
void put(double* d, const Vec3& v) {
    d[0] = v.x();
    d[1] = v.y();
    d[2] = v.z();
}
}  // namespace

Vec3 SourceHelpers::angleToUnitDirection(double theta, double phi) {
    return {std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta)};
}

midsx::Matrix SourceHelpers::readCSV(const std::string& file) {
    std::string ext = file.size() > 4 ? file.substr(file.size() - 4) : "";
    if (ext != ".csv" && ext != ".txt") throw std::invalid_argument("File is not a csv or txt file");
    std::ifstream in(file);
    if (!in) throw std::invalid_argument("File does not exist");
    std::vector<std::vector<double>> rows;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::stringstream ls(line);
        std::string cell;
        std::vector<double> row;
        while (std::getline(ls, cell, ',')) row.push_back(std::stod(cell));
        rows.push_back(row);
    }
    return midsx::Matrix(rows);
}

void EnergySpectrum::describe(midsx_source_spec&) const {
    throw std::invalid_argument("this EnergySpectrum type has no GPU implementation");
}
void Directionality::describe(midsx_source_spec&) const {
    throw std::invalid_argument("this Directionality type has no GPU implementation");
}
void SourceGeometry::describe(midsx_source_spec&) const {
    throw std::invalid_argument("this SourceGeometry type has no GPU implementation");
}

void MonoenergeticSpectrum::describe(midsx_source_spec& s) const {
    s.spectrum_kind = MIDSX_SPEC_MONO;
    s.mono_energy = energy_;
}

PolyenergeticSpectrum::PolyenergeticSpectrum(const std::vector<std::pair<double, double>>& p) {
    for (auto& r : p) {
        energy_.push_back(r.first);
        prob_.push_back(r.second);
    }
    init();
}

PolyenergeticSpectrum::PolyenergeticSpectrum(const std::vector<std::vector<double>>& p) {
    for (auto& r : p) {
        if (r.size() < 2) throw std::invalid_argument("spectrum rows need (energy, probability)");
        energy_.push_back(r[0]);
        prob_.push_back(r[1]);
    }
    init();
}

void PolyenergeticSpectrum::init() {
    if (energy_.empty() || energy_.size() > MIDSX_MAX_SPECTRUM_BINS) throw std::invalid_argument("bad spectrum size");
    double sum = 0;
    for (double p : prob_) sum += p;
    if (sum != 1.0)
        for (double& p : prob_) p /= sum;
    cdf_.resize(prob_.size());
    double acc = 0;
    for (size_t i = 0; i < prob_.size(); ++i) cdf_[i] = acc = (i == 0 ? prob_[i] : acc + prob_[i]);
}

double PolyenergeticSpectrum::sampleEnergy() {
    size_t idx = size_t(std::lower_bound(cdf_.begin(), cdf_.end(), uni()) - cdf_.begin());
    return energy_[std::min(idx, energy_.size() - 1)];
}

double PolyenergeticSpectrum::getExpectationValue() const {
    double e = 0;
    for (size_t i = 0; i < energy_.size(); ++i) e += energy_[i] * prob_[i];
    return e;
}

void PolyenergeticSpectrum::describe(midsx_source_spec& s) const {
    s.spectrum_kind = MIDSX_SPEC_POLY;
    s.n_bins = int32_t(energy_.size());
    s.bin_energy = energy_.data();
    s.bin_prob = prob_.data();
}

Vec3 IsotropicDirectionality::sampleDirection(const Vec3&) {
    double theta = PI * uni();
    double phi = 2 * PI * uni();
    return SourceHelpers::angleToUnitDirection(theta, phi);
}
void IsotropicDirectionality::describe(midsx_source_spec& s) const { s.direction_kind = MIDSX_DIR_ISOTROPIC; }

Vec3 BeamDirectionality::sampleDirection(const Vec3& p) { return (pass_through_point_ - p).normalized(); }
void BeamDirectionality::describe(midsx_source_spec& s) const {
    s.direction_kind = MIDSX_DIR_BEAM;
    put(s.a, pass_through_point_);
}

RectangularIsotropicDirectionality::RectangularIsotropicDirectionality(Vec3 corner, Vec3 edge1, Vec3 edge2)
    : corner_(corner), edge1_(edge1), edge2_(edge2) {
    if (!(std::abs(edge1_.dot(edge2_)) < 1e-9)) throw std::invalid_argument("Edges are not orthogonal");
}
Vec3 RectangularIsotropicDirectionality::sampleDirection(const Vec3& p) {
    double a1 = uni(), a2 = uni();
    return (corner_ + a1 * edge1_ + a2 * edge2_ - p).normalized();
}
void RectangularIsotropicDirectionality::describe(midsx_source_spec& s) const {
    s.direction_kind = MIDSX_DIR_RECTANGLE;
    put(s.a, corner_);
    put(s.b, edge1_);
    put(s.c, edge2_);
}

DiscIsotropicDirectionality::DiscIsotropicDirectionality(Vec3 center, Vec3 normal, double radius)
    : center_(center), normal_(normal), radius_(radius) {
    if (std::abs(normal_.dot(Vec3(1, 0, 0))) < 1e-9)
        u_ = normal_.cross(Vec3(0, 1, 0)).normalized();
    else
        u_ = normal_.cross(Vec3(1, 0, 0)).normalized();
    v_ = normal_.cross(u_).normalized();
}
Vec3 DiscIsotropicDirectionality::sampleDirection(const Vec3& p) {
    double theta = 2 * PI * uni();
    double r = radius_ * uni();
    return (center_ + r * (u_ * std::cos(theta) + v_ * std::sin(theta)) - p).normalized();
}
void DiscIsotropicDirectionality::describe(midsx_source_spec& s) const {
    s.direction_kind = MIDSX_DIR_DISC;
    put(s.a, center_);
    put(s.b, normal_);
    s.radius = radius_;
}

void PointGeometry::describe(midsx_source_spec& s) const { put(s.position, position_); }

PhotonSource::PhotonSource(std::unique_ptr<EnergySpectrum> e, std::unique_ptr<Directionality> d,
                           std::unique_ptr<SourceGeometry> g)
    : energy_spectrum_(std::move(e)), directionality_(std::move(d)), source_geometry_(std::move(g)) {}

Photon PhotonSource::generatePhoton() {
    Vec3 p = source_geometry_->samplePosition();
    Vec3 d = directionality_->sampleDirection(p);
    double e = energy_spectrum_->sampleEnergy();
    return Photon(p, d, e);
}

midsx_source_spec PhotonSource::describe() const {
    if (!energy_spectrum_ || !directionality_ || !source_geometry_)
        throw std::invalid_argument("PhotonSource is incomplete");
    midsx_source_spec s;
    std::memset(&s, 0, sizeof(s));
    source_geometry_->describe(s);
    directionality_->describe(s);
    energy_spectrum_->describe(s);
    return s;
}
