// core_quantities.cpp - quantities, containers and tally descriptions of the MIDSX C++ API.
// Reference: src/MIDSX/Core/quantity.cpp, volume_quantity.cpp, surface_quantity.cpp,
// volume_quantity_container.cpp, surface_quantity_container.cpp, volume_tally.cpp:33-36,
// surface_tally.cpp:142-188.
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <unordered_map>

#include "MIDSX/Core/surface_quantity_container.h"
#include "MIDSX/Core/surface_tally.h"
#include "MIDSX/Core/volume_quantity_container.h"
#include "MIDSX/Core/volume_tally.h"

// ------------------------------------------------------------------- VectorValue ---
VectorValue VectorValue::operator+(VectorValue& other) const {
    VectorValue s = *this;
    s.values_.insert(s.values_.end(), other.values_.begin(), other.values_.end());
    s.n_ += other.n_;
    s.sum_ += other.sum_;
    s.sumsq_ += other.sumsq_;
    s.summary_only_ = summary_only_ || other.summary_only_;
    return s;
}

void VectorValue::addValue(double value) {
    values_.push_back(value);
    n_ += 1;
    sum_ += value;
    sumsq_ += value * value;
}

void VectorValue::addValues(const std::vector<double>& values) {
    for (double v : values) addValue(v);
}

void VectorValue::addSummary(double count, double sum, double sum_of_squares) {
    n_ += count;
    sum_ += sum;
    sumsq_ += sum_of_squares;
    if (count > 0) summary_only_ = true;
}

std::vector<double>& VectorValue::getVector() {
    if (summary_only_)
        throw std::logic_error("VectorValue filled by the GPU path holds count/sum/sum of squares only");
    return values_;
}

double VectorValue::getSum() { return sum_; }
double VectorValue::getCount() { return n_; }
double VectorValue::getCountSTD() { return std::sqrt(n_); }
double VectorValue::getMean() { return sum_ / n_; }

double VectorValue::getVariance() {
    // sample variance, (n - 1) denominator (quantity.cpp:77-94)
    double mean = sum_ / n_;
    double var = (sumsq_ - n_ * mean * mean) / (n_ - 1);
    return var < 0 ? 0.0 : var;
}

double VectorValue::getSumSTD() { return std::sqrt(n_ * getVariance()); }
double VectorValue::getMeanSTD() { return std::sqrt(getVariance() / n_); }

CountValue CountValue::operator+(const CountValue& other) const {
    CountValue s;
    s.count_ = count_ + other.count_;
    return s;
}
void CountValue::addCount() { ++count_; }
void CountValue::addCounts(long long count) { count_ += count; }
long long CountValue::getCount() const { return count_; }
double CountValue::getCountSTD() const { return std::sqrt(double(count_)); }

// -------------------------------------------------------------------- quantities ---
std::string VectorVolumeQuantityHelper::toString(VectorVolumeQuantityType t) {
    return t == VectorVolumeQuantityType::EnergyDeposition ? "EnergyDeposition" : "IncidentEnergy";
}
std::string CountVolumeQuantityHelper::toString(CountVolumeQuantityType t) {
    return t == CountVolumeQuantityType::NumberOfPhotons ? "NumberOfPhotons" : "NumberOfInteractions";
}
std::string VectorSurfaceQuantityHelper::toString(VectorSurfaceQuantityType t) {
    return t == VectorSurfaceQuantityType::IncidentEnergy ? "IncidentEnergy" : "EntranceCosine";
}
std::string CountSurfaceQuantityHelper::toString(CountSurfaceQuantityType) { return "NumberOfPhotons"; }

VectorVolumeQuantity VectorVolumeQuantity::operator+(VectorVolumeQuantity& o) const {
    if (type_ != o.type_) throw std::runtime_error("Cannot add VectorVolumeQuantity objects of different types");
    VectorVolumeQuantity r(type_);
    for (int c = 0; c < 4; ++c) r.cls_[c] = cls_[c] + o.cls_[c];
    return r;
}

VectorValue& VectorVolumeQuantity::getTotalValues() {
    total_ = VectorValue();
    for (int c = 0; c < 4; ++c) total_ = total_ + cls_[c];
    return total_;
}

CountVolumeQuantity CountVolumeQuantity::operator+(const CountVolumeQuantity& o) const {
    if (type_ != o.type_) throw std::runtime_error("Cannot add CountVolumeQuantity objects of different types");
    CountVolumeQuantity r(type_);
    for (int c = 0; c < 4; ++c) r.cls_[c] = cls_[c] + o.cls_[c];
    return r;
}

CountValue CountVolumeQuantity::getTotalValues() const {
    CountValue t;
    for (int c = 0; c < 4; ++c) t.addCounts(cls_[c].getCount());
    return t;
}

VectorSurfaceQuantity VectorSurfaceQuantity::operator+(VectorSurfaceQuantity& o) const {
    if (type_ != o.type_) throw std::runtime_error("Cannot add VectorSurfaceQuantity objects of different types");
    VectorSurfaceQuantity r(type_);
    for (int c = 0; c < 4; ++c) r.cls_[c] = cls_[c] + o.cls_[c];
    return r;
}

VectorValue& VectorSurfaceQuantity::getTotalValues() {
    total_ = VectorValue();
    for (int c = 0; c < 4; ++c) total_ = total_ + cls_[c];
    return total_;
}

CountSurfaceQuantity CountSurfaceQuantity::operator+(const CountSurfaceQuantity& o) const {
    if (type_ != o.type_) throw std::runtime_error("Cannot add CountSurfaceQuantity objects of different types");
    CountSurfaceQuantity r(type_);
    for (int c = 0; c < 4; ++c) r.cls_[c] = cls_[c] + o.cls_[c];
    return r;
}

CountValue CountSurfaceQuantity::getTotalValues() const {
    CountValue t;
    for (int c = 0; c < 4; ++c) t.addCounts(cls_[c].getCount());
    return t;
}

// -------------------------------------------------------------------- containers ---
void VolumeQuantityContainer::addVectorQuantity(const VectorVolumeQuantity& q) { vector_.emplace(q.getType(), q); }
void VolumeQuantityContainer::addCountQuantity(const CountVolumeQuantity& q) { count_.emplace(q.getType(), q); }
void VolumeQuantityContainer::clear() {
    vector_.clear();
    count_.clear();
}

VolumeQuantityContainer VolumeQuantityContainer::operator+(VolumeQuantityContainer& o) const {
    if (vector_.empty() && count_.empty()) return o;
    if (o.vector_.empty() && o.count_.empty()) return *this;
    for (auto& v : vector_)
        if (!o.vector_.count(v.first))
            throw std::runtime_error("Cannot add VolumeQuantityContainers with different vector quantities.");
    for (auto& c : count_)
        if (!o.count_.count(c.first))
            throw std::runtime_error("Cannot add VolumeQuantityContainers with different count quantities.");
    if (volume_ != o.volume_) throw std::runtime_error("Cannot add VolumeQuantityContainers with different volumes.");
    VolumeQuantityContainer r;
    r.setVolume(volume_);
    for (auto& v : vector_) {
        VectorVolumeQuantity a = v.second;
        r.addVectorQuantity(a + o.vector_.at(v.first));
    }
    for (auto& c : count_) r.addCountQuantity(c.second + o.count_.at(c.first));
    return r;
}

void SurfaceQuantityContainer::addVectorQuantity(const VectorSurfaceQuantity& q) { vector_.emplace(q.getType(), q); }
void SurfaceQuantityContainer::addCountQuantity(const CountSurfaceQuantity& q) { count_.emplace(q.getType(), q); }
void SurfaceQuantityContainer::clear() {
    vector_.clear();
    count_.clear();
}

SurfaceQuantityContainer SurfaceQuantityContainer::operator+(SurfaceQuantityContainer& o) const {
    if (vector_.empty() && count_.empty()) return o;
    if (o.vector_.empty() && o.count_.empty()) return *this;
    for (auto& v : vector_)
        if (!o.vector_.count(v.first))
            throw std::runtime_error("Cannot add SurfaceQuantityContainers with different vector quantities.");
    for (auto& c : count_)
        if (!o.count_.count(c.first))
            throw std::runtime_error("Cannot add SurfaceQuantityContainers with different count quantities.");
    if (area_ != o.area_) throw std::runtime_error("Cannot add SurfaceQuantityContainers with different areas.");
    SurfaceQuantityContainer r;
    r.setArea(area_);
    for (auto& v : vector_) {
        VectorSurfaceQuantity a = v.second;
        r.addVectorQuantity(a + o.vector_.at(v.first));
    }
    for (auto& c : count_) r.addCountQuantity(c.second + o.count_.at(c.first));
    if (spectrum_.empty()) {
        r.spectrum_ = o.spectrum_;
    } else if (o.spectrum_.empty()) {
        r.spectrum_ = spectrum_;
    } else {
        if (spectrum_.n != o.spectrum_.n || spectrum_.e_min != o.spectrum_.e_min ||
            spectrum_.e_width != o.spectrum_.e_width)
            throw std::runtime_error("Cannot add SurfaceQuantityContainers with different energy spectra.");
        r.spectrum_ = spectrum_;
        for (size_t i = 0; i < r.spectrum_.count.size(); ++i) {
            r.spectrum_.count[i] += o.spectrum_.count[i];
            r.spectrum_.cosine[i] += o.spectrum_.cosine[i];
        }
    }
    return r;
}

VolumeQuantityContainer VolumeQuantityContainerFactory::AllQuantities() {
    VolumeQuantityContainer c;
    c.addVectorQuantity(VectorVolumeQuantity(VectorVolumeQuantityType::EnergyDeposition));
    c.addVectorQuantity(VectorVolumeQuantity(VectorVolumeQuantityType::IncidentEnergy));
    c.addCountQuantity(CountVolumeQuantity(CountVolumeQuantityType::NumberOfPhotons));
    c.addCountQuantity(CountVolumeQuantity(CountVolumeQuantityType::NumberOfInteractions));
    return c;
}

VolumeQuantityContainer VolumeQuantityContainerFactory::EnergyDeposition() {
    VolumeQuantityContainer c;
    c.addVectorQuantity(VectorVolumeQuantity(VectorVolumeQuantityType::EnergyDeposition));
    return c;
}

SurfaceQuantityContainer SurfaceQuantityContainerFactory::AllQuantities() {
    SurfaceQuantityContainer c;
    c.addVectorQuantity(VectorSurfaceQuantity(VectorSurfaceQuantityType::IncidentEnergy));
    c.addVectorQuantity(VectorSurfaceQuantity(VectorSurfaceQuantityType::EntranceCosine));
    c.addCountQuantity(CountSurfaceQuantity(CountSurfaceQuantityType::NumberOfPhotons));
    return c;
}

// ----------------------------------------------------------------------- tallies ---
namespace {
midsx_tally_spec blank_spec() {
    midsx_tally_spec s;
    std::memset(&s, 0, sizeof(s));
    return s;
}
void put(double* d, const Vec3& v) {
    d[0] = v.x();
    d[1] = v.y();
    d[2] = v.z();
}
}  // namespace

midsx_tally_spec VolumeTally::describe() const {
    throw std::invalid_argument("this VolumeTally type has no GPU implementation");
}

AACuboidVolumeTally::AACuboidVolumeTally(Vec3 min_corner, Vec3 max_corner, const VolumeQuantityContainer& quantities)
    : min_corner_(min_corner), max_corner_(max_corner) {
    quantities_ = quantities;
    Vec3 e = max_corner_ - min_corner_;
    quantities_.setVolume(e.x() * e.y() * e.z());
}

midsx_tally_spec AACuboidVolumeTally::describe() const {
    midsx_tally_spec s = blank_spec();
    s.kind = MIDSX_TALLY_VOLUME_AACUBOID;
    put(s.a, min_corner_);
    put(s.b, max_corner_);
    return s;
}

midsx_tally_spec SurfaceTally::describe() const {
    throw std::invalid_argument("this SurfaceTally type has no GPU implementation");
}

void SurfaceTally::setEnergyBins(double e_min, double e_width, int n) {
    if (n < 1 || n > MIDSX_MAX_ENERGY_BINS || !(e_width > 0) || !std::isfinite(e_min) || !std::isfinite(e_width))
        throw std::invalid_argument("energy bins need 1 <= n <= MIDSX_MAX_ENERGY_BINS and e_width > 0");
    e_min_ = e_min;
    e_width_ = e_width;
    n_energy_ = n;
}

void SurfaceTally::describeSpectrum(midsx_tally_spec& s) const {
    s.n_energy = n_energy_;
    s.e_min = e_min_;
    s.e_width = e_width_;
}

DiscSurfaceTally::DiscSurfaceTally(Vec3 center, Vec3 norm, double radius, const SurfaceQuantityContainer& quantities)
    : center_(center), radius_(radius) {
    surface_quantities_ = quantities;
    norm_ = norm;
    surface_quantities_.setArea(M_PI * radius_ * radius_);
}

midsx_tally_spec DiscSurfaceTally::describe() const {
    midsx_tally_spec s = blank_spec();
    s.kind = MIDSX_TALLY_SURFACE_DISC;
    put(s.a, center_);
    put(s.b, norm_);
    s.radius = radius_;
    describeSpectrum(s);
    return s;
}

RectangularSurfaceTally::RectangularSurfaceTally(Vec3 corner, Vec3 edge1, Vec3 edge2,
                                                 const SurfaceQuantityContainer& quantities)
    : corner_(corner), edge1_(edge1), edge2_(edge2) {
    surface_quantities_ = quantities;
    norm_ = edge1_.cross(edge2_).normalized();
    surface_quantities_.setArea(edge1_.cross(edge2_).norm());
    if (!(std::abs(edge1_.dot(edge2_)) < 1e-9)) throw std::invalid_argument("Edges are not orthogonal");
}

midsx_tally_spec RectangularSurfaceTally::describe() const {
    midsx_tally_spec s = blank_spec();
    s.kind = MIDSX_TALLY_SURFACE_RECT;
    put(s.a, corner_);
    put(s.b, edge1_);
    put(s.c, edge2_);
    describeSpectrum(s);
    return s;
}

BinnedRectangularSurfaceTally::BinnedRectangularSurfaceTally(Vec3 corner, Vec3 edge1, Vec3 edge2, int nu, int nv)
    : RectangularSurfaceTally(corner, edge1, edge2, SurfaceQuantityContainer()), nu_(nu), nv_(nv) {
    if (nu < 1 || nv < 1) throw std::invalid_argument("binned surface tally needs nu, nv >= 1");
    energy_.assign(size_t(nu) * nv * 4, 0.0);
    count_.assign(size_t(nu) * nv * 4, 0.0);
}

midsx_tally_spec BinnedRectangularSurfaceTally::describe() const {
    midsx_tally_spec s = RectangularSurfaceTally::describe();
    s.kind = MIDSX_TALLY_SURFACE_BINNED_RECT;
    s.nu = nu_;
    s.nv = nv_;
    if (n_energy_ > 0) throw std::invalid_argument("a binned surface tally keeps no energy spectrum");
    s.n_energy = 0;
    return s;
}
