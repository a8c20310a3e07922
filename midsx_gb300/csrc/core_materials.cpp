// core_materials.cpp - InteractionData, Material, MaterialData and MaterialProperties of the
// MIDSX C++ API on top of the host table builder of the C ABI.
// Reference: src/MIDSX/Core/interaction_data.cpp, material.cpp, material_data.cpp,
// material_properties.cpp, include/MIDSX/Core/material_helpers.h:110-121.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <random>
#include <stdexcept>
#include <string>

#include "MIDSX/Core/interaction_data.h"

namespace midsx {

class BlobHolder {
public:
    explicit BlobHolder(midsx_table_blob* b) : blob(b) {}
    ~BlobHolder() { midsx_tables_free(blob); }
    midsx_table_blob* blob;
};

std::string data_dir() {
    if (const char* env = std::getenv("MIDSX_DATA_DIR")) return env;
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&data_dir), &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        size_t k = p.find_last_of('/');
        std::string lib = k == std::string::npos ? "." : p.substr(0, k);
        return lib + "/../data";
    }
    return "midsx_gb300/data";
}

namespace {
void check(midsx_status s, const char* what) {
    if (s == MIDSX_OK) return;
    std::string msg = std::string(what) + ": " + midsx_status_string(s) + " (" + midsx_last_error() + ")";
    if (s == MIDSX_NOT_FOUND) throw std::out_of_range(msg);
    if (s == MIDSX_INVALID_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

double host_uniform() {
    thread_local std::mt19937_64 gen{std::random_device{}()};
    thread_local std::uniform_real_distribution<double> unit(0.0, 1.0);
    return unit(gen);
}
}  // namespace

}  // namespace midsx

double MaterialData::eval(int which, double x) const {
    double y = 0;
    midsx::check(midsx_tables_eval(blob_->blob, index_, which, &x, &y, 1), "midsx_tables_eval");
    return y;
}

double MaterialData::interpolateMassEnergyAbsorptionCoefficient(double energy) const {
    if (!mu_en_table_.empty()) {
        // LogLogLinear clamped at the table's ends (src/MIDSX/Core/interpolators.cpp:33-76)
        const auto& t = mu_en_table_;
        const double lx = std::log10(energy);
        if (lx <= std::log10(t.front().first)) return t.front().second;
        if (lx >= std::log10(t.back().first)) return t.back().second;
        const size_t j = size_t(std::upper_bound(t.begin(), t.end(), energy,
                                                 [](double v, const std::pair<double, double>& p) {
                                                     return v < p.first;
                                                 }) -
                                t.begin());
        const double x1 = std::log10(t[j - 1].first), x2 = std::log10(t[j].first);
        const double y1 = std::log10(t[j - 1].second), y2 = std::log10(t[j].second);
        return std::pow(10.0, y1 + (y2 - y1) / (x2 - x1) * (lx - x1));
    }
    double y = 0;
    midsx::check(midsx_tables_mu_en(blob_->blob, index_, &energy, &y, 1), "midsx_tables_mu_en");
    return y;
}

void MaterialData::setMassEnergyAbsorptionCoefficients(std::vector<std::pair<double, double>> table) {
    if (table.size() < 2) throw std::invalid_argument("a mu_en/rho table needs at least two nodes");
    for (size_t i = 0; i < table.size(); ++i) {
        if (!(table[i].first > 0) || !(table[i].second > 0) || (i && !(table[i].first > table[i - 1].first)))
            throw std::invalid_argument("mu_en/rho table: positive values at ascending energies");
    }
    mu_en_table_ = std::move(table);
}

double MaterialData::sampleCoherentScatteringDCS(double energy) const {
    double mu = 0;
    midsx::check(midsx_tables_rita(blob_->blob, index_, energy, midsx::host_uniform(), &mu), "midsx_tables_rita");
    return mu;
}

std::vector<std::pair<double, double>> MaterialData::getTableMatrix(int which) const {
    const midsx_material_table& m = blob_->blob->mat[index_];
    const midsx_lin_table* t = which == 0 ? &m.total : which == 1 ? &m.photo : which == 4 ? &m.sfunc : &m.ffactor;
    std::vector<std::pair<double, double>> out(size_t(t->n));
    const double* D = blob_->blob->data;
    for (int i = 0; i < t->n; ++i) out[size_t(i)] = {D[t->x + i], std::pow(10.0, D[t->ly + i])};
    return out;
}

InteractionData::InteractionData(const std::vector<std::string>& material_names, double e_max)
    : material_names_(material_names), e_max_(e_max) {
    if (material_names.empty()) return;  // a catalogue helper, as InteractionData({}) in the reference
    const std::string dir = midsx::data_dir();
    for (auto& name : material_names) {
        int32_t id = 0;
        midsx::check(midsx_catalog_id(dir.c_str(), name.c_str(), &id), "material lookup");
        ids_.push_back(id);
    }
    midsx_table_blob* b = nullptr;
    midsx::check(midsx_tables_build(dir.c_str(), ids_.data(), int32_t(ids_.size()), e_max, &b), "midsx_tables_build");
    blob_ = std::make_shared<midsx::BlobHolder>(b);
    for (size_t i = 0; i < ids_.size(); ++i) {
        Material m;
        MaterialProperties& p = m.properties_;
        p.name_ = material_names[i];
        p.material_id_ = ids_[i];
        int32_t n = 0, z[64];
        double w[64], aw[64];
        midsx::check(midsx_catalog_material(dir.c_str(), ids_[i], &p.mass_density_, &n, z, w, aw, 64),
                     "midsx_catalog_material");
        double nd = 0, awt = 0;
        for (int k = 0; k < n && k < 64; ++k) {
            p.elemental_composition_[z[k]] = w[k];
            p.elemental_atomic_weight_[z[k]] = aw[k];
            double nz = 6.022140857e23 * p.mass_density_ * w[k] / aw[k];  // material_properties.cpp:66-73
            p.elemental_number_density_[z[k]] = nz;
            nd += nz;
            awt += w[k] * aw[k];
        }
        p.number_density_ = nd;
        p.atomic_weight_ = awt;
        m.data_.blob_ = blob_;
        m.data_.index_ = int(i);
        material_map_.emplace(ids_[i], m);
    }
}

const midsx_table_blob* InteractionData::blob() const { return blob_ ? blob_->blob : nullptr; }

double InteractionData::interpolateMaxTotalCrossSection(double energy) const {
    if (!blob_) throw std::logic_error("InteractionData has no materials");
    double y = 0;
    midsx::check(midsx_tables_eval(blob_->blob, 0, 6, &energy, &y, 1), "midsx_tables_eval");
    return y;
}

std::vector<std::pair<double, double>> InteractionData::getMaxTotalCrossSectionsMatrix() const {
    if (!blob_) return {};
    const midsx_lin_table& t = blob_->blob->majorant;
    const double* D = blob_->blob->data;
    std::vector<std::pair<double, double>> out(size_t(t.n));
    for (int i = 0; i < t.n; ++i) out[size_t(i)] = {D[t.x + i], std::pow(10.0, D[t.ly + i])};
    return out;
}

std::string InteractionData::getAnyMaterialNameFromId(int id) {
    char buf[256];
    midsx::check(midsx_catalog_name(midsx::data_dir().c_str(), id, buf, 256), "material lookup");
    return buf;
}

uint8_t InteractionData::getAnyMaterialIdFromName(std::string name) {
    int32_t id = 0;
    midsx::check(midsx_catalog_id(midsx::data_dir().c_str(), name.c_str(), &id), "material lookup");
    return uint8_t(id);
}
