// interaction_data.h / material.h - interaction tables of the MIDSX C++ API (reference:
// include/MIDSX/Core/interaction_data.h, material.h, material_data.h, material_properties.h).
//
// InteractionData(material names) builds every material's tables and the global majorant
// with the host table builder behind the C ABI (midsx_tables_build), from the data files of
// midsx_gb300/data (EPDL97 element tables, material catalogue).  The data directory is
// $MIDSX_DATA_DIR, else the package directory next to the loaded library.  The tables cover
// photon energies up to e_max (default 150 keV).
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../midsx_gpu.h"

namespace midsx {
std::string data_dir();
class BlobHolder;
}  // namespace midsx

class MaterialProperties {
public:
    std::string getName() const { return name_; }
    int getMaterialId() const { return material_id_; }
    double getMassDensity() const { return mass_density_; }
    double getNumberDensity() const { return number_density_; }
    double getAtomicWeight() const { return atomic_weight_; }
    std::unordered_map<int, double> getElementalComposition() const { return elemental_composition_; }
    std::unordered_map<int, double> getElementalNumberDensity() const { return elemental_number_density_; }
    std::unordered_map<int, double> getElementalAtomicWeight() const { return elemental_atomic_weight_; }

private:
    friend class InteractionData;
    std::string name_;
    int material_id_ = 0;
    double mass_density_ = 0, number_density_ = 0, atomic_weight_ = 0;
    std::unordered_map<int, double> elemental_composition_, elemental_number_density_, elemental_atomic_weight_;
};

class MaterialData {
public:
    double interpolateTotalCrossSection(double energy) const { return eval(0, energy); }
    double interpolatePhotoelectricCrossSection(double energy) const { return eval(1, energy); }
    double interpolateCoherentScatteringCrossSection(double energy) const { return eval(2, energy); }
    double interpolateIncoherentScatteringCrossSection(double energy) const { return eval(3, energy); }
    double interpolateIncoherentScatteringFunction(double x) const { return eval(4, x); }
    double interpolateCoherentFormFactor(double x) const { return eval(5, x); }
    // mu_en/rho, cm2/g (reference: material_data.h:143).  The reference's table comes from
    // NIST via its database; without one it follows from the built tables and the
    // transport's deposition model (midsx_tables_mu_en).  A table set here - (energy eV,
    // mu_en/rho cm2/g) pairs, ascending - is interpolated LogLogLinear, clamped at its ends,
    // as the reference interpolates its own.
    double interpolateMassEnergyAbsorptionCoefficient(double energy) const;
    void setMassEnergyAbsorptionCoefficients(std::vector<std::pair<double, double>> table);
    // Rayleigh cosine by RITA inversion with a host uniform (src/MIDSX/Core/probability_dist.cpp:73-88).
    double sampleCoherentScatteringDCS(double energy) const;
    // (x, y) node table of one interpolator: 0 total, 1 photo, 4 S(x), 5 F(x)
    std::vector<std::pair<double, double>> getTableMatrix(int which) const;
    int denseIndex() const { return index_; }

private:
    friend class InteractionData;
    double eval(int which, double x) const;
    std::shared_ptr<midsx::BlobHolder> blob_;
    int index_ = 0;
    std::vector<std::pair<double, double>> mu_en_table_;
};

class Material {
public:
    const MaterialProperties& getProperties() const { return properties_; }
    const MaterialData& getData() const { return data_; }

private:
    friend class InteractionData;
    MaterialProperties properties_;
    MaterialData data_;
};

class InteractionData {
public:
    explicit InteractionData(const std::vector<std::string>& material_names, double e_max = 150e3);
    Material& getMaterialFromId(int id) { return material_map_.at(id); }
    double interpolateMaxTotalCrossSection(double energy) const;
    std::vector<std::pair<double, double>> getMaxTotalCrossSectionsMatrix() const;
    std::string getAnyMaterialNameFromId(int id);
    uint8_t getAnyMaterialIdFromName(std::string name);
    const std::map<int, Material>& getMaterialMap() const { return material_map_; }
    // Material ids in dense-index order (the order of the device tables).
    const std::vector<int>& getMaterialIds() const { return ids_; }
    const midsx_table_blob* blob() const;
    double getEMax() const { return e_max_; }

private:
    std::vector<std::string> material_names_;
    std::vector<int> ids_;
    std::map<int, Material> material_map_;
    std::shared_ptr<midsx::BlobHolder> blob_;
    double e_max_;
};
