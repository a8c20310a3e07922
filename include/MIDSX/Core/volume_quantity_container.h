// volume_quantity_container.h - reference: include/MIDSX/Core/volume_quantity_container.h.
#pragma once
#include <unordered_map>

#include "volume_quantity.h"

class VolumeQuantityContainer {
public:
    void addVectorQuantity(const VectorVolumeQuantity& quantity);
    void addCountQuantity(const CountVolumeQuantity& quantity);
    // Sum of two containers of the same tally (src/MIDSX/Core/volume_quantity_container.cpp:20-54).
    VolumeQuantityContainer operator+(VolumeQuantityContainer& other) const;
    void clear();
    std::unordered_map<VectorVolumeQuantityType, VectorVolumeQuantity>& getVectorQuantities() { return vector_; }
    std::unordered_map<CountVolumeQuantityType, CountVolumeQuantity>& getCountQuantities() { return count_; }
    void setVolume(double volume) { volume_ = volume; }
    double getVolume() const { return volume_; }

private:
    std::unordered_map<VectorVolumeQuantityType, VectorVolumeQuantity> vector_;
    std::unordered_map<CountVolumeQuantityType, CountVolumeQuantity> count_;
    double volume_ = 0;
};

namespace VolumeQuantityContainerFactory {
VolumeQuantityContainer AllQuantities();
VolumeQuantityContainer EnergyDeposition();
}  // namespace VolumeQuantityContainerFactory
