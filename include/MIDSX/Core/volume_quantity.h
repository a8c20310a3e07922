// volume_quantity.h - quantities of a volume tally (reference: include/MIDSX/Core/
// volume_quantity.h).  Values are split by scatter class as in
// src/MIDSX/Core/volume_quantity.cpp:53-67: primary, single coherent, single incoherent,
// multiple.  On the GPU path they are filled from device sums by PhysicsEngine.
#pragma once
#include <string>

#include "quantity.h"

enum class VectorVolumeQuantityType { EnergyDeposition, IncidentEnergy };
enum class CountVolumeQuantityType { NumberOfPhotons, NumberOfInteractions };

namespace VectorVolumeQuantityHelper {
std::string toString(VectorVolumeQuantityType type);
}
namespace CountVolumeQuantityHelper {
std::string toString(CountVolumeQuantityType type);
}

class VectorVolumeQuantity {
public:
    explicit VectorVolumeQuantity(VectorVolumeQuantityType type) : type_(type) {}
    VectorVolumeQuantity operator+(VectorVolumeQuantity& other) const;
    VectorVolumeQuantityType getType() const { return type_; }
    VectorValue& getTotalValues();
    VectorValue& getPrimaryValues() { return cls_[0]; }
    VectorValue& getSingleCoherentScatterValues() { return cls_[1]; }
    VectorValue& getSingleIncoherentScatterValues() { return cls_[2]; }
    VectorValue& getMultipleScatterValues() { return cls_[3]; }
    // class index 0 primary, 1 single coherent, 2 single incoherent, 3 multiple
    VectorValue& getClassValues(int cls) { return cls_[cls]; }

private:
    VectorVolumeQuantityType type_;
    VectorValue cls_[4];
    VectorValue total_;
};

class CountVolumeQuantity {
public:
    explicit CountVolumeQuantity(CountVolumeQuantityType type) : type_(type) {}
    CountVolumeQuantity operator+(const CountVolumeQuantity& other) const;
    CountVolumeQuantityType getType() const { return type_; }
    CountValue getTotalValues() const;
    CountValue getPrimaryValues() const { return cls_[0]; }
    CountValue getSingleCoherentScatterValues() const { return cls_[1]; }
    CountValue getSingleIncoherentScatterValues() const { return cls_[2]; }
    CountValue getMultipleScatterValues() const { return cls_[3]; }
    CountValue& getClassValues(int cls) { return cls_[cls]; }

private:
    CountVolumeQuantityType type_;
    CountValue cls_[4];
};
