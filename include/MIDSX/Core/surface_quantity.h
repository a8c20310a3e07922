// surface_quantity.h - quantities of a surface tally (reference: include/MIDSX/Core/
// surface_quantity.h), split by the scatter class of the photon crossing the surface
// (src/MIDSX/Core/surface_quantity.cpp:49-63).
#pragma once
#include <string>

#include "quantity.h"

enum class VectorSurfaceQuantityType { IncidentEnergy, EntranceCosine };
enum class CountSurfaceQuantityType { NumberOfPhotons };

namespace VectorSurfaceQuantityHelper {
std::string toString(VectorSurfaceQuantityType type);
}
namespace CountSurfaceQuantityHelper {
std::string toString(CountSurfaceQuantityType type);
}

class VectorSurfaceQuantity {
public:
    explicit VectorSurfaceQuantity(VectorSurfaceQuantityType type) : type_(type) {}
    VectorSurfaceQuantity operator+(VectorSurfaceQuantity& other) const;
    VectorSurfaceQuantityType getType() const { return type_; }
    VectorValue& getTotalValues();
    VectorValue& getPrimaryValues() { return cls_[0]; }
    VectorValue& getSingleCoherentScatterValues() { return cls_[1]; }
    VectorValue& getSingleIncoherentScatterValues() { return cls_[2]; }
    VectorValue& getMultipleScatterValues() { return cls_[3]; }
    VectorValue& getClassValues(int cls) { return cls_[cls]; }

private:
    VectorSurfaceQuantityType type_;
    VectorValue cls_[4];
    VectorValue total_;
};

class CountSurfaceQuantity {
public:
    explicit CountSurfaceQuantity(CountSurfaceQuantityType type) : type_(type) {}
    CountSurfaceQuantity operator+(const CountSurfaceQuantity& other) const;
    CountSurfaceQuantityType getType() const { return type_; }
    CountValue getTotalValues() const;
    CountValue getPrimaryValues() const { return cls_[0]; }
    CountValue getSingleCoherentScatterValues() const { return cls_[1]; }
    CountValue getSingleIncoherentScatterValues() const { return cls_[2]; }
    CountValue getMultipleScatterValues() const { return cls_[3]; }
    CountValue& getClassValues(int cls) { return cls_[cls]; }

private:
    CountSurfaceQuantityType type_;
    CountValue cls_[4];
};
