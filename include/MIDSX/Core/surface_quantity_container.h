// surface_quantity_container.h - reference: include/MIDSX/Core/surface_quantity_container.h.
#pragma once
#include <unordered_map>

#include "surface_quantity.h"

class SurfaceQuantityContainer {
public:
    void addVectorQuantity(const VectorSurfaceQuantity& quantity);
    void addCountQuantity(const CountSurfaceQuantity& quantity);
    SurfaceQuantityContainer operator+(SurfaceQuantityContainer& other) const;
    void clear();
    std::unordered_map<VectorSurfaceQuantityType, VectorSurfaceQuantity>& getVectorQuantities() { return vector_; }
    std::unordered_map<CountSurfaceQuantityType, CountSurfaceQuantity>& getCountQuantities() { return count_; }
    void setArea(double area) { area_ = area; }
    double getArea() const { return area_; }

private:
    std::unordered_map<VectorSurfaceQuantityType, VectorSurfaceQuantity> vector_;
    std::unordered_map<CountSurfaceQuantityType, CountSurfaceQuantity> count_;
    double area_ = 0;
};

namespace SurfaceQuantityContainerFactory {
SurfaceQuantityContainer AllQuantities();
}
