// surface_quantity_container.h - reference: include/MIDSX/Core/surface_quantity_container.h.
#pragma once
#include <unordered_map>
#include <vector>

#include "surface_quantity.h"

// Incident-energy spectrum of a surface tally's crossings, the device's summary of the raw
// IncidentEnergy / EntranceCosine vectors that DerivedQuantity scans in the reference
// (src/MIDSX/Core/derived_quantities.cpp:3-45): bins [e_min + k e_width, e_min + (k+1) e_width)
// eV, per bin and scatter class the number of crossings and the sum of their entrance cosines.
struct IncidentSpectrum {
    double e_min = 0, e_width = 0;
    int n = 0;
    std::vector<double> count, cosine;  // [bin * 4 + class]
    bool empty() const { return n == 0; }
    double centre(int k) const { return e_min + (k + 0.5) * e_width; }
};

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
    IncidentSpectrum& getIncidentSpectrum() { return spectrum_; }
    const IncidentSpectrum& getIncidentSpectrum() const { return spectrum_; }

private:
    std::unordered_map<VectorSurfaceQuantityType, VectorSurfaceQuantity> vector_;
    std::unordered_map<CountSurfaceQuantityType, CountSurfaceQuantity> count_;
    double area_ = 0;
    IncidentSpectrum spectrum_;
};

namespace SurfaceQuantityContainerFactory {
SurfaceQuantityContainer AllQuantities();
}
