// core_derived.cpp - DerivedQuantity of the MIDSX C++ API over the device's incident-energy
// spectra (reference: src/MIDSX/Core/derived_quantities.cpp:3-68).
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "MIDSX/Core/derived_quantities.h"

namespace {
constexpr int kAirId = 3;  // "Air, Dry (near sea level)", derived_quantities.cpp:50

// Bins whose centre lies in [energy - width/2, energy + width/2] (a relative 1e-12 of slack
// keeps a zero-width window on a centre that rounds by one unit).
template <typename F>
void for_window(const IncidentSpectrum& sp, double energy, double width, F f) {
    const double slack = 1e-12 * std::max(std::fabs(energy), std::fabs(sp.e_width));
    const double lo = energy - width / 2 - slack, hi = energy + width / 2 + slack;
    for (int k = 0; k < sp.n; ++k) {
        const double c = sp.centre(k);
        if (c >= lo && c <= hi) f(k);
    }
}
}  // namespace

double DerivedQuantity::getPrimaryFluence(SurfaceQuantityContainer& surface_quantity_container, double energy,
                                          double energy_width, bool is_cosine_weighted) {
    if (!surface_quantity_container.getVectorQuantities().count(VectorSurfaceQuantityType::IncidentEnergy))
        throw std::runtime_error(
            "SurfaceQuantityContainer does not contain incident energy vector quantity required for fluence calculation");
    if (is_cosine_weighted &&
        !surface_quantity_container.getVectorQuantities().count(VectorSurfaceQuantityType::EntranceCosine))
        throw std::runtime_error(
            "SurfaceQuantityContainer does not contain entrance cosine vector quantity required for cosine-weighted "
            "fluence calculation");
    const IncidentSpectrum& sp = surface_quantity_container.getIncidentSpectrum();
    if (sp.empty()) throw std::runtime_error("SurfaceQuantityContainer holds no incident-energy spectrum");
    double total = 0;
    for_window(sp, energy, energy_width, [&](int k) {
        total += is_cosine_weighted ? sp.cosine[size_t(k) * 4] : sp.count[size_t(k) * 4];
    });
    return total / surface_quantity_container.getArea();
}

double DerivedQuantity::getPrimaryAirKerma(SurfaceQuantityContainer& surface_quantity_container,
                                           InteractionData& interaction_data, double energy, double energy_width,
                                           bool is_cosine_weighted) {
    const MaterialData& air = interaction_data.getMaterialFromId(kAirId).getData();
    const double mu_en = air.interpolateMassEnergyAbsorptionCoefficient(energy);  // cm2/g
    const double fluence = getPrimaryFluence(surface_quantity_container, energy, energy_width, is_cosine_weighted);
    return energy * fluence * mu_en;  // eV/g
}

double DerivedQuantity::getPrimarySpectrumAirKerma(SurfaceQuantityContainer& surface_quantity_container,
                                                   InteractionData& interaction_data, std::vector<double> energy_spectrum,
                                                   bool is_cosine_weighted) {
    if (energy_spectrum.size() < 2) throw std::invalid_argument("an energy spectrum needs at least two midpoints");
    const double width = energy_spectrum[1] - energy_spectrum[0];
    double total = 0;
    for (double e : energy_spectrum)
        total += getPrimaryAirKerma(surface_quantity_container, interaction_data, e, width, is_cosine_weighted);
    return total;
}
