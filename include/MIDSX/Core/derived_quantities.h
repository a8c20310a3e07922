// derived_quantities.h - DerivedQuantity of the MIDSX C++ API (reference:
// include/MIDSX/Core/derived_quantities.h, src/MIDSX/Core/derived_quantities.cpp:3-68).
//
// The reference scans a surface tally's raw IncidentEnergy / EntranceCosine vectors for the
// primary photons whose energy lies in [energy - width/2, energy + width/2].  The GPU tallies
// keep no raw vectors; they keep the container's IncidentSpectrum, and a bin counts when its
// centre lies in that window.  A primary photon keeps its source energy, so with bins centred
// on the source's lines (the default that PhysicsEngine chooses) every primary sits at a bin
// centre and the count equals the reference's.
#pragma once
#include <vector>

#include "interaction_data.h"
#include "surface_quantity_container.h"

#include "matrix.h"  // Eigen::VectorXd without Eigen

namespace DerivedQuantity {
// Primary photons (or, cosine-weighted, the sum of their entrance cosines) in the energy
// window per unit area of the tally, 1/cm^2.  Throws std::runtime_error without a spectrum.
double getPrimaryFluence(SurfaceQuantityContainer& surface_quantity_container, double energy, double energy_width,
                         bool is_cosine_weighted = false);

// energy * fluence * mu_en/rho of material id 3 (air) at `energy`, eV/g.
double getPrimaryAirKerma(SurfaceQuantityContainer& surface_quantity_container, InteractionData& interaction_data,
                          double energy, double energy_width, bool is_cosine_weighted = false);

// Sum of getPrimaryAirKerma over evenly spaced bin midpoints, width = spacing of the first two.
double getPrimarySpectrumAirKerma(SurfaceQuantityContainer& surface_quantity_container,
                                  InteractionData& interaction_data, std::vector<double> energy_spectrum,
                                  bool is_cosine_weighted = false);
}  // namespace DerivedQuantity
