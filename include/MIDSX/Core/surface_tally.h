// surface_tally.h - surface tallies (reference: include/MIDSX/Core/surface_tally.h).
//
// DiscSurfaceTally and RectangularSurfaceTally as in the reference (one-directional plane
// crossings, src/MIDSX/Core/surface_tally.cpp:16-112).  BinnedRectangularSurfaceTally is new:
// a rectangle split into nu x nv cells, each equal to a RectangularSurfaceTally over that
// cell, holding per cell and scatter class the incident-energy sum and photon count (a
// pixelated detector, which the reference would need nu * nv rectangle tallies for).
#pragma once
#include <vector>

#include "../../midsx_gpu.h"
#include "surface_quantity_container.h"
#include "vec3.h"

class SurfaceTally {
public:
    virtual ~SurfaceTally() = default;
    SurfaceQuantityContainer& getSurfaceQuantityContainer() { return surface_quantities_; }
    virtual midsx_tally_spec describe() const;
    // Incident-energy spectrum bins of a disc or rectangle (IncidentSpectrum).  Without a
    // call, a tally whose container holds IncidentEnergy gets bins centred on the energies of
    // the source of the engine's first run (one bin per spectrum line), which puts every
    // primary photon at a bin centre.
    void setEnergyBins(double e_min, double e_width, int n);
    bool hasEnergyBins() const { return n_energy_ > 0; }

protected:
    Vec3 norm_;
    SurfaceQuantityContainer surface_quantities_;
    double e_min_ = 0, e_width_ = 0;
    int n_energy_ = 0;
    void describeSpectrum(midsx_tally_spec& s) const;
};

class DiscSurfaceTally : public SurfaceTally {
public:
    DiscSurfaceTally(Vec3 center, Vec3 norm, double radius, const SurfaceQuantityContainer& quantities);
    midsx_tally_spec describe() const override;

private:
    Vec3 center_;
    double radius_;
};

class RectangularSurfaceTally : public SurfaceTally {
public:
    RectangularSurfaceTally(Vec3 corner, Vec3 edge1, Vec3 edge2, const SurfaceQuantityContainer& quantities);
    midsx_tally_spec describe() const override;

protected:
    Vec3 corner_;
    Vec3 edge1_;
    Vec3 edge2_;
};

class BinnedRectangularSurfaceTally : public RectangularSurfaceTally {
public:
    BinnedRectangularSurfaceTally(Vec3 corner, Vec3 edge1, Vec3 edge2, int nu, int nv);
    midsx_tally_spec describe() const override;
    int getNu() const { return nu_; }
    int getNv() const { return nv_; }
    // Incident energy (eV) summed per bin (iu along edge1, iv along edge2) and class
    // (0 primary, 1 single coherent, 2 single incoherent, 3 multiple); photon counts.
    double getEnergy(int iu, int iv, int cls) const { return energy_[(size_t(iv) * nu_ + iu) * 4 + cls]; }
    double getCount(int iu, int iv, int cls) const { return count_[(size_t(iv) * nu_ + iu) * 4 + cls]; }
    std::vector<double>& energies() { return energy_; }
    std::vector<double>& counts() { return count_; }

private:
    int nu_, nv_;
    std::vector<double> energy_, count_;
};
