// source.h / photon.h - photon source of the MIDSX C++ API (reference: include/MIDSX/Core/
// source.h, photon.h).
//
// The classes keep the reference's constructors and host-side sampling methods
// (src/MIDSX/Core/source.cpp:44-155).  The transport kernel samples the same source on the
// device from describe(); a subclass of EnergySpectrum / Directionality / SourceGeometry that
// the GPU does not implement throws std::invalid_argument from describe().
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../midsx_gpu.h"
#include "matrix.h"
#include "vec3.h"

namespace SourceHelpers {
Vec3 angleToUnitDirection(double theta, double phi);
// Rows of comma-separated numbers (src/MIDSX/Core/source.cpp:11-42), as a matrix that also
// converts to rows of numbers.
midsx::Matrix readCSV(const std::string& file);
}  // namespace SourceHelpers

struct Photon {
    Vec3 position, direction;
    double energy = 0;
    int coherent = 0, incoherent = 0;
    Photon() = default;
    Photon(const Vec3& p, const Vec3& d, double e) : position(p), direction(d), energy(e) {}
    Vec3 getPosition() const { return position; }
    Vec3 getDirection() const { return direction; }
    double getEnergy() const { return energy; }
    int getCoherentScatterCount() const { return coherent; }
    int getIncoherentScatterCount() const { return incoherent; }
    int getTotalScatterCount() const { return coherent + incoherent; }
};

class EnergySpectrum {
public:
    virtual ~EnergySpectrum() = default;
    virtual double sampleEnergy() = 0;
    virtual void describe(midsx_source_spec& spec) const;
};

class MonoenergeticSpectrum : public EnergySpectrum {
public:
    explicit MonoenergeticSpectrum(double energy) : energy_(energy) {}
    double sampleEnergy() override { return energy_; }
    void describe(midsx_source_spec& spec) const override;

private:
    double energy_;
};

class PolyenergeticSpectrum : public EnergySpectrum {
public:
    // rows of (energy eV, probability); probabilities are normalised if they do not sum to 1
    explicit PolyenergeticSpectrum(const std::vector<std::pair<double, double>>& probabilities);
    explicit PolyenergeticSpectrum(const std::vector<std::vector<double>>& probabilities);
    double sampleEnergy() override;
    double getExpectationValue() const;
    void describe(midsx_source_spec& spec) const override;

private:
    std::vector<double> energy_, prob_, cdf_;
    void init();
};

class Directionality {
public:
    virtual ~Directionality() = default;
    virtual Vec3 sampleDirection(const Vec3& photon_initial_position) = 0;
    virtual void describe(midsx_source_spec& spec) const;
};

class IsotropicDirectionality : public Directionality {
public:
    Vec3 sampleDirection(const Vec3& photon_initial_position) override;
    void describe(midsx_source_spec& spec) const override;
};

class BeamDirectionality : public Directionality {
public:
    explicit BeamDirectionality(Vec3 pass_through_point) : pass_through_point_(pass_through_point) {}
    Vec3 sampleDirection(const Vec3& photon_initial_position) override;
    void describe(midsx_source_spec& spec) const override;

private:
    Vec3 pass_through_point_;
};

class RectangularIsotropicDirectionality : public Directionality {
public:
    RectangularIsotropicDirectionality(Vec3 corner, Vec3 edge1, Vec3 edge2);
    Vec3 sampleDirection(const Vec3& photon_initial_position) override;
    void describe(midsx_source_spec& spec) const override;

private:
    Vec3 corner_, edge1_, edge2_;
};

class DiscIsotropicDirectionality : public Directionality {
public:
    DiscIsotropicDirectionality(Vec3 center, Vec3 normal, double radius);
    Vec3 sampleDirection(const Vec3& photon_initial_position) override;
    void describe(midsx_source_spec& spec) const override;

private:
    Vec3 center_, normal_;
    double radius_;
    Vec3 u_, v_;
};

class SourceGeometry {
public:
    virtual ~SourceGeometry() = default;
    virtual Vec3 samplePosition() = 0;
    virtual void describe(midsx_source_spec& spec) const;

protected:
    explicit SourceGeometry(Vec3 position) : position_(position) {}
    Vec3 position_;
};

class PointGeometry : public SourceGeometry {
public:
    explicit PointGeometry(const Vec3& position) : SourceGeometry(position) {}
    Vec3 samplePosition() override { return position_; }
    void describe(midsx_source_spec& spec) const override;
};

class PhotonSource {
public:
    PhotonSource() = default;
    PhotonSource(std::unique_ptr<EnergySpectrum> energy_spectrum, std::unique_ptr<Directionality> directionality,
                 std::unique_ptr<SourceGeometry> source_geometry);
    Photon generatePhoton();
    // The C ABI description of this source.  The spectrum arrays it points to live in the
    // spectrum object.
    midsx_source_spec describe() const;

private:
    std::unique_ptr<EnergySpectrum> energy_spectrum_;
    std::unique_ptr<Directionality> directionality_;
    std::unique_ptr<SourceGeometry> source_geometry_;
};
