// hvl.cpp - half-value-layer scene through the MIDSX C++ API, in the form of the reference's
// cpp_simulations/half_value_layer/hvl_30keV.cpp: a 4 x 4 x 100 cm air domain, an aluminium
// slab at z = 10 cm, a disc source beam from (2, 2, 0) through a 1 mm disc at z = 10 cm and a
// disc surface tally of radius 1 cm at z = 100 cm.  Prints the primary photon count on the
// tally disc, the primary incident-energy sum, the primary air kerma of the reference program
// (DerivedQuantity::getPrimarySpectrumAirKerma over the 0.5 keV midpoints 0.25 ... 119.25 keV
// of the reference's spectrum files) and the run time.
//
//   hvl <scene.json | -> <energy_eV | spectrum.csv> <n_photons> [slab_voxels slab_voxel_cm]
//
// A CSV argument (rows "keV, weight", the format of data/source_distributions) makes the
// source polyenergetic, as in hvl_30kVp.cpp.
// With "-" the domain is built in memory (slab_voxels x 4 cm x 4 cm x slab_voxel_cm of Al);
// otherwise it is read from a scene JSON naming a NIfTI voxel grid.
#include <MIDSX/Core.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

std::vector<std::unique_ptr<SurfaceTally>> initializeSurfaceTallies() {
    std::vector<std::unique_ptr<SurfaceTally>> tallies;
    tallies.emplace_back(std::make_unique<DiscSurfaceTally>(Eigen::Vector3d(2, 2, 100), Eigen::Vector3d(0, 0, 1), 1.0,
                                                            SurfaceQuantityContainerFactory::AllQuantities()));
    return tallies;
}

PhotonSource initializeSource(const std::string& energy_arg) {
    std::unique_ptr<EnergySpectrum> spectrum;
    if (energy_arg.size() > 4 && energy_arg.substr(energy_arg.size() - 4) == ".csv") {
        std::vector<std::vector<double>> rows = SourceHelpers::readCSV(energy_arg);
        for (auto& r : rows) r.at(0) *= 1000;  // keV to eV
        spectrum = std::make_unique<PolyenergeticSpectrum>(rows);
    } else {
        spectrum = std::make_unique<MonoenergeticSpectrum>(std::atof(energy_arg.c_str()));
    }
    std::unique_ptr<Directionality> directionality = std::make_unique<DiscIsotropicDirectionality>(
        Eigen::Vector3d(2, 2, 10), Eigen::Vector3d(0, 0, 1), 0.1);
    std::unique_ptr<SourceGeometry> geometry = std::make_unique<PointGeometry>(Eigen::Vector3d(2, 2, 0));
    return PhotonSource(std::move(spectrum), std::move(directionality), std::move(geometry));
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <scene.json | -> <energy_eV> <n_photons> [slab_voxels slab_voxel_cm]\n", argv[0]);
        return 2;
    }
    const std::string scene = argv[1];
    const std::string energy = argv[2];
    const int n = std::atoi(argv[3]);
    try {
        std::unique_ptr<ComputationalDomain> comp_domain;
        if (scene == "-") {
            int nz = argc > 4 ? std::atoi(argv[4]) : 1;
            double dz = argc > 5 ? std::atof(argv[5]) : 1e-4;
            uint8_t id = argc > 4 ? 61 : 3;  // Al slab, or only air
            std::vector<std::pair<VoxelGrid, Vec3>> grids;
            grids.emplace_back(VoxelGrid({{1, 1, nz}}, Vec3(4, 4, dz), std::vector<uint8_t>(size_t(nz), id)),
                               Vec3(0, 0, 10));
            comp_domain = std::make_unique<ComputationalDomain>(Vec3(4, 4, 100), "Air, Dry (near sea level)",
                                                                std::move(grids));
        } else {
            comp_domain = std::make_unique<ComputationalDomain>(scene);
        }
        InteractionData interaction_data = comp_domain->getInteractionData();
        PhysicsEngine physics_engine(*comp_domain, interaction_data);
        PhotonSource source = initializeSource(energy);
        double run_time = 0;
        runSimulation(source, physics_engine, initializeSurfaceTallies,
                      []() { return std::vector<std::unique_ptr<VolumeTally>>(); }, n, run_time);
        auto results = physics_engine.getSurfaceQuantityContainers();
        auto& counts = results.at(0).getCountQuantities();
        auto& vectors = results.at(0).getVectorQuantities();
        std::cout.precision(17);
        std::cout << "primary_photons " << counts.at(CountSurfaceQuantityType::NumberOfPhotons).getPrimaryValues().getCount()
                  << "\n";
        std::cout << "primary_energy " << vectors.at(VectorSurfaceQuantityType::IncidentEnergy).getPrimaryValues().getSum()
                  << "\n";
        std::cout << "total_photons " << counts.at(CountSurfaceQuantityType::NumberOfPhotons).getTotalValues().getCount()
                  << "\n";
        std::cout << "area " << results.at(0).getArea() << "\n";
        // displayResults of hvl_*.cpp: the spectrum air kerma over the spectrum files' midpoints
        Eigen::VectorXd energy_bin;
        for (int k = 0; k < 239; ++k) energy_bin.push_back((0.25 + 0.5 * k) * 1000);
        std::cout << "primary_air_kerma "
                  << DerivedQuantity::getPrimarySpectrumAirKerma(results.at(0), interaction_data, energy_bin, false)
                  << "\n";
        std::cout << "primary_fluence_cosine "
                  << DerivedQuantity::getPrimaryFluence(results.at(0), energy_bin[0] + 0.5 * (energy_bin.back() - energy_bin[0]),
                                                        energy_bin.back() - energy_bin[0] + 500, true)
                  << "\n";
        std::cout << "run_time " << run_time << "\n";
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
