// lead_attenuation.cpp - the reference's lead-attenuation simulation
// (cpp_simulations/lead_attenuation/lead_attenuation.cpp) on the C++ API: a scene JSON with
// several voxel grids (two lead blocks and a scintillator in the reference's scene), a point
// source at the middle of the domain's x = 0 face emitting isotropically into the
// rectangle x = 10 (RectangularIsotropicDirectionality), a monoenergetic spectrum, and an
// AACuboid volume tally (energy deposition, photons, interactions) over the scintillator.
// Prints the tally totals and the energy deposited in each grid's voxels.
//
//   lead_attenuation <scene.json> <photons> <seed> <precision 0=FP64|1=mixed> <energy_eV>
//                    <scin_x> <scin_y> <scin_z> <scin_dx> <scin_dy> <scin_dz>
//                    [tracking 0=reference|1=background fast|2=macro cells [cell edge]]
//
// The reference runs 661.7 keV (Cs-137); the mixed form takes energies up to 262 keV, so the
// energy is an argument.  The interaction tables are built up to max(150 keV, energy).
#include <MIDSX/Core.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <iostream>

int main(int argc, char** argv) {
    if (argc < 12) {
        std::fprintf(stderr,
                     "usage: %s <scene.json> <photons> <seed> <precision> <energy_eV> <scin origin x y z> <scin size "
                     "x y z>\n",
                     argv[0]);
        return 2;
    }
    try {
        ComputationalDomain domain(argv[1]);
        const int n_photons = std::atoi(argv[2]);
        const uint64_t seed = std::strtoull(argv[3], nullptr, 10);
        const int precision = std::atoi(argv[4]);
        const double energy = std::atof(argv[5]);
        const Vec3 scin_origin(std::atof(argv[6]), std::atof(argv[7]), std::atof(argv[8]));
        const Vec3 scin_size(std::atof(argv[9]), std::atof(argv[10]), std::atof(argv[11]));
        const Vec3 dim = domain.getDimSpace();

        InteractionData data(domain.getMaterialNames(), std::max(150e3, energy * 1.001));
        PhysicsEngine engine(domain, data);
        engine.setPrecision(precision ? MIDSX_PREC_MIXED : MIDSX_PREC_FP64);
        engine.setSeed(seed);
        if (argc > 12) engine.setTracking(static_cast<midsx_tracking>(std::atoi(argv[12])));
        if (argc > 13) engine.setMacroCellEdge(std::atoi(argv[13]));

        PhotonSource source(std::make_unique<MonoenergeticSpectrum>(energy),
                            std::make_unique<RectangularIsotropicDirectionality>(
                                Vec3(10, 0, 0), Vec3(0, dim.y(), 0), Vec3(0, 0, dim.z())),
                            std::make_unique<PointGeometry>(Vec3(0, dim.y() / 2, dim.z() / 2)));

        auto surface = []() { return std::vector<std::unique_ptr<SurfaceTally>>(); };
        auto volume = [&]() {
            std::vector<std::unique_ptr<VolumeTally>> tallies;
            VolumeQuantityContainer c;
            c.addVectorQuantity(VectorVolumeQuantity(VectorVolumeQuantityType::EnergyDeposition));
            c.addCountQuantity(CountVolumeQuantity(CountVolumeQuantityType::NumberOfPhotons));
            c.addCountQuantity(CountVolumeQuantity(CountVolumeQuantityType::NumberOfInteractions));
            tallies.emplace_back(std::make_unique<AACuboidVolumeTally>(scin_origin, scin_origin + scin_size, c));
            return tallies;
        };
        double run_time = 0;
        runSimulation(source, engine, surface, volume, n_photons, run_time);

        std::cout.precision(17);
        auto containers = engine.getVolumeQuantityContainers();
        for (auto& q : containers[0].getVectorQuantities())
            std::cout << "energy_deposition " << q.second.getTotalValues().getSum() << " "
                      << q.second.getTotalValues().getCount() << "\n";
        for (auto& q : containers[0].getCountQuantities())
            std::cout << "count " << CountVolumeQuantityHelper::toString(q.first) << " "
                      << q.second.getTotalValues().getCount() << "\n";
        for (int k = 0; k < domain.getNumVoxelGrids(); ++k)
            std::cout << "grid_deposit " << k << " " << domain.getVoxelGridN(k).getTotalEnergyDeposited() << "\n";
        std::cout << "run_time " << run_time << "\n";
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
