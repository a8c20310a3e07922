// scene_info.cpp - loads a MIDSX scene JSON (dim_space, background_material_name, NIfTI voxel
// grids) through the C++ API and prints the domain, the grids and a few interaction-table
// values.  Needs no GPU.
//
//   scene_info <scene.json> [energy_eV]
#include <MIDSX/Core.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <scene.json> [energy_eV]\n", argv[0]);
        return 2;
    }
    const double energy = argc > 2 ? std::atof(argv[2]) : 60e3;
    try {
        ComputationalDomain domain(argv[1]);
        std::cout.precision(17);
        Vec3 d = domain.getDimSpace();
        std::cout << "dim_space " << d.x() << " " << d.y() << " " << d.z() << "\n";
        std::cout << "background " << domain.getBackgroundMaterialName() << "\n";
        std::cout << "grids " << domain.getNumVoxelGrids() << "\n";
        for (int i = 0; i < domain.getNumVoxelGrids(); ++i) {
            VoxelGrid& g = domain.getVoxelGridN(i);
            VoxelIndex n = g.getDimVox();
            Vec3 s = g.getSpacing(), o = domain.getVoxelGridOriginN(i);
            std::cout << "grid " << i << " dims " << n[0] << " " << n[1] << " " << n[2] << " spacing " << s.x() << " "
                      << s.y() << " " << s.z() << " origin " << o.x() << " " << o.y() << " " << o.z() << "\n";
            for (int id : g.getMaterialIds()) std::cout << "material " << id << "\n";
        }
        InteractionData data = domain.getInteractionData();
        for (auto& kv : data.getMaterialMap()) {
            const MaterialData& m = kv.second.getData();
            std::cout << "mu " << kv.first << " " << kv.second.getProperties().getName() << " "
                      << m.interpolateTotalCrossSection(energy) << " density " << kv.second.getProperties().getMassDensity()
                      << "\n";
        }
        std::cout << "majorant " << data.interpolateMaxTotalCrossSection(energy) << "\n";
        Voxel& v = domain.getVoxel(domain.getVoxelGridOriginN(0) + Vec3(1e-6, 1e-6, 1e-6));
        std::cout << "first_voxel_material " << int(v.materialID) << "\n";
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
