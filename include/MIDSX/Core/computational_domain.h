// computational_domain.h - reference: include/MIDSX/Core/computational_domain.h.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "interaction_data.h"
#include "voxel_grid.h"

class ComputationalDomain {
public:
    ComputationalDomain() = default;
    // Scene JSON (src/MIDSX/Core/computational_domain.cpp:50-107).  NIfTI paths are relative
    // to the JSON file.  The reference's is_python_environment flag is accepted and ignored.
    explicit ComputationalDomain(const std::string& json_file_path, bool is_python_environment = false);
    // In-memory scene.
    ComputationalDomain(const Vec3& dim_space, const std::string& background_material_name,
                        std::vector<std::pair<VoxelGrid, Vec3>> voxel_grids);

    InteractionData getInteractionData() const;
    bool isInComputationalDomain(const Vec3& position) const;
    Voxel& getVoxel(const Vec3& position);
    VoxelGrid& getVoxelGridN(int N) { return voxel_grids_.at(size_t(N)).first; }
    Vec3 getVoxelGridOriginN(int N) { return voxel_grids_.at(size_t(N)).second; }
    Vec3 getVoxelGridDimSpaceN(int N) { return voxel_grids_.at(size_t(N)).first.getDimSpace(); }
    int getNumVoxelGrids() const { return int(voxel_grids_.size()); }
    Vec3 getDimSpace() const { return dim_space_; }
    std::string getBackgroundMaterialName() const;
    std::vector<std::string> getMaterialNames() const;

    Voxel background_voxel;

private:
    std::vector<std::pair<VoxelGrid, Vec3>> voxel_grids_;
    Vec3 dim_space_;
};
