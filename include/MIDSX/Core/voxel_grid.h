// voxel.h / voxel_grid.h / computational_domain.h - geometry of the MIDSX C++ API
// (reference: include/MIDSX/Core/voxel.h, voxel_grid.h, computational_domain.h).
//
// A ComputationalDomain is the box [0, dim_space] (cm) filled with a background material and
// holding voxel grids at origins; a VoxelGrid is a uint8 material-id array, x fastest, with a
// voxel size in cm.  Grids load from NIfTI-1 files (.nii; .nii.gz when built with zlib) named
// by the scene JSON {dim_space, background_material_name, voxel_grids: [{file_path, origin}]}
// (src/MIDSX/Core/computational_domain.cpp:50-154, src/MIDSX/Core/voxel_grid.cpp:109-181), or
// are built in memory.  The GPU path transports through the first grid; a domain with more
// than one grid is rejected by PhysicsEngine with std::invalid_argument.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "quantity.h"
#include "vec3.h"

struct Voxel {
    uint8_t materialID = 0;
    VectorValue dose;  // energy deposited (eV): count, sum, sum of squares of the deposits
};

using VoxelIndex = std::array<int, 3>;

class VoxelGrid {
public:
    VoxelGrid() = default;
    explicit VoxelGrid(const std::string& nifti_filename);
    // In-memory grid: ids of dims[0]*dims[1]*dims[2] voxels, x fastest; spacing in cm.
    VoxelGrid(const VoxelIndex& dims, const Vec3& spacing, std::vector<uint8_t> ids);

    Voxel& getVoxel(const VoxelIndex& voxel_index);
    void setVoxel(const VoxelIndex& voxel_index, Voxel& value);
    Vec3 getVoxelPosition(const VoxelIndex& voxel_index) const;
    bool withinGrid(const Vec3& position) const;
    VoxelIndex getVoxelIndex(const Vec3& position) const;  // throws std::out_of_range outside
    std::vector<std::string> getMaterialNames() const;
    std::vector<int> getMaterialIds() const;
    double getTotalEnergyDeposited();
    std::unordered_map<int, VectorValue> getEnergyDepositedInMaterials();
    Vec3 getDimSpace() const { return dim_space_; }
    VoxelIndex getDimVox() const { return dim_vox_; }
    Vec3 getSpacing() const { return spacing_; }
    size_t getNumberOfVoxels() const { return voxels_.size(); }
    std::vector<uint8_t> getMaterialIdArray() const;
    std::vector<Voxel>& voxels() { return voxels_; }

private:
    VoxelIndex dim_vox_{{0, 0, 0}};
    Vec3 spacing_;
    Vec3 dim_space_;
    std::vector<Voxel> voxels_;
    int voxelNumber(const VoxelIndex& voxel_index) const;
};
