// voxel.h - reference: include/MIDSX/Core/voxel.h (Voxel is declared with VoxelGrid).
#pragma once
#include "voxel_grid.h"
