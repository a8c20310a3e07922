// Core.h - umbrella header of the MIDSX C++ API (reference: include/MIDSX/Core.h).
#pragma once
#include <iostream>  // the reference's programs use std::cout through this header

#include "Core/computational_domain.h"
#include "Core/constants.h"
#include "Core/derived_quantities.h"
#include "Core/interaction_data.h"
#include "Core/physics_engine.h"
#include "Core/quantity.h"
#include "Core/run_simulation.h"
#include "Core/source.h"
#include "Core/surface_quantity.h"
#include "Core/surface_quantity_container.h"
#include "Core/surface_tally.h"
#include "Core/vec3.h"
#include "Core/volume_quantity.h"
#include "Core/volume_quantity_container.h"
#include "Core/volume_tally.h"
#include "Core/voxel_grid.h"
