// material_properties.h - reference: include/MIDSX/Core/material_properties.h (declared with InteractionData).
#pragma once
#include "interaction_data.h"
