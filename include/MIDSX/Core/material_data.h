// material_data.h - reference: include/MIDSX/Core/material_data.h (declared with InteractionData).
#pragma once
#include "interaction_data.h"
