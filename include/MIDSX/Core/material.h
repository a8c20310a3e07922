// material.h - reference: include/MIDSX/Core/material.h (declared with InteractionData).
#pragma once
#include "interaction_data.h"
