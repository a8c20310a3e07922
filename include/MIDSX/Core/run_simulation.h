// run_simulation.h - reference: include/MIDSX/Core/run_simulation.h (declared with PhysicsEngine).
#pragma once
#include "physics_engine.h"
