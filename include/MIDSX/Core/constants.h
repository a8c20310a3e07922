// constants.h - physical constants of the transport (reference: include/MIDSX/Core/constants.h:13-23).
// cgs units, energies in eV.
#pragma once
#include <cmath>
#include <limits>

const double PI = 3.14159265358979323846;
const double EPSILON = 1e-9;
const double INF = std::numeric_limits<double>::infinity();
const double ELECTRON_REST_MASS = 0.51099895000E6;  // eV
const double ELECTRON_CHARGE = 1.6021766208e-19;    // C
const double ELECTRON_RADIUS = 2.8179403227e-13;    // cm
const double SPEED_OF_LIGHT = 299792458E2;          // cm/s
const double PLANCK_CONSTANT = 4.135667662e-15;     // eV s
const double NUMBER_DENSITY_AT_STP = 0.02504E21;    // 1/cm3
const double AVOGADRO_CONSTANT = 6.022140857e23;    // 1/mol
const double ALPHA = ELECTRON_REST_MASS / (std::sqrt(2.0) * PLANCK_CONSTANT * SPEED_OF_LIGHT * 1E8);  // 1/Angstrom
