// photon.h - reference: include/MIDSX/Core/photon.h (Photon is declared with PhotonSource).
#pragma once
#include "source.h"
