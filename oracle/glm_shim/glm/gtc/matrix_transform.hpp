// Part of the glm stand-in: the camera header includes it; everything it
// needs is in glm/glm.hpp.
#pragma once
#include "../glm.hpp"
