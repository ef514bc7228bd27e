// Compatibility header: the reference's STPChunk static coordinate functions
// from the C++ façade, with glm result types (glm is included first).
#pragma once
#include <glm/vec2.hpp>
#include <glm/vec3.hpp>

#include "stpgb.hpp"
