// Stand-in for glm/gtc/type_ptr.hpp: the vector types only.
#pragma once
#include <glm/vec2.hpp>
#include <glm/vec3.hpp>
