// Stand-in for the CUDA header of this name in the host compilation of
// the reference's device sources (test infrastructure only).
#pragma once
#include "device_prelude.hpp"
