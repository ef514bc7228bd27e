// Compatibility header: the reference's exception types from the C++ façade.
#pragma once
#include "stpgb.hpp"
