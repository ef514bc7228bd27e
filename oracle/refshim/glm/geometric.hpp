#pragma once
#include "detail_vec.hpp"
#include "exponential.hpp"
