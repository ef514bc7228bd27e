#pragma once
#include "detail_vec.hpp"
