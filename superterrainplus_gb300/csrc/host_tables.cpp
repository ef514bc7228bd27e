// Host-side tables and setting validation: permutation/gradient table,
// erosion brush, lifetime helper, error strings.
#include "internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace stpgb {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) {
	g_last_error = msg;
}

void clear_error() {
	g_last_error.clear();
}

const char* last_error_cstr() {
	return g_last_error.c_str();
}

} // namespace stpgb

using namespace stpgb;

namespace {

constexpr double kTwoPi = 2.0 * 3.14159265358979323846264338327950288;

bool in_range(float v, float lo, float hi) {
	return v >= lo && v <= hi;
}

} // namespace

extern "C" {

const char* stpgb_last_error(void) {
	return last_error_cstr();
}

const char* stpgb_version(void) {
	return "stpgb 0.1.0 (sm_103a)";
}

// STPAlgorithmEnvironment.cpp:13-17
int stpgb_simplex_setting_validate(const stpgb_simplex_setting* s) {
	if (!s) {
		return inval("STPSimplexNoiseSetting: null setting");
	}
	if (s->Distribution == 0u) {
		return inval("STPSimplexNoiseSetting: Distribution != 0 failed");
	}
	if (!(s->Offset >= 0.0)) {
		return inval("STPSimplexNoiseSetting: Offset >= 0 failed");
	}
	if (!(s->Offset < kTwoPi)) {
		return inval("STPSimplexNoiseSetting: Offset < 2*pi failed");
	}
	return STPGB_OK;
}

// STPEnvironment.cpp:48-66
int stpgb_raindrop_setting_validate(const stpgb_raindrop_setting* s) {
	if (!s) {
		return inval("STPRainDropSetting: null setting");
	}
	struct Check {
		bool ok;
		const char* what;
	};
	const Check checks[] = {
		{ s->RainDropCount > 0u, "RainDropCount > 0" },
		{ in_range(s->Inertia, 0.0f, 1.0f), "Inertia in [0,1]" },
		{ s->SedimentCapacityFactor > 0.0f, "SedimentCapacityFactor > 0" },
		{ s->minSedimentCapacity >= 0.0f, "minSedimentCapacity >= 0" },
		{ s->initWaterVolume > 0.0f, "initWaterVolume > 0" },
		{ s->minWaterVolume >= 0.0f, "minWaterVolume >= 0" },
		{ in_range(s->Friction, 0.0f, 1.0f), "Friction in [0,1]" },
		{ s->initSpeed >= 0.0f, "initSpeed >= 0" },
		{ in_range(s->ErodeSpeed, 0.0f, 1.0f), "ErodeSpeed in [0,1]" },
		{ in_range(s->DepositSpeed, 0.0f, 1.0f), "DepositSpeed in [0,1]" },
		{ in_range(s->EvaporateSpeed, 0.0f, 1.0f), "EvaporateSpeed in [0,1]" },
		{ s->Gravity > 0.0f, "Gravity > 0" },
		{ s->ErosionBrushRadius != 0u, "ErosionBrushRadius != 0" },
	};
	for (const Check& c : checks) {
		if (!c.ok) {
			return inval(std::string("STPRainDropSetting: ") + c.what + " failed");
		}
	}
	return STPGB_OK;
}

// STPPermutationGenerator.cpp:40-73.  The shuffle must be libstdc++'s
// std::shuffle driven by std::mt19937_64 for the table to match; the
// gradient angle is accumulated by repeated double addition as there.
int stpgb_permutation_generate(const stpgb_simplex_setting* setting, uint8_t* perm512, float* grad,
	uint32_t grad_capacity) {
	STPGB_TRY(stpgb_simplex_setting_validate(setting));
	if (!perm512 || !grad) {
		return inval("stpgb_permutation_generate: null output");
	}
	const uint32_t n = setting->Distribution;
	if (grad_capacity < 2u * n) {
		set_error("stpgb_permutation_generate: gradient capacity below 2*Distribution");
		return STPGB_ECAPACITY;
	}
	std::mt19937_64 rng(setting->Seed);
	for (uint32_t i = 0u; i < 256u; i++) {
		perm512[i] = static_cast<uint8_t>(i);
	}
	std::shuffle(perm512, perm512 + 256, rng);
	std::memcpy(perm512 + 256, perm512, 256);

	const double step = kTwoPi / (n * 1.0);
	uint32_t counter = 0u;
	for (double angle = 0.0; angle < kTwoPi; angle += step, counter++) {
		if (counter >= n) {
			// the reference writes this extra entry past its table; it is dropped here
			continue;
		}
		const double a = angle + setting->Offset;
		grad[counter * 2u] = static_cast<float>(std::cos(a));
		grad[counter * 2u + 1u] = static_cast<float>(std::sin(a));
	}
	return STPGB_OK;
}

// STPHeightfieldGenerator.cpp:44-77
int stpgb_erosion_brush_generate(uint32_t dimension_x, uint32_t radius, int32_t* index, float* weight,
	uint32_t capacity, uint32_t* size) {
	if (radius == 0u) {
		return inval("Erosion brush radius must be a positive integer");
	}
	if (dimension_x == 0u) {
		return inval("Dimension row count should be positive");
	}
	const int r = static_cast<int>(radius), r2 = r * r;
	double sum = 0.0;
	std::vector<int32_t> idx;
	std::vector<float> w;
	for (int by = -r; by <= r; by++) {
		for (int bx = -r; bx <= r; bx++) {
			const double d2 = static_cast<double>(bx * bx + by * by);
			if (d2 < r2) {
				const double cw = 1.0 - std::sqrt(d2) / r;
				sum += cw;
				idx.push_back(by * static_cast<int>(dimension_x) + bx);
				w.push_back(static_cast<float>(cw));
			}
		}
	}
	const double f = 1.0 / sum;
	if (size) {
		*size = static_cast<uint32_t>(idx.size());
	}
	if (capacity < idx.size() || !index || !weight) {
		set_error("stpgb_erosion_brush_generate: capacity below brush size");
		return STPGB_ECAPACITY;
	}
	for (size_t k = 0u; k < idx.size(); k++) {
		index[k] = idx[k];
		weight[k] = static_cast<float>(w[k] * f);
	}
	return STPGB_OK;
}

float stpgb_lifetime_min_water_volume(float init_water_volume, float evaporate_speed, uint32_t lifetime) {
	float v = init_water_volume;
	for (uint32_t i = 0u; i < lifetime; i++) {
		v *= 1.0f - evaporate_speed;
	}
	return std::nextafter(v, INFINITY);
}

} // extern "C"
