// The reference's own erosion brush generator: the static template
// generateErosionBrush (SuperTerrain+/Private/World/Chunk/STPHeightfieldGenerator.cpp:44-77),
// whose text up to its device upload oracle/build_ref.sh extracts into the
// build folder as brush_generator.inc.  This file supplies what that text
// uses and ends the function by returning the two host vectors (test
// infrastructure only).
#include <algorithm>
#include <cassert>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include <glm/exponential.hpp>

using std::vector;
#define STP_ASSERTION_NUMERIC_DOMAIN(expr, msg) \
	do { \
		if (!(expr)) { \
			throw std::invalid_argument(msg); \
		} \
	} while (0)

namespace {

struct BrushVectors {
	vector<int> Index;
	vector<float> Weight;
};

template<class T>
#include "brush_generator.inc"
	return T { indexCache, weightCache };
}

} // namespace

extern "C" {

// Writes the brush of `radius` for rows of `dim_x` cells; returns its size, 0 for a refused argument.
uint32_t ref_brush(uint32_t dim_x, uint32_t radius, int32_t* index, float* weight) {
	try {
		const BrushVectors b = generateErosionBrush<BrushVectors>(dim_x, radius);
		std::copy(b.Index.begin(), b.Index.end(), index);
		std::copy(b.Weight.begin(), b.Weight.end(), weight);
		return static_cast<uint32_t>(b.Index.size());
	} catch (const std::invalid_argument&) {
		return 0u;
	}
}

} // extern "C"
