// Chunk coordinate arithmetic of the world pipeline: the static functions of
// STPChunk (SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPChunk.cpp:63-108)
// that map a viewer position to a chunk, a chunk to the map offset its noise
// is generated at, and a chunk index of a neighbourhood to its local
// coordinate and world offset.  A chunk coordinate is in world units: a
// multiple of the chunk size.
//
// The reference computes these in glm with no checks (an integer overflow or
// a zero range is undefined there); here every result is computed in 64-bit
// integers or double and an argument that has no int32 result, a zero size
// or a non-finite position is refused with STPGB_EINVAL.
#include "internal.hpp"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

namespace {

bool fits_i32(const int64_t v) {
	return v >= INT32_MIN && v <= INT32_MAX;
}

// STPChunk::offsetChunk (:87-89): chunkCoord + chunkSize * offset
bool offset_chunk(const int32_t* coord, const uint32_t* size, const int64_t ox, const int64_t oy, int32_t* out) {
	const int64_t x = static_cast<int64_t>(coord[0]) + static_cast<int64_t>(size[0]) * ox;
	const int64_t y = static_cast<int64_t>(coord[1]) + static_cast<int64_t>(size[1]) * oy;
	if (!fits_i32(x) || !fits_i32(y)) {
		return false;
	}
	out[0] = static_cast<int32_t>(x);
	out[1] = static_cast<int32_t>(y);
	return true;
}

bool nonzero(const uint32_t* v) {
	return v && v[0] != 0u && v[1] != 0u;
}

// a rounded product, then a rounded sum: the volatile keeps the compiler from
// fusing them into one multiply-add, whose single rounding would differ
double mul_add_unfused(const double a, const double b, const double c) {
	volatile double p = a * b;
	return p + c;
}

} // namespace

using namespace stpgb;

extern "C" {

int stpgb_chunk_world_coordinate(double point_x, double point_z, const uint32_t* chunk_size, const double* scale,
	int32_t* out) {
	if (!nonzero(chunk_size) || !scale || !out) {
		return inval("stpgb_chunk_world_coordinate: chunk size must be non-zero");
	}
	int32_t unit[2];
	const double p[2] = { point_x, point_z };
	for (int k = 0; k < 2; k++) {
		// floor(position / (chunkSize * scale)), STPChunk.cpp:64-67
		const double scaled = static_cast<double>(chunk_size[k]) * scale[k];
		const double u = std::floor(p[k] / scaled);
		if (!std::isfinite(u) || u < INT32_MIN || u > INT32_MAX) {
			return inval("stpgb_chunk_world_coordinate: the position has no int32 chunk coordinate");
		}
		unit[k] = static_cast<int32_t>(u);
	}
	const int32_t zero[2] = { 0, 0 };
	if (!offset_chunk(zero, chunk_size, unit[0], unit[1], out)) {
		return inval("stpgb_chunk_world_coordinate: the chunk coordinate overflows int32");
	}
	return STPGB_OK;
}

int stpgb_chunk_local_coordinate(uint32_t chunk_id, const uint32_t* chunk_range, uint32_t* out) {
	if (!nonzero(chunk_range) || !out) {
		return inval("stpgb_chunk_local_coordinate: chunk range must be non-zero");
	}
	// STPChunk.cpp:71-73
	out[0] = chunk_id % chunk_range[0];
	out[1] = chunk_id / chunk_range[0];
	return STPGB_OK;
}

int stpgb_chunk_local_origin(const int32_t* centre, const uint32_t* chunk_size, const uint32_t* neighbour_size,
	int32_t* out) {
	if (!centre || !chunk_size || !neighbour_size || !out) {
		return inval("stpgb_chunk_local_origin: null argument");
	}
	// STPChunk.cpp:75-79: move half the neighbourhood (rounded down) towards the origin
	if (!offset_chunk(centre, chunk_size, -static_cast<int64_t>(neighbour_size[0] / 2u),
			-static_cast<int64_t>(neighbour_size[1] / 2u), out)) {
		return inval("stpgb_chunk_local_origin: the chunk coordinate overflows int32");
	}
	return STPGB_OK;
}

int stpgb_chunk_map_offset(const int32_t* chunk_coord, const uint32_t* chunk_size, const uint32_t* map_size,
	const double* map_offset, double* out) {
	if (!chunk_coord || !nonzero(chunk_size) || !map_size || !map_offset || !out) {
		return inval("stpgb_chunk_map_offset: chunk size must be non-zero");
	}
	// STPChunk.cpp:81-85: (chunkCoord / chunkSize) * mapSize + mapOffset in double
	for (int k = 0; k < 2; k++) {
		const double unit = static_cast<double>(chunk_coord[k]) / static_cast<double>(chunk_size[k]);
		out[k] = mul_add_unfused(unit, static_cast<double>(map_size[k]), map_offset[k]);
	}
	return STPGB_OK;
}

int stpgb_chunk_offset(const int32_t* chunk_coord, const uint32_t* chunk_size, const int32_t* offset, int32_t* out) {
	if (!chunk_coord || !chunk_size || !offset || !out) {
		return inval("stpgb_chunk_offset: null argument");
	}
	if (!offset_chunk(chunk_coord, chunk_size, offset[0], offset[1], out)) {
		return inval("stpgb_chunk_offset: the chunk coordinate overflows int32");
	}
	return STPGB_OK;
}

int stpgb_chunk_neighbour_offset(const uint32_t* chunk_size, const uint32_t* region_size, int32_t* offsets_xy,
	uint32_t capacity, uint32_t* count) {
	if (!chunk_size || !nonzero(region_size) || !count) {
		return inval("stpgb_chunk_neighbour_offset: region size must be non-zero");
	}
	const uint64_t n = static_cast<uint64_t>(region_size[0]) * region_size[1];
	if (n > UINT32_MAX) {
		return inval("stpgb_chunk_neighbour_offset: region holds more than 2^32 chunks");
	}
	*count = static_cast<uint32_t>(n);
	if (capacity < n || (!offsets_xy && n > 0u)) {
		set_error("stpgb_chunk_neighbour_offset: output capacity too small");
		return STPGB_ECAPACITY;
	}
	// STPChunk.cpp:91-108: the local origin of a neighbourhood centred on chunk (0, 0), then every
	// chunk index converted to its local coordinate and offset from that origin
	const int32_t zero[2] = { 0, 0 };
	int32_t base[2];
	STPGB_TRY(stpgb_chunk_local_origin(zero, chunk_size, region_size, base));
	for (uint32_t i = 0u; i < n; i++) {
		uint32_t local[2];
		STPGB_TRY(stpgb_chunk_local_coordinate(i, region_size, local));
		if (!offset_chunk(base, chunk_size, local[0], local[1], offsets_xy + 2u * i)) {
			return inval("stpgb_chunk_neighbour_offset: the chunk coordinate overflows int32");
		}
	}
	return STPGB_OK;
}

} // extern "C"

// Host half of STPNearestNeighbourTextureBuffer::STPMergedBuffer
// (SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPNearestNeighbourTextureBuffer.cpp:18-113):
// the chunk maps of a neighbourhood packed into one row-major merged map,
// chunk i at its local chunk coordinate (i % nx, i / nx), and back.
namespace {

int check_nn(const stpgb_nn_info* nn, const uint32_t element_size, const char* what) {
	if (!nn || element_size == 0u) {
		return inval(std::string(what) + ": null neighbour information or zero element size");
	}
	for (int k = 0; k < 2; k++) {
		if (nn->MapSize[k] == 0u || nn->ChunkNearestNeighbour[k] == 0u
			|| static_cast<uint64_t>(nn->MapSize[k]) * nn->ChunkNearestNeighbour[k] != nn->TotalMapSize[k]) {
			return inval(std::string(what) + ": TotalMapSize must equal MapSize * ChunkNearestNeighbour, all positive");
		}
	}
	return STPGB_OK;
}

template<bool Pack>
int copy_neighbours(unsigned char* merged, unsigned char* const* chunks, const uint32_t es, const stpgb_nn_info& nn) {
	const uint32_t count = nn.ChunkNearestNeighbour[0] * nn.ChunkNearestNeighbour[1];
	const size_t row = static_cast<size_t>(nn.MapSize[0]) * es, total_row = static_cast<size_t>(nn.TotalMapSize[0]) * es;
	for (uint32_t i = 0u; i < count; i++) {
		if (!chunks[i]) {
			return inval("stpgb_nn_merge_host / stpgb_nn_unmerge_host: null chunk pointer");
		}
	}
	for (uint32_t i = 0u; i < count; i++) {
		uint32_t local[2];
		STPGB_TRY(stpgb_chunk_local_coordinate(i, nn.ChunkNearestNeighbour, local));
		unsigned char* const corner = merged + static_cast<size_t>(local[1]) * nn.MapSize[1] * total_row
			+ static_cast<size_t>(local[0]) * row;
		for (uint32_t y = 0u; y < nn.MapSize[1]; y++) {
			if (Pack) {
				std::memcpy(corner + y * total_row, chunks[i] + y * row, row);
			} else {
				std::memcpy(chunks[i] + y * row, corner + y * total_row, row);
			}
		}
	}
	return STPGB_OK;
}

} // namespace

extern "C" {

int stpgb_nn_merge_host(const void* const* chunks, uint32_t element_size, const stpgb_nn_info* nn, void* merged) {
	STPGB_TRY(check_nn(nn, element_size, "stpgb_nn_merge_host"));
	if (!chunks || !merged) {
		return inval("stpgb_nn_merge_host: null pointer argument");
	}
	return copy_neighbours<true>(static_cast<unsigned char*>(merged),
		const_cast<unsigned char* const*>(reinterpret_cast<const unsigned char* const*>(chunks)), element_size, *nn);
}

int stpgb_nn_unmerge_host(const void* merged, uint32_t element_size, const stpgb_nn_info* nn, void* const* chunks) {
	STPGB_TRY(check_nn(nn, element_size, "stpgb_nn_unmerge_host"));
	if (!chunks || !merged) {
		return inval("stpgb_nn_unmerge_host: null pointer argument");
	}
	return copy_neighbours<false>(const_cast<unsigned char*>(static_cast<const unsigned char*>(merged)),
		reinterpret_cast<unsigned char* const*>(chunks), element_size, *nn);
}

} // extern "C"
