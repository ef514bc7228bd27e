// Single histogram filter for callers that cannot allocate device memory.
//
// Some callers of the filter may not call cudaMalloc or cudaFree at all: a
// chunk streamer running inside a renderer's frame loop (cudaFree waits for
// the whole device, and an allocation can stall the frame), or an engine
// whose device memory is carved out of one budget by its own allocator, where
// a driver allocation behind its back breaks the accounting.  They still
// provide the filter's input and outputs, but not its scratch.  This entry
// point takes the scratch from a fixed array in the library's own device
// image instead of a caller workspace:
//
//   * the array holds kNoAllocScratchBytes (16 MiB); every GPU that loads the
//     library keeps it until the process exits;
//   * a call whose scratch would not fit is rejected with STPGB_ECAPACITY
//     (16 MiB covers, for example, a 512 x 512 chunk with radius 32 and
//     max_items up to 13);
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current); make that first call
//     before any stream capture begins;
//   * all calls share the one array and it keeps the last call's contents:
//     the filter writes every scratch entry before it reads it, so nothing
//     needs clearing, but calls whose work overlaps on the GPU (different
//     streams, or different host threads) race on the scratch and must be
//     serialised by the caller.
//
// No memory is allocated: no cudaMalloc, cudaFree or allocating library call.
#include "shf.cuh"

#include <mutex>

namespace stpgb {

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device; in host code the array's name is only a host-side stand-in).
int noalloc_scratch(unsigned char** out) {
	int dev = 0;
	STPGB_CUDA_TRY(cudaGetDevice(&dev));
	if (dev < 0 || dev >= kMaxDevices) {
		return inval("stpgb_shf_filter_noalloc: device ordinal out of range");
	}
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	if (!g_noalloc_ptr[dev]) {
		void* p = nullptr;
		STPGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
		g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
	}
	*out = g_noalloc_ptr[dev];
	return STPGB_OK;
}

} // namespace

} // namespace stpgb

using namespace stpgb;

extern "C" int stpgb_shf_filter_noalloc(const uint16_t* samplemap, const stpgb_nn_info* nn, uint32_t radius,
	uint32_t max_items, uint32_t* offsets, stpgb_bin* bins, uint64_t bins_capacity, uint32_t* status, void* stream) {
	size_t need = 0u;
	STPGB_TRY(stpgb_shf_workspace_size(nn, radius, max_items, &need));
	if (need > kNoAllocScratchBytes) {
		set_error("stpgb_shf_filter_noalloc: this chunk needs " + std::to_string(need)
			+ " bytes of filter scratch, above the fixed 16 MiB array; use stpgb_shf_filter with a workspace");
		return STPGB_ECAPACITY;
	}
	unsigned char* scratch = nullptr;
	STPGB_TRY(noalloc_scratch(&scratch));
	return stpgb_shf_filter(samplemap, nn, radius, max_items, scratch, kNoAllocScratchBytes, offsets, bins,
		bins_capacity, status, stream);
}
