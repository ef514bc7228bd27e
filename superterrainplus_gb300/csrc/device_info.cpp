// Per-device properties and one-time per-device set-up, shared by the
// launches of every translation unit (thread-safe; a process may drive
// several devices).
#include "internal.hpp"

#include <mutex>

namespace stpgb {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
uint32_t g_sm_count[kMaxDevices] = {};
uint64_t g_done[kMaxDevices] = {};

} // namespace

uint32_t current_sm_count() {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
		cudaGetLastError();
		return 152u;
	}
	const std::lock_guard<std::mutex> lock(g_mutex);
	if (g_sm_count[dev] == 0u) {
		int sms = 0;
		if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
			cudaGetLastError();
			sms = 152;
		}
		g_sm_count[dev] = static_cast<uint32_t>(sms);
	}
	return g_sm_count[dev];
}

int once_per_device(const unsigned key, int (*const setup)()) {
	int dev = 0;
	STPGB_CUDA_TRY(cudaGetDevice(&dev));
	if (dev < 0 || dev >= kMaxDevices || key >= 64u) {
		return inval("device index or set-up key out of range");
	}
	const std::lock_guard<std::mutex> lock(g_mutex);
	const uint64_t bit = uint64_t { 1 } << key;
	if (g_done[dev] & bit) {
		return STPGB_OK;
	}
	const int rc = setup();
	if (rc == STPGB_OK) {
		g_done[dev] |= bit;
	}
	return rc;
}

} // namespace stpgb

extern "C" int stpgb_copy(void* dst, const void* src, size_t bytes, void* stream, int wait) {
	if (bytes == 0u) {
		return STPGB_OK;
	}
	if (!dst || !src) {
		return stpgb::inval("stpgb_copy: null buffer");
	}
	const cudaStream_t s = stpgb::as_stream(stream);
	STPGB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
	if (wait) {
		STPGB_CUDA_TRY(cudaStreamSynchronize(s));
	}
	return STPGB_OK;
}
