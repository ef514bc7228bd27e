// Internal helpers shared by the translation units of libstpgb.so.
#pragma once

#include "stpgb.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

namespace stpgb {

// Thread-local message behind stpgb_last_error().
void set_error(const std::string& msg);
void clear_error();

// Device status word bits (set by kernels with atomicOr, read by stpgb_status_check).
enum : uint32_t {
	STATUS_CAPACITY = 1u << 0, // a caller-sized output or a per-window item bound was exceeded
	STATUS_TIMEOUT = 1u << 1   // a droplet reached the step cap
};

inline int cuda_fail(cudaError_t e, const char* what) {
	set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
	return STPGB_ECUDA;
}

inline int inval(const std::string& msg) {
	set_error(msg);
	return STPGB_EINVAL;
}

inline cudaStream_t as_stream(void* s) {
	return static_cast<cudaStream_t>(s);
}

// SM count of the current device, queried once per device (152 if the query fails).
uint32_t current_sm_count();

// Keys of one-time per-device set-up steps (function attributes are per device).
enum : unsigned { SETUP_SHF_SMEM = 0u, SETUP_SHF_BAND_SMEM = 1u };

// Runs `setup` on the current device the first time `key` is asked for there and it succeeds;
// serialised under a lock, so concurrent first calls from several host threads set up once.
int once_per_device(unsigned key, int (*setup)());

} // namespace stpgb

#define STPGB_CUDA_TRY(expr)                                   \
	do {                                                       \
		const cudaError_t stpgb_e_ = (expr);                   \
		if (stpgb_e_ != cudaSuccess) {                         \
			return ::stpgb::cuda_fail(stpgb_e_, #expr);        \
		}                                                      \
	} while (0)

#define STPGB_TRY(expr)                                        \
	do {                                                       \
		const int stpgb_rc_ = (expr);                          \
		if (stpgb_rc_ != STPGB_OK) {                           \
			return stpgb_rc_;                                  \
		}                                                      \
	} while (0)
