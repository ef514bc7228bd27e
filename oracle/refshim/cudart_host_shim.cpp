// Host-memory stand-ins for the few CUDA runtime calls the reference's host
// sources make (cudaMallocHost for pinned staging, cudaMalloc + cudaMemcpy in
// the permutation generator).  Linked only into oracle/_ref, the compiled
// reference used as a checker in a container without a GPU: "device" memory
// is plain host memory there.
#include <cuda_runtime_api.h>
#include <cstdlib>
#include <cstring>

extern "C" {

cudaError_t CUDARTAPI cudaMallocHost(void** ptr, size_t size) {
	*ptr = std::malloc(size ? size : 1);
	return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t CUDARTAPI cudaHostAlloc(void** ptr, size_t size, unsigned int) {
	*ptr = std::malloc(size ? size : 1);
	return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t CUDARTAPI cudaFreeHost(void* ptr) {
	std::free(ptr);
	return cudaSuccess;
}

cudaError_t CUDARTAPI cudaMalloc(void** ptr, size_t size) {
	*ptr = std::malloc(size ? size : 1);
	return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t CUDARTAPI cudaFree(void* ptr) {
	std::free(ptr);
	return cudaSuccess;
}

cudaError_t CUDARTAPI cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind) {
	std::memcpy(dst, src, count);
	return cudaSuccess;
}

const char* CUDARTAPI cudaGetErrorString(cudaError_t) {
	return "host shim";
}

const char* CUDARTAPI cudaGetErrorName(cudaError_t) {
	return "host shim";
}

}
