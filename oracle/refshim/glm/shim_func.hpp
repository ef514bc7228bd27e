// Function qualifier of the vector subset: host and device functions where a
// CUDA compiler (or the host stand-in of its language extensions) reads the
// header, so that the reference's device sources compile against it with
// nvcc as well as with a host compiler; plain functions elsewhere.
#pragma once
#if defined(__CUDACC__)
#define GLM_SHIM_FUNC __host__ __device__
#else
#define GLM_SHIM_FUNC
#endif
