/* cudashim.h — lets the reference's CUDA kernel sources compile as host C++ for the
   oracle pin (oracle/ref). Kernel qualifiers vanish, launch indices become
   thread-local variables that the driver sets before calling a kernel body for
   one particle, and the few runtime calls the kernel files make map to memcpy. */
#ifndef ORC_CUDASHIM_H
#define ORC_CUDASHIM_H
#include <math.h>
#include <stdio.h>
#include <string.h>
#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __align__(n) __attribute__((aligned(n)))
struct orc_dim3 { unsigned int x, y, z; };
extern thread_local orc_dim3 blockIdx, threadIdx, blockDim, gridDim;
typedef int cudaError_t;
#define cudaSuccess 0
template <class T> inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n) {
    memcpy((void*)&sym, src, n);
    return 0;
}
inline float rsqrt(float x) { return 1.0f / sqrtf(x); }
inline int __mul24(int a, int b) { return a * b; }
inline unsigned int __mul24(unsigned int a, unsigned int b) { return a * b; }
inline const char* cudaGetErrorString(cudaError_t) { return "host"; }
inline cudaError_t cudaGetLastError() { return 0; }
#endif
