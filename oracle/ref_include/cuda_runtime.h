/*
 * Host stand-in for the CUDA runtime, used ONLY to compile the unmodified
 * reference program (kernel.cu + IDIC.h + data.h) with g++ so that its own
 * step loop can be run on the CPU to produce golden snapshots that pin the
 * oracle.  Test infrastructure: nothing in the product includes this file.
 *
 * What it provides, and why:
 *  - __global__/__device__/__host__ vanish, so every kernel becomes a plain
 *    host function that reads blockIdx/threadIdx from thread-local globals;
 *  - "device" memory is host memory: cudaMalloc = calloc, cudaMemcpy = memcpy;
 *  - cudaSetDevice / cudaDeviceSynchronize are no-ops (the reference ignores
 *    their return codes, kernel.cu:1793);
 *  - ds_ref_launch(grid, block, kernel)(args...) runs the kernel body once per
 *    (block, thread) index.  build_ref.sh rewrites the launch syntax
 *    `Kernel <<<grid, block>>> (args)` into that call, which is the only
 *    change made to the reference text.
 */
#pragma once
#include <cstdlib>
#include <cstring>
#include <cmath>
using std::abs;

#define __global__
#define __device__
#define __host__

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct ds_ref_idx { unsigned x, y, z; };
static thread_local ds_ref_idx blockIdx;
static thread_local ds_ref_idx threadIdx;

enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
                      cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
typedef int cudaError_t;
static inline cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(n ? n : 1, 1);
  return *p ? 0 : 2;
}
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, n);
}
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  memmove(d, s, n);
  return 0;
}
static inline cudaError_t cudaSetDevice(int) { return 0; }
static inline cudaError_t cudaDeviceSynchronize() { return 0; }

template <class F> struct ds_ref_launcher {
  dim3 g, b;
  F f;
  template <class... A> void operator()(A... a) const {
    /* Blocks are independent in every kernel the step loop launches (each
     * thread writes only its own particle), so blocks run in parallel. */
#pragma omp parallel for schedule(dynamic, 4)
    for (long bx = 0; bx < (long)g.x; bx++) {
      blockIdx.x = (unsigned)bx; blockIdx.y = 0; blockIdx.z = 0;
      for (unsigned tz = 0; tz < b.z; tz++)
        for (unsigned ty = 0; ty < b.y; ty++)
          for (unsigned tx = 0; tx < b.x; tx++) {
            threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
            f(a...);
          }
    }
  }
};
template <class F> static inline ds_ref_launcher<F> ds_ref_launch(dim3 g, dim3 b, F f) {
  return ds_ref_launcher<F>{g, b, f};
}
