// ds_sort.cuh -- stable LSD radix sort of (key, value) pairs (ds_sort.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <utility>

// Launches kernel k and returns the status of that launch alone (the value
// cudaLaunchKernelEx returns), without reading or clearing the thread's
// last-error state, so an earlier unrelated error is neither consumed nor
// blamed on this launch.
template <class... KArgs, class... Args>
static inline cudaError_t ds_launch(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Keys per radix tile and the most digit values of one pass (histogram rows).
constexpr int DS_RADIX_TILE = 2048;
constexpr int DS_RADIX_BINS = 1024;

// 32-bit words of scratch the sort of n pairs needs.
size_t ds_radix_scratch_words(int n);
int ds_radix_passes(int key_bits);

// Sorts the low key_bits of keys[0..n) with their vals, stably.  The sorted
// pairs end in (keys, vals) or, when *result_in_alt, in (keys_alt, vals_alt).
// Launch-only: capturable into a CUDA graph.  Returns the first failed
// launch's status (cudaSuccess if every pass launched); the thread's
// last-error state is left as the launches left it.  run_if: when given, the
// kernels do nothing if *run_if == 0 at run time (the pairs stay as they were).
cudaError_t ds_radix_sort(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt, int n,
                          int key_bits, uint32_t *scratch, cudaStream_t stream, bool *result_in_alt,
                          const int *run_if = nullptr);
