// ds_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs.
//
// Used twice per step: by neighbour-cell key (the reference's per-cell linked
// lists in ascending particle index, kernel.cu:1937-1955, become contiguous
// slot ranges) and by IDIC cell key (the reference's per-cell sums in particle
// order, kernel.cu:2114-2174, become segmented runs).  Stability is what makes
// both orders equal to the reference's: the input is fed in caller-index
// order, so equal keys keep ascending index.
//
// One pass per digit of <= 10 bits (as few passes as the key needs, digits as
// narrow as they allow), three kernels per pass:
//   rs_hist    per-tile digit histogram            -> hist[digit][tile]
//   rs_rowscan per-digit exclusive scan over tiles -> hist (in place) + totals
//   rs_scatter per-tile stable ranks (warp match-any + per-warp counters),
//              global offset = scan(totals)[digit] + hist[digit][tile]
// HBM traffic per pass: read key+value, write key+value (16 B per element)
// plus 2 x 4 B per digit value per tile of histogram.
#include <cstdint>
#include <cuda_runtime.h>

#include "ds_sort.cuh"

namespace {
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;                      // keys per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // 2048 keys per tile
static_assert(RS_TILE == DS_RADIX_TILE, "tile size is part of the scratch layout");
constexpr int RS_WARP_SPAN = 32 * RS_ITEMS;      // contiguous keys handled by one warp
#ifndef DS_RADIX_MAX_BITS
#define DS_RADIX_MAX_BITS 10
#endif
constexpr int RS_MAX_BITS = DS_RADIX_MAX_BITS;
constexpr int RS_BINS = 1 << RS_MAX_BITS;        // digit values at most
static_assert(RS_BINS <= DS_RADIX_BINS, "histogram rows are sized for DS_RADIX_BINS digit values");
constexpr int RS_DPT = RS_BINS / RS_THREADS;     // digit values per thread in the scatter's scan

// run_if (all three kernels): nullptr, or the sort is skipped when *run_if == 0
// (the whole grid returns at once, before any barrier).
__global__ void __launch_bounds__(RS_THREADS) rs_hist(const uint32_t *__restrict__ keys, int n, int shift,
                                                      uint32_t mask, uint32_t *__restrict__ hist, int ntiles,
                                                      const int *run_if) {
  if (run_if && *run_if == 0) return;
  __shared__ uint32_t h[RS_BINS];
  const int nbins = (int)mask + 1;
  for (int t = threadIdx.x; t < nbins; t += RS_THREADS) h[t] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  for (int k = threadIdx.x; k < RS_TILE; k += RS_THREADS) {
    int i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nbins; d += RS_THREADS) hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// One block per digit: exclusive scan of hist[d][0..ntiles) and its total.
__global__ void __launch_bounds__(256) rs_rowscan(uint32_t *__restrict__ hist, int ntiles,
                                                  uint32_t *__restrict__ totals, const int *run_if) {
  if (run_if && *run_if == 0) return;
  __shared__ uint32_t wsum[8];
  __shared__ uint32_t carry;
  uint32_t *row = hist + (size_t)blockIdx.x * ntiles;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < ntiles; base += 256) {
    int i = base + threadIdx.x;
    uint32_t v = i < ntiles ? row[i] : 0u;
    uint32_t s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) wsum[w] = s;
    __syncthreads();
    uint32_t wpre = 0, tot = 0;
    for (int k = 0; k < 8; k++) {
      uint32_t t = wsum[k];
      if (k < w) wpre += t;
      tot += t;
    }
    uint32_t c = carry;
    if (i < ntiles) row[i] = c + wpre + s - v;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(RS_THREADS) rs_scatter(const uint32_t *__restrict__ kin,
                                                         const uint32_t *__restrict__ vin,
                                                         uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                         int n, int shift, uint32_t mask,
                                                         const uint32_t *__restrict__ hist, int ntiles,
                                                         const uint32_t *__restrict__ totals, const int *run_if) {
  if (run_if && *run_if == 0) return;
  __shared__ uint32_t wcount[RS_WARPS][RS_BINS];
  __shared__ uint32_t goff[RS_BINS];
  __shared__ uint32_t wtot[RS_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nbins = (int)mask + 1;
  for (int k = 0; k < RS_WARPS; k++)
    for (int t = threadIdx.x; t < nbins; t += RS_THREADS) wcount[k][t] = 0;
  // digit bases: exclusive scan of the digit totals, RS_DPT consecutive digit
  // values per thread (thread order = digit order)
  {
    const int d0 = threadIdx.x * RS_DPT;
    uint32_t v[RS_DPT], local = 0;
#pragma unroll
    for (int j = 0; j < RS_DPT; j++) {
      v[j] = d0 + j < nbins ? totals[d0 + j] : 0u;
      local += v[j];
    }
    uint32_t s = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) wtot[w] = s;
    __syncthreads();
    uint32_t pre = s - local;
    for (int k = 0; k < w; k++) pre += wtot[k];
#pragma unroll
    for (int j = 0; j < RS_DPT; j++) {
      if (d0 + j < nbins) goff[d0 + j] = pre + hist[(size_t)(d0 + j) * ntiles + blockIdx.x];
      pre += v[j];
    }
  }
  __syncthreads();

  const unsigned lt_mask = (1u << lane) - 1u;
  const int base = blockIdx.x * RS_TILE + w * RS_WARP_SPAN;
  uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const int i = base + r * 32 + lane;
    const bool ok = i < n;
    key[r] = ok ? kin[i] : 0u;
    val[r] = ok ? vin[i] : 0u;
    const uint32_t d = ok ? ((key[r] >> shift) & mask) : (uint32_t)RS_BINS;  // RS_BINS: no digit
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = ok ? wcount[w][d] : 0u;
    rank[r] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) wcount[w][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive prefix over warps (warps cover consecutive sub-ranges)
  for (int d = threadIdx.x; d < nbins; d += RS_THREADS) {
    uint32_t run = 0;
    for (int k = 0; k < RS_WARPS; k++) {
      uint32_t t = wcount[k][d];
      wcount[k][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const int i = base + r * 32 + lane;
    if (i < n) {
      const uint32_t d = (key[r] >> shift) & mask;
      const uint32_t dst = goff[d] + wcount[w][d] + rank[r];
      kout[dst] = key[r];
      vout[dst] = val[r];
    }
  }
}
}  // namespace

size_t ds_radix_scratch_words(int n) {
  int ntiles = (n + RS_TILE - 1) / RS_TILE;
  if (ntiles < 1) ntiles = 1;
  return (size_t)RS_BINS * ntiles + RS_BINS;
}

int ds_radix_passes(int key_bits) { return key_bits <= 0 ? 0 : (key_bits + RS_MAX_BITS - 1) / RS_MAX_BITS; }

cudaError_t ds_radix_sort(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt, int n,
                          int key_bits, uint32_t *scratch, cudaStream_t stream, bool *result_in_alt,
                          const int *run_if) {
  *result_in_alt = false;
  if (n <= 0 || key_bits <= 0) return cudaSuccess;
  const int passes = ds_radix_passes(key_bits);
  const int width = (key_bits + passes - 1) / passes;
  const int ntiles = (n + RS_TILE - 1) / RS_TILE;
  uint32_t *hist = scratch;
  uint32_t *totals = scratch + (size_t)RS_BINS * ntiles;
  uint32_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
  for (int p = 0; p < passes; p++) {
    const int shift = p * width;
    int bits = key_bits - shift < width ? key_bits - shift : width;
    const uint32_t mask = (1u << bits) - 1u;
    cudaError_t e =
        ds_launch(rs_hist, dim3(ntiles), dim3(RS_THREADS), stream, ki, n, shift, mask, hist, ntiles, run_if);
    if (e == cudaSuccess)
      e = ds_launch(rs_rowscan, dim3((int)mask + 1), dim3(256), stream, hist, ntiles, totals, run_if);
    if (e == cudaSuccess)
      e = ds_launch(rs_scatter, dim3(ntiles), dim3(RS_THREADS), stream, ki, vi, ko, vo, n, shift, mask, hist,
                    ntiles, totals, run_if);
    if (e != cudaSuccess) return e;
    uint32_t *t = ki; ki = ko; ko = t;
    t = vi; vi = vo; vo = t;
  }
  *result_in_alt = (passes & 1) != 0;
  return cudaSuccess;
}
