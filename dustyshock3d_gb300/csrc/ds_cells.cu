// ds_cells.cu -- per-particle and per-cell kernels of one step (everything but
// the neighbour sweeps and the radix sort).
//
// Compiled with -fmad=false: the FP64 arithmetic follows the reference's
// operation order (IDIC.h, kernel.cu:2060-2523) without FMA contraction, so
// the results equal the oracle's (and the reference's CPU build) bit for bit.
//
// Order of one step (ds_api.cu enqueues it, graph-captured):
//   k_step_begin   per tube: active = Tm < T_end, reset the CFL minimum
//   k_keys         neighbour key per slot, scattered to caller-index order
//   (radix sort)   stable by key
//   k_reorder      gather every persistent field into the sorted order; FP32
//                  copies; IDIC key per slot, scattered to caller-index order
//   k_cell_start   first sorted slot of every key
//   (radix sort)   IDIC keys, stable
//   (sweeps)       density + EOS (+ dust density), t_stop, dt, force (FP32 path:
//                  the force walk of overflowed warps on a second stream)
//   k_idic_reduce  per IDIC cell and species: count, sum v, sum t_stop / sum A
//                  (FP32 path: k_idic_reduce_split, several lanes per cell)
//   k_idic_solve   per IDIC cell: means, eps, the implicit drag solve
//   k_relax_move   per particle: relax to the cell solution, move, energy
//   k_step_end     per tube: Tm += dt
#include <cstdint>
#include <cuda_runtime.h>

#include "ds_common.cuh"
#include "ds_kernels.cuh"

namespace {

__device__ __forceinline__ unsigned long long dbl_bits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// isfinite on the exponent bits (integer pipe; the same answer as isfinite)
__device__ __forceinline__ bool finite_bits(double v) {
  return ((unsigned)__double2hiint(v) & 0x7ff00000u) != 0x7ff00000u;
}

__global__ void k_step_begin(const TubeDesc *tubes, TubeState *ts, int ntubes, int *work) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (work && t < DS_NSWEEP) work[t] = 0;  // the persistent sweeps' chunk counters
  if (t >= ntubes) return;
  ts[t].active = ts[t].Tm < tubes[t].t_end ? 1 : 0;
  ts[t].dtmin_bits = dbl_bits(__longlong_as_double(0x7ff0000000000000LL));  // +inf
  ts[t].dt = 0.0;
}

// IDIC cell of a position, FP32 path: one FMA and one rounding conversion per
// axis (the index maps) instead of an FP64 division; GB300 runs FP64 at 2 lanes
// per SM per clock, so these per-particle kernels are bound by that pipe.
__device__ __forceinline__ int fast_idic_cell(const TubeDesc &T, double x, double y, double z) {
  const int ix = __double2int_rd(fma(x, T.iaa, T.iab[0]));
  const int iy = __double2int_rd(fma(y, T.iaa, T.iab[1]));
  const int iz = __double2int_rd(fma(z, T.iaa, T.iab[2]));
  if (ix < 0 || ix >= T.anx || iy < 0 || iy >= T.any_ || iz < 0 || iz >= T.anz) return -1;
  const int c = ix + iy * T.asy + iz * T.asz;
  return (c < 0 || c > T.n_idic) ? -1 : c;
}

// Neighbour key of each slot (kernel.cu:1949; out-of-range keys are not
// listed, kernel.cu:1950, and go to the orphan bucket ncells+1).  Reference
// order: written at the particle's caller index, so the stable sort keeps
// ascending index within a cell as the reference's lists do.  FP32 path:
// written in slot order (coalesced); a cell then keeps its previous order.
//
// List reuse (ts != nullptr): a tube that keeps its recorded lists this step
// keeps its slot order.  Its slots get the keys of the last sort (prev, the
// sort's output of the previous step, slot by slot) with their own slot as the
// value, so the stable sort leaves them where they are.
//
// slot_pid (FP32 path, a step on bound host arrays with list reuse): st holds
// the host's state in caller order, and slot i of the previous order holds
// particle slot_pid[i].  Slot i then keys that particle (st at seg_begin +
// slot_pid[i], which is also the value), so cells keep the previous slot
// order exactly as a step on the resident state does.
template <bool FAST>
__global__ void k_keys(const TubeDesc *tubes, const Chunk *chunks, int nchunks, DevState st, uint32_t *kin,
                       uint32_t *vin, const TubeState *ts, const uint32_t *prev, const int *slot_pid) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    const TubeDesc &T = tubes[ch.tube];
    const int j = (FAST && slot_pid) ? T.seg_begin[ch.species] + slot_pid[i] : i;  // the particle of slot i
    if (FAST && ts && !ts[ch.tube].rebuild) {
      kin[i] = prev[i];
      vin[i] = (uint32_t)j;
      continue;
    }
    int local;
    uint32_t bin = 0;
    if (FAST && (T.mode & M_GRID_PROPER)) {
      int ix, iy, iz;
      ds_fast_proper_cell(T, st.x[j], st.y[j], st.z[j], ix, iy, iz);
      const bool in = ix >= 0 && ix < T.nx && iy >= 0 && iy < T.ny && iz >= 0 && iz < T.nz;
      local = in ? ix + iy * T.sy + iz * T.sz : T.ncells + 1;
      // FP32 path: the particle's x within its cell in 2^xl bins, below the
      // cell in the key, so that each cell -- and so each row of cells -- is
      // sorted by x (the low bits of the fine x index)
      if (in) bin = (uint32_t)ds_fast_fine_x(T, st.x[j]) & ((1u << T.xl) - 1u);
    } else {
      const int key = ds_raw_key(T, st.x[i], st.y[i], st.z[i]);
      if (!(T.mode & M_GRID_PROPER))
        local = (key >= 0 && key <= T.ncells) ? key : T.ncells + 1;
      else
        local = key >= 0 ? key : T.ncells + 1;
    }
    const int dst = FAST ? i : T.seg_begin[ch.species] + st.pid[i];
    kin[dst] = FAST ? ((uint32_t)(T.key_base[ch.species] + local) << T.xl) | bin
                    : (uint32_t)(T.key_base[ch.species] + local);
    vin[dst] = (uint32_t)j;
  }
}

// FP32 coordinates of a slot's particle: offsets from the own (listed) cell's
// origin (proper grid), or from the tube's reference point (reference grid).
// FP32 path: x relative to the x-block origin (row walks), y, z to the cell's;
// the origins of grid cells from the tube's table (the same FP64 values,
// without the FP64 multiply-adds); a particle of a tube that kept its lists
// may have wrapped through a periodic face since its cell was set.  Shared by
// the reorder and the early FP32 copies of a bound step, so both give the
// same bits.
template <bool FAST>
__device__ __forceinline__ float4 slot_offsets(const TubeDesc &T, int species, uint32_t key, double x, double y,
                                               double z, bool keep) {
  float4 p4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (T.cellrel) {
    const int local = (int)(key >> (FAST ? T.xl : 0)) - T.key_base[species];
    int ix, iy, iz;
    if (local < T.ncells) {
      ix = local % T.nx;
      iy = (local / T.nx) % T.ny;
      iz = local / (T.nx * T.ny);
    } else if (FAST) {
      ds_fast_proper_cell(T, x, y, z, ix, iy, iz);
    } else {
      ds_proper_cell(T, x, y, z, ix, iy, iz);
    }
    const int bx = FAST ? ((ix >> DS_XB_LOG) << DS_XB_LOG) : ix;
    if (FAST && local < T.ncells) {
      p4.x = ds_d2f(x - T.orig[ix >> DS_XB_LOG]);
      double dy = y - T.orig[T.nbx + iy], dz = z - T.orig[T.nbx + T.ny + iz];
      if (keep) {
        if (T.mode & M_PER_Y) dy += dy > 0.5 * T.Ly ? -T.Ly : (dy < -0.5 * T.Ly ? T.Ly : 0.0);
        if (T.mode & M_PER_Z) dz += dz > 0.5 * T.Lz ? -T.Lz : (dz < -0.5 * T.Lz ? T.Lz : 0.0);
      }
      p4.y = ds_d2f(dy);
      p4.z = ds_d2f(dz);
    } else {
      p4.x = ds_d2f(x - (T.ox + bx * T.wx));
      p4.y = ds_d2f(y - (T.oy + iy * T.wy));
      p4.z = ds_d2f(z - (T.oz + iz * T.wz));
    }
  } else {
    p4.x = ds_d2f(x - T.fx);
    p4.y = ds_d2f(y - T.fy);
    p4.z = ds_d2f(z - T.fz);
  }
  return p4;
}

// A bound step with list reuse (early, before the host's other fields have
// arrived): the FP32 copies the streamed density reads -- pos32 (offsets and
// h) and pm32 (offsets and mass) -- for the gas of the tubes that keep their
// lists, from the host's positions, h and mass in caller order (slot q holds
// particle slot_pid[q]).  The reorder later writes the same values.
__global__ void k_early_fp32(const TubeDesc *tubes, const Chunk *chunks, int nchunks, const TubeState *ts,
                             const uint32_t *skey, DevState cs, const int *slot_pid, float4 *pos32, float4 *pm32) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int q = ch.begin + threadIdx.x;
    if (q >= ch.end || ts[ch.tube].rebuild) continue;
    const TubeDesc &T = tubes[ch.tube];
    const int j = T.seg_begin[ch.species] + slot_pid[q];
    float4 p4 = slot_offsets<true>(T, ch.species, skey[q], cs.x[j], cs.y[j], cs.z[j], true);
    const float mf = ds_d2f(cs.m[j]);
    p4.w = ds_d2f(cs.h[j]);
    pos32[q] = p4;
    pm32[q] = make_float4(p4.x, p4.y, p4.z, mf);
  }
}

// Gather every persistent field from the previous order (src) into the new
// sorted order (dst); build the FP32 copies and the IDIC keys (reference
// order: at the caller index, so the IDIC sums run in ascending index as the
// reference's host loops do; FP32 path: in slot order).
//
// List reuse (ts != nullptr): a tube keeping its lists is copied slot for slot
// (its order did not change), and its FP32 offsets stay relative to the cells
// the lists were recorded in (its keys are those of the last sort), taken to
// the nearest periodic image.  A tube that re-sorts stores its new offsets in
// pos_ref, the reference its later displacements are measured from.
template <bool FAST>
__global__ void k_reorder(const TubeDesc *tubes, const Chunk *chunks, int nchunks, const uint32_t *order,
                          const uint32_t *skey, DevState src, DevState dst, float4 *pos32, float4 *vm32,
                          int *idic_local, uint32_t *ikin, uint32_t *ivin, int *slot_of_pid, int *ind_of_pid,
                          int *flags, const TubeState *ts, float4 *pos_ref, const int *slot_pid, float4 *pm32) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int q = ch.begin + threadIdx.x;
    if (q >= ch.end) continue;
    const TubeDesc &T = tubes[ch.tube];
    const bool keep = FAST && ts && !ts[ch.tube].rebuild;
    // a kept tube's slot q holds the particle it held (k_keys): in src at q,
    // or, from bound host arrays in caller order, at seg_begin + slot_pid[q]
    const int j = keep ? (slot_pid ? T.seg_begin[ch.species] + slot_pid[q] : q) : (int)order[q];
    const double x = src.x[j], y = src.y[j], z = src.z[j];
    dst.x[q] = x; dst.y[q] = y; dst.z[q] = z;
    const double vx = src.vx[j], vy = src.vy[j], vz = src.vz[j];
    dst.vx[q] = vx; dst.vy[q] = vy; dst.vz[q] = vz;
    dst.ax[q] = src.ax[j]; dst.ay[q] = src.ay[j]; dst.az[q] = src.az[j];
    dst.rho[q] = src.rho[j]; dst.p[q] = src.p[j]; dst.e[q] = src.e[j];
    const double m = src.m[j], h = src.h[j];
    dst.m[q] = m; dst.h[q] = h;
    // proper grid: the cut-off 2h must stay within the stencil's cells, or the
    // walks (ds_radius clamps to the stencil) would miss partners.  Compared as
    // bit patterns (integer pipe): h in [+0, reach] passes; NaN, negative h
    // and h beyond the reach are flagged.
    if (dbl_bits((T.mode & M_HPP) ? h : T.h) > dbl_bits(T.reach_hmax)) atomicOr(flags, 8);  // DS_FLAG_REACH
    dst.ts[q] = src.ts[j];
    const int ind = src.ind[j], pid = src.pid[j];
    dst.ind[q] = ind; dst.pid[q] = pid;
    const int gp = T.seg_begin[ch.species] + pid;
    if (!(T.mode & M_TSTOP_CONST)) slot_of_pid[gp] = q;  // index-coupled stopping time (IDIC.h:86)
    if (T.mode & M_REF_COUPLING) ind_of_pid[gp] = ind;    // index-coupled dust rho zeroing (IDIC.h:8)
    // FP32 copies converted on the integer pipe (ds_d2f: the IEEE conversion)
    float4 p4 = slot_offsets<FAST>(T, ch.species, skey[q], x, y, z, keep);
    p4.w = ds_d2f(h);
    pos32[q] = p4;
    if (pm32) pm32[q] = make_float4(p4.x, p4.y, p4.z, ds_d2f(m));
    if (pos_ref && !keep) pos_ref[q] = p4;
    vm32[q] = make_float4(ds_d2f(vx), ds_d2f(vy), ds_d2f(vz), ds_d2f(m));
    const int ic = FAST ? fast_idic_cell(T, x, y, z) : ds_idic_cell(T, x, y, z);
    idic_local[q] = ic;
    const int idst = FAST ? q : gp;
    ikin[idst] = (uint32_t)(T.idic_base[ch.species] + (ic >= 0 ? ic : T.n_idic + 1));
    ivin[idst] = (uint32_t)q;
  }
}

// cell_start[k] = first sorted slot whose key is >= k, for k = 0..nkeys.
// run_if: skipped when *run_if == 0 (list reuse: no tube re-sorted, so the
// keys and their table are those of the last sort).
__global__ void k_cell_start(const uint32_t *skey, int n, int nkeys, int *cell_start, const int *run_if) {
  if (run_if && *run_if == 0) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > n) return;
  const long long prev = q > 0 ? (long long)skey[q - 1] : -1LL;
  const long long cur = q < n ? (long long)skey[q] : (long long)nkeys;
  for (long long k = prev + 1; k <= cur; k++) cell_start[k] = q;
}

// Index of the segment whose IDIC key range contains key (seg_key0 ascending).
__device__ __forceinline__ int find_seg(const int *seg_key0, int nseg, int key) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (seg_key0[mid] <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Per IDIC cell and species (one thread per key; run bounds from start[]):
// count and sums in the sorted order -- ascending particle index on the
// reference path, as the reference's host loops sum (kernel.cu:2114-2123,
// 2137-2146, 2165-2174, 2294-2300).  Empty cells get count 0.
__global__ void k_idic_reduce(const uint32_t *islot, int nikeys, const int *seg_key0, const int *seg_species,
                              const int *seg_orphan, int nseg, DevState st, CellArrays ca) {
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  if (key >= nikeys) return;
  const int sg = find_seg(seg_key0, nseg, key);
  if (key == seg_orphan[sg]) return;  // outside the IDIC grid
  const int s = seg_species[sg];
  const int r0 = ca.start[key], r1 = ca.start[key + 1];
  double vx = 0.0, vy = 0.0, vz = 0.0, a0 = 0.0, a1 = 0.0, a2 = 0.0;
  if (s == 0) {
#pragma unroll 4
    for (int r = r0; r < r1; r++) {
      const int j = (int)islot[r];
      vx = vx + st.vx[j];
      vy = vy + st.vy[j];
      vz = vz + st.vz[j];
      a0 = a0 + st.ax[j];
      a1 = a1 + st.ay[j];
      a2 = a2 + st.az[j];
    }
  } else {
#pragma unroll 4
    for (int r = r0; r < r1; r++) {
      const int j = (int)islot[r];
      a0 = a0 + st.ts[j];
      vx = vx + st.vx[j];
      vy = vy + st.vy[j];
      vz = vz + st.vz[j];
    }
  }
  ca.cnt[key] = r1 - r0;
  if (r1 > r0) {
    ca.vx[key] = vx; ca.vy[key] = vy; ca.vz[key] = vz;
    ca.a0[key] = a0; ca.a1[key] = a1; ca.a2[key] = a2;
  }
}

// FP32 path: the same sums with LANES lanes per key, each over a contiguous
// part of the key's slots in order, the parts added in order by the key's
// first lane: LANES times the threads of the one-lane walk (the FP32 path's
// 1.44M-particle tube has ~40k keys for 152 SMs, so that walk is latency-bound).
// The split depends only on the key's own slot count, so a tube sums the same
// alone and in a batch.
template <int LANES>
__global__ void k_idic_reduce_split(const uint32_t *islot, int nikeys, const int *seg_key0, const int *seg_species,
                                    const int *seg_orphan, int nseg, DevState st, CellArrays ca) {
  static_assert(LANES == 2 || LANES == 4 || LANES == 8, "lanes per key: a power of two dividing 32");
  const unsigned FULL = 0xffffffffu;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int key = (int)(t / LANES), part = (int)(t % LANES);
  bool ok = key < nikeys;
  int s = 0, r0 = 0, r1 = 0;
  if (ok) {
    const int sg = find_seg(seg_key0, nseg, key);
    ok = key != seg_orphan[sg];  // outside the IDIC grid
    s = seg_species[sg];
    r0 = ca.start[key];
    r1 = ca.start[key + 1];
  }
  const int n = r1 - r0;
  const int a = r0 + (int)((long long)n * part / LANES), b = r0 + (int)((long long)n * (part + 1) / LANES);
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (ok && s == 0) {
#pragma unroll 4
    for (int r = a; r < b; r++) {
      const int j = (int)islot[r];
      v[0] = v[0] + st.vx[j];
      v[1] = v[1] + st.vy[j];
      v[2] = v[2] + st.vz[j];
      v[3] = v[3] + st.ax[j];
      v[4] = v[4] + st.ay[j];
      v[5] = v[5] + st.az[j];
    }
  } else if (ok) {
#pragma unroll 4
    for (int r = a; r < b; r++) {
      const int j = (int)islot[r];
      v[3] = v[3] + st.ts[j];
      v[0] = v[0] + st.vx[j];
      v[1] = v[1] + st.vy[j];
      v[2] = v[2] + st.vz[j];
    }
  }
  // the parts in order, (((q0 + q1) + q2) + ...), at the key's first lane
#pragma unroll
  for (int k = 0; k < 6; k++) {
    double sum = v[k];
#pragma unroll
    for (int d = 1; d < LANES; d++) sum = sum + __shfl_down_sync(FULL, v[k], d);
    v[k] = sum;
  }
  if (!ok || part != 0) return;
  ca.cnt[key] = n;
  if (n > 0) {
    ca.vx[key] = v[0]; ca.vy[key] = v[1]; ca.vz[key] = v[2];
    ca.a0[key] = v[3]; ca.a1[key] = v[4]; ca.a2[key] = v[5];
  }
}

// One component of the per-cell implicit solve (kernel.cu:2310-2437); the
// reference's two-species operation order when ref2, Sherman-Morrison for any
// species count otherwise (the same algebra).  ND is a compile-time species
// count so every array below lives in registers (fully unrolled loops).
template <int ND>
__device__ __forceinline__ void solve_comp(const double (&eps)[ND], const double (&t)[ND], double vg,
                                           const double (&vd)[ND], double psi, double tau, bool ref2,
                                           double &g_out, double (&d_out)[ND]) {
  if constexpr (ND == 2) {
    if (ref2) {
      double y = vg, x1 = vg - vd[0], x2 = vg - vd[1];
      y = y + eps[0] * vd[0] + eps[1] * vd[1];
      double b1 = (t[0] + tau) / (eps[0] * tau);
      double b2 = (t[1] + tau) / (eps[1] * tau);
      double beta = 1.0;
      beta = beta + 1.0 / b1 + 1.0 / b2;
      double yn = y + tau * psi;
      double x1n = -1.0 * b1 * beta * (x1 + tau * psi) / (b1 * b1);
      x1n = x1n + (x1 + tau * psi) / (b1 * b1) + (x2 + tau * psi) / (b1 * b2);
      x1n = x1n * (-1.0 * t[0]) / (tau * eps[0] * beta);
      double x2n = -1.0 * b2 * beta * (x2 + tau * psi) / (b2 * b2);
      x2n = x2n + (x1 + tau * psi) / (b2 * b1) + (x2 + tau * psi) / (b2 * b2);
      x2n = x2n * (-1.0 * t[1]) / (tau * eps[1] * beta);
      double tmp1 = 1.0;
      tmp1 = tmp1 + eps[0] + eps[1];
      double g = yn;
      g = g + eps[0] * x1n;
      double d1 = yn;
      d1 = d1 + eps[1] * x2n;
      d1 = d1 - (tmp1 - eps[0]) * x1n;
      d1 = d1 / tmp1;
      g = g + eps[1] * x2n;
      double d2 = yn;
      d2 = d2 + eps[0] * x1n;
      d2 = d2 - (tmp1 - eps[1]) * x2n;
      d2 = d2 / tmp1;
      g = g / tmp1;
      g_out = g;
      d_out[0] = d1;
      d_out[1] = d2;
      return;
    }
  }
  double b[ND], r[ND], xn[ND];
  double y = vg, beta = 1.0, S = 0.0, E = 1.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    y = y + eps[k] * vd[k];
    b[k] = (t[k] + tau) / (eps[k] * tau);
    beta = beta + 1.0 / b[k];
    r[k] = (vg - vd[k]) + tau * psi;
    S = S + r[k] / b[k];
    E = E + eps[k];
  }
  const double yn = y + tau * psi;
  double g = yn;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    const double u = r[k] / b[k] - S / (b[k] * beta);
    xn[k] = u * t[k] / (eps[k] * tau);
    g = g + eps[k] * xn[k];
  }
  g = g / E;
  g_out = g;
#pragma unroll
  for (int k = 0; k < ND; k++) d_out[k] = g - xn[k];
}

// FP32 path: the same per-cell solve (means, eps, Psi, the implicit drag and
// the relax coefficients) with every quantity that does not depend on the
// component computed once per cell and reciprocals in place of divisions:
// ~8 FP64 divisions per cell instead of ~28 (GB300's FP64 pipe runs 2 lanes
// per SM per clock).  With 1/b_k = eps_k tau / (t_k + tau) the
// Sherman-Morrison terms of solve_comp reduce to
//   xn_k = t_k / (t_k + tau) (r_k - S / beta),  S = sum_k r_k / b_k,
// and a species with eps_k = 0 gives NaN there as solve_comp does.
template <int ND>
__device__ __forceinline__ void idic_solve_cell_fast(const TubeDesc &T, int c, double tau, CellArrays &ca) {
  const int kg = T.idic_base[0] + c;
  const int cg = ca.cnt[kg];
  const double icg = cg > 0 ? 1.0 / cg : 0.0;
  double vg[3] = {0.0, 0.0, 0.0}, ps[3] = {0.0, 0.0, 0.0};
  if (cg > 0) {
    vg[0] = ca.vx[kg] * icg; vg[1] = ca.vy[kg] * icg; vg[2] = ca.vz[kg] * icg;
    ps[0] = ca.a0[kg] * icg; ps[1] = ca.a1[kg] * icg; ps[2] = ca.a2[kg] * icg;
  }
  double eps[ND], tt[ND], vd[3][ND], q[ND], q0[ND], ib[ND];
  double beta = 1.0, E = 1.0;
  const int c1 = ca.cnt[T.idic_base[1] + c];
#pragma unroll
  for (int k = 0; k < ND; k++) {
    const int kd = T.idic_base[k + 1] + c;
    const int cd = ca.cnt[kd];
    if (cd > 0) {
      const double icd = 1.0 / cd;
      vd[0][k] = ca.vx[kd] * icd; vd[1][k] = ca.vy[kd] * icd; vd[2][k] = ca.vz[kd] * icd;
      tt[k] = ca.a0[kd] * icd;
    } else {
      vd[0][k] = 0.0; vd[1][k] = 0.0; vd[2][k] = 0.0;
      tt[k] = T.t_empty;
    }
    const int guard = (T.mode & M_REF_EPS_GUARD) ? c1 : cd;
    eps[k] = ((cg > 0) && (guard > 0)) ? (cd * T.mass_ratio[k]) * icg : T.eps_empty[k];
    q[k] = 1.0 / (tt[k] + tau);
    q0[k] = tt[k] * q[k];
    ib[k] = eps[k] * tau * q[k];
    beta = beta + ib[k];
    E = E + eps[k];
  }
  const double ibeta = 1.0 / beta, iE = 1.0 / E;
  double gnew[3], dnew[3][ND];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double tp = tau * ps[a];
    double y = vg[a], S = 0.0, r[ND];
#pragma unroll
    for (int k = 0; k < ND; k++) {
      y = fma(eps[k], vd[a][k], y);
      r[k] = (vg[a] - vd[a][k]) + tp;
      S = fma(r[k], ib[k], S);
    }
    const double Sb = S * ibeta;
    double g = y + tp, xn[ND];
#pragma unroll
    for (int k = 0; k < ND; k++) {
      xn[k] = eps[k] != 0.0 ? (r[k] - Sb) * q0[k] : __longlong_as_double(0x7ff8000000000000LL);
      g = fma(eps[k], xn[k], g);
    }
    g = g * iE;
    gnew[a] = g;
#pragma unroll
    for (int k = 0; k < ND; k++) dnew[a][k] = g - xn[k];
  }
  ca.nvx[kg] = gnew[0]; ca.nvy[kg] = gnew[1]; ca.nvz[kg] = gnew[2];
  ca.px[kg] = ps[0]; ca.py[kg] = ps[1]; ca.pz[kg] = ps[2];
  // relax coefficients (the relaxations of IDIC.h:276-313 as v_new = q0 v + q1 (...)):
  //   dust  t/(t+tau) v + tau/(t+tau) g;  gas  (v/tau + N + a)/D, D = 1/tau + sum eps/t
  const double itau = 1.0 / tau;
  double D = itau, Nx = 0.0, Ny = 0.0, Nz = 0.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    const int kd = T.idic_base[k + 1] + c;
    ca.nvx[kd] = dnew[0][k]; ca.nvy[kd] = dnew[1][k]; ca.nvz[kd] = dnew[2][k];
    ca.px[kd] = tt[k];   // dust: mean t_stop
    ca.py[kd] = eps[k];  // dust: eps
    const double w = eps[k] / tt[k];
    D = D + w;
    Nx = fma(w, dnew[0][k], Nx); Ny = fma(w, dnew[1][k], Ny); Nz = fma(w, dnew[2][k], Nz);
    ca.q0[kd] = q0[k];
    ca.q1[kd] = tau * q[k];
  }
  const double iD = 1.0 / D;
  ca.q0[kg] = iD * itau;
  ca.q1[kg] = iD;
  ca.a0[kg] = Nx; ca.a1[kg] = Ny; ca.a2[kg] = Nz;
}

// Per (tube, IDIC cell): means (kernel.cu:2126-2190), eps (2192-2211),
// Psi (2302-2309), solve (2310-2437).  Results are written at the cell's key
// of each species: new velocities; for gas Psi; for dust the mean t_stop and eps.
template <int ND, bool FAST>
__device__ __forceinline__ void idic_solve_cell(const TubeDesc &T, int c, double tau, CellArrays &ca) {
  if constexpr (FAST) {
    idic_solve_cell_fast<ND>(T, c, tau, ca);
    return;
  }
  const int kg = T.idic_base[0] + c;
  const int cg = ca.cnt[kg];
  double vgx = 0.0, vgy = 0.0, vgz = 0.0, psx = 0.0, psy = 0.0, psz = 0.0;
  if (cg > 0) {
    vgx = ca.vx[kg] / cg; vgy = ca.vy[kg] / cg; vgz = ca.vz[kg] / cg;
    psx = ca.a0[kg] / cg; psy = ca.a1[kg] / cg; psz = ca.a2[kg] / cg;
  }
  double eps[ND], tt[ND], vdx[ND], vdy[ND], vdz[ND];
  const int c1 = ca.cnt[T.idic_base[1] + c];
#pragma unroll
  for (int k = 0; k < ND; k++) {
    const int kd = T.idic_base[k + 1] + c;
    const int cd = ca.cnt[kd];
    if (cd > 0) {
      vdx[k] = ca.vx[kd] / cd; vdy[k] = ca.vy[kd] / cd; vdz[k] = ca.vz[kd] / cd;
      tt[k] = ca.a0[kd] / cd;
    } else {
      vdx[k] = 0.0; vdy[k] = 0.0; vdz[k] = 0.0;
      tt[k] = T.t_empty;
    }
    const int guard = (T.mode & M_REF_EPS_GUARD) ? c1 : cd;
    eps[k] = ((cg > 0) && (guard > 0)) ? cd * T.mass_ratio[k] / cg : T.eps_empty[k];
  }
  const bool ref2 = (T.mode & M_REF_SOLVE2) != 0;
  double gx, gy, gz, ox[ND], oy[ND], oz[ND];
  solve_comp<ND>(eps, tt, vgx, vdx, psx, tau, ref2, gx, ox);
  solve_comp<ND>(eps, tt, vgy, vdy, psy, tau, ref2, gy, oy);
  solve_comp<ND>(eps, tt, vgz, vdz, psz, tau, ref2, gz, oz);
  ca.nvx[kg] = gx; ca.nvy[kg] = gy; ca.nvz[kg] = gz;
  ca.px[kg] = psx; ca.py[kg] = psy; ca.pz[kg] = psz;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    const int kd = T.idic_base[k + 1] + c;
    ca.nvx[kd] = ox[k]; ca.nvy[kd] = oy[k]; ca.nvz[kd] = oz[k];
    ca.px[kd] = tt[k];   // dust: mean t_stop
    ca.py[kd] = eps[k];  // dust: eps
  }
}

template <bool FAST>
__global__ void k_idic_solve(const TubeDesc *tubes, const TubeState *tstate, const int *tube_cell0, int ntubes,
                             int ncell_total, CellArrays ca) {
  const int gc = blockIdx.x * blockDim.x + threadIdx.x;
  if (gc >= ncell_total) return;
  int lo = 0, hi = ntubes - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tube_cell0[mid] <= gc) lo = mid; else hi = mid - 1;
  }
  const int t = lo;
  if (!tstate[t].active) return;
  const TubeDesc &T = tubes[t];
  const int c = gc - tube_cell0[t];
  const double tau = tstate[t].dt;
  switch (T.n_dust) {
    case 1: idic_solve_cell<1, FAST>(T, c, tau, ca); break;
    case 2: idic_solve_cell<2, FAST>(T, c, tau, ca); break;
    case 3: idic_solve_cell<3, FAST>(T, c, tau, ca); break;
    default: idic_solve_cell<4, FAST>(T, c, tau, ca); break;
  }
}

// V_dustKernel_IDIC / V_gasKernel_IDIC (IDIC.h:264-315), MoveKernel_IDIC
// (IDIC.h:319-333, periodic wrap as an extension), EnergyKernel_IDIC (335-346).
template <bool FAST>
__global__ void k_relax_move(const TubeDesc *tubes, const TubeState *tstate, const Chunk *chunks, int nchunks,
                             DevState st, const int *idic_local, const double *edot, CellArrays ca, int *flags) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    if (!tstate[ch.tube].active) continue;
    if (st.ind[i] != 0) continue;
    const TubeDesc &T = tubes[ch.tube];
    const double tau = tstate[ch.tube].dt;
    const int s = ch.species;
    const int cell = idic_local[i];
    double vx = st.vx[i], vy = st.vy[i], vz = st.vz[i];
    if (cell < 0) {
      atomicOr(flags, 1);  // DS_FLAG_IDIC_RANGE: left unrelaxed
    } else if (FAST) {
      const int kg = T.idic_base[0] + cell;
      // FP32 path: fused multiply-adds (fewer FP64-pipe instructions)
      if (s > 0) {
        const int kd = T.idic_base[s] + cell;
        const double a0 = ca.q0[kd], a1 = ca.q1[kd];
        vx = fma(a1, ca.nvx[kg], a0 * vx);
        vy = fma(a1, ca.nvy[kg], a0 * vy);
        vz = fma(a1, ca.nvz[kg], a0 * vz);
      } else {
        const bool own = (T.mode & M_GAS_ACC_P) != 0;
        const double a0 = ca.q0[kg], a1 = ca.q1[kg];
        vx = fma(a1, ca.a0[kg] + (own ? st.ax[i] : ca.px[kg]), a0 * vx);
        vy = fma(a1, ca.a1[kg] + (own ? st.ay[i] : ca.py[kg]), a0 * vy);
        vz = fma(a1, ca.a2[kg] + (own ? st.az[i] : ca.pz[kg]), a0 * vz);
      }
    } else if (s > 0) {
      const int kg = T.idic_base[0] + cell, kd = T.idic_base[s] + cell;
      const double ts = ca.px[kd];
      vx = (vx / tau + ca.nvx[kg] / ts) / (1.0 / tau + 1.0 / ts);
      vy = (vy / tau + ca.nvy[kg] / ts) / (1.0 / tau + 1.0 / ts);
      vz = (vz / tau + ca.nvz[kg] / ts) / (1.0 / tau + 1.0 / ts);
    } else {
      const int kg = T.idic_base[0] + cell;
      double tmp1 = 0.0, tmp_x = 0.0, tmp_y = 0.0, tmp_z = 0.0;
      for (int k = 1; k <= T.n_dust; k++) {
        const int kd = T.idic_base[k] + cell;
        tmp1 = tmp1 + ca.py[kd] / ca.px[kd];
      }
      for (int k = 1; k <= T.n_dust; k++) {
        const int kd = T.idic_base[k] + cell;
        tmp_x = tmp_x + ca.py[kd] * ca.nvx[kd] / ca.px[kd];
      }
      for (int k = 1; k <= T.n_dust; k++) {
        const int kd = T.idic_base[k] + cell;
        tmp_y = tmp_y + ca.py[kd] * ca.nvy[kd] / ca.px[kd];
      }
      for (int k = 1; k <= T.n_dust; k++) {
        const int kd = T.idic_base[k] + cell;
        tmp_z = tmp_z + ca.py[kd] * ca.nvz[kd] / ca.px[kd];
      }
      const bool own = (T.mode & M_GAS_ACC_P) != 0;
      const double ax = own ? st.ax[i] : ca.px[kg];
      const double ay = own ? st.ay[i] : ca.py[kg];
      const double az = own ? st.az[i] : ca.pz[kg];
      vx = (vx / tau + tmp_x + ax) / (1.0 / tau + tmp1);
      vy = (vy / tau + tmp_y + ay) / (1.0 / tau + tmp1);
      vz = (vz / tau + tmp_z + az) / (1.0 / tau + tmp1);
    }
    st.vx[i] = vx; st.vy[i] = vy; st.vz[i] = vz;
    double x = FAST ? fma(vx, tau, st.x[i]) : st.x[i] + vx * tau;
    double y = FAST ? fma(vy, tau, st.y[i]) : st.y[i] + vy * tau;
    double z = FAST ? fma(vz, tau, st.z[i]) : st.z[i] + vz * tau;
    if (FAST) {  // the same comparisons on order keys (integer pipe)
      if (T.mode & M_PER_Y) {
        const int64_t k = ds_order_key(y);
        if (k < T.wrap_key[0]) y = y + T.Ly;
        else if (k >= T.wrap_key[1]) y = y - T.Ly;
      }
      if (T.mode & M_PER_Z) {
        const int64_t k = ds_order_key(z);
        if (k < T.wrap_key[2]) z = z + T.Lz;
        else if (k >= T.wrap_key[3]) z = z - T.Lz;
      }
    } else {
      if (T.mode & M_PER_Y) {
        if (y < T.oy) y = y + T.Ly;
        else if (y >= T.ymax) y = y - T.Ly;
      }
      if (T.mode & M_PER_Z) {
        if (z < T.oz) z = z + T.Lz;
        else if (z >= T.zmax) z = z - T.Lz;
      }
    }
    st.x[i] = x; st.y[i] = y; st.z[i] = z;
    double e = 0.0;
    if (s == 0) {
      e = FAST ? fma(edot[i], tau, st.e[i]) : st.e[i] + edot[i] * tau;
      st.e[i] = e;
    }
    if (!(finite_bits(vx) && finite_bits(vy) && finite_bits(vz) && finite_bits(x) && finite_bits(y) &&
          finite_bits(z) && finite_bits(e)))
      atomicOr(flags, 4);  // DS_FLAG_NONFINITE
  }
}

// t_stop_Kernel_IDIC (IDIC.h:78-91): t = R / (sqrt(gam p/rho) rho) with the GAS
// p, rho at the dust particle's own index (kernel.cu:2049); or constant.
__global__ void k_tstop(const TubeDesc *tubes, const TubeState *tstate, const Chunk *chunks, int nchunks,
                        DevState st, const int *gas_slot_of_pid, int *flags) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    if (!tstate[ch.tube].active) continue;
    if (st.ind[i] != 0) continue;
    const TubeDesc &T = tubes[ch.tube];
    const int k = ch.species - 1;
    if (T.mode & M_TSTOP_CONST) {
      st.ts[i] = T.t_stop_const[k];
      continue;
    }
    const int q = st.pid[i];
    const int ng = T.seg_end[0] - T.seg_begin[0];
    if (q >= ng) {
      atomicOr(flags, 2);
      continue;
    }
    const int g = gas_slot_of_pid[T.seg_begin[0] + q];
    const double p = st.p[g], rho = st.rho[g];
    st.ts[i] = T.R_dust[k] / (sqrt(T.gam * p / rho) * rho);
  }
}

// Step size per tube: fixed tau (kernel.cu:1931) or CFL number x min over
// gas of h/(c + |v|), clipped to end exactly at T_end.
__global__ void k_dt(const TubeDesc *tubes, TubeState *ts, int ntubes) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntubes) return;
  if (!ts[t].active) return;
  const TubeDesc &T = tubes[t];
  double dt = T.tau;
  if (T.mode & M_CFL) {
    dt = T.cfl * __longlong_as_double((long long)ts[t].dtmin_bits);
    if (ts[t].Tm + dt > T.t_end) dt = T.t_end - ts[t].Tm;
  }
  ts[t].dt = dt;
}

__global__ void k_step_end(TubeState *ts, int ntubes) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntubes) return;
  if (!ts[t].active) return;
  ts[t].Tm = ts[t].Tm + ts[t].dt;
  ts[t].nstep = ts[t].nstep + 1;
}

// Conservation sums of one tube, deterministic: one block, fixed order.
__global__ void k_conservation(const TubeDesc *tubes, int tube, DevState st, double *out) {
  __shared__ double sh[6][256];
  const TubeDesc &T = tubes[tube];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const int ns = 1 + T.n_dust;
  for (int s = 0; s < ns; s++)
    for (int i = T.seg_begin[s] + threadIdx.x; i < T.seg_end[s]; i += blockDim.x) {
      const double m = st.m[i];
      acc[0] += m;
      acc[1] += m * st.vx[i];
      acc[2] += m * st.vy[i];
      acc[3] += m * st.vz[i];
      if (s == 0) acc[4] += m * st.e[i];
      acc[5] += 0.5 * m * (st.vx[i] * st.vx[i] + st.vy[i] * st.vy[i] + st.vz[i] * st.vz[i]);
    }
  for (int k = 0; k < 6; k++) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 6; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; k++) out[k] = sh[k][0];
}

// Reference linked lists of one segment from the sorted order: head[c] = pid
// of the first slot of cell c, next[pid] = pid of the following slot in the
// same cell (kernel.cu:1937-1955), plus the raw key per pid.
__global__ void k_debug_lists(const TubeDesc *tubes, int tube, int s, DevState st, const int *cell_start, int xl,
                              int *head, int *next, int *rawkey) {
  const TubeDesc &T = tubes[tube];
  const int b = T.seg_begin[s], e = T.seg_end[s];
  const int q = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (q < e) {
    const int pid = st.pid[q];
    rawkey[pid] = ds_raw_key(T, st.x[q], st.y[q], st.z[q]);
  }
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= T.ncells) {
    const int kb = T.key_base[s];
    const int j0 = cell_start[(kb + c) << xl], j1 = cell_start[(kb + c + 1) << xl];
    head[c] = j0 < j1 ? st.pid[j0] : -1;
    for (int j = j0; j < j1; j++) next[st.pid[j]] = (j + 1 < j1) ? st.pid[j + 1] : -1;
  }
}

// Stencil radius each cell's force sweep needs: the cells its particles'
// partners (r < 2 max(h_i, h_j)) can lie in, i.e. ceil(2 H rw) with H the
// largest h within the tube's stencil (ds_radius), so cells whose cut-offs are
// short walk fewer cells.  Separable passes over the key space: h_max per cell,
// its maximum over the x window, the y window, then the z window (periodic
// axes wrap).  Reference grids and the orphan buckets keep the tube's stencil;
// tubes without per-particle h (every cut-off 2 h of the run) take its radius.
__global__ void k_cell_hmax(const int *cell_start, int nkeys, int xl, const double *h, double *hmax,
                            const int *run_if) {
  if (run_if && *run_if == 0) return;
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  if (key >= nkeys) return;
  // maximum as bit patterns (integer pipe): the same value as fmax for h >= 0
  long long m = 0;
  for (int j = cell_start[key << xl]; j < cell_start[(key + 1) << xl]; j++) {
    const long long b = __double_as_longlong(h[j]);
    m = b > m ? b : m;
  }
  hmax[key] = __longlong_as_double(m);
}

// axis 0: x window, 1: y window, 2: z window (then the radius)
template <int AXIS>
__global__ void k_cell_window(const TubeDesc *tubes, const int *nseg_key0, const int *nseg_tube,
                              const int *nseg_species, int nseg, int nkeys, const double *in, double *out,
                              unsigned char *krad, const int *run_if) {
  if (run_if && *run_if == 0) return;
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  if (key >= nkeys) return;
  const int sg = find_seg(nseg_key0, nseg, key);
  const TubeDesc &T = tubes[nseg_tube[sg]];
  const int kb = T.key_base[nseg_species[sg]];
  const int local = key - kb;
  const bool whole = T.stencil == 1 || local >= T.ncells || !(T.mode & M_GRID_PROPER);
  if (whole) {
    if (AXIS == 2) krad[key] = (unsigned char)T.stencil;
    else out[key] = in[key];
    return;
  }
  if (!(T.mode & M_HPP)) {  // one h for every pair (the run's h, not the h field): one radius
    if (AXIS == 2) krad[key] = (unsigned char)ds_radius(T, 2.0 * T.h + T.skin);
    return;
  }
  const int ix = local % T.nx, iy = (local / T.nx) % T.ny, iz = local / (T.nx * T.ny);
  const int R = T.stencil;
  double m = 0.0;
  for (int d = -R; d <= R; d++) {
    int c;
    if (AXIS == 0) {
      if (ix + d < 0 || ix + d >= T.nx) continue;
      c = key + d;
    } else if (AXIS == 1) {
      int cy = iy + d;
      if (T.mode & M_PER_Y) cy = (cy + T.ny) % T.ny;
      else if (cy < 0 || cy >= T.ny) continue;
      c = kb + ix + cy * T.sy + iz * T.sz;
    } else {
      int cz = iz + d;
      if (T.mode & M_PER_Z) cz = (cz + T.nz) % T.nz;
      else if (cz < 0 || cz >= T.nz) continue;
      c = kb + ix + iy * T.sy + cz * T.sz;
    }
    m = fmax(m, in[c]);
  }
  if (AXIS == 2) krad[key] = (unsigned char)ds_radius(T, 2.0 * m + T.skin);  // the recorded cut-off
  else out[key] = m;
}

// FP32 path origins (TubeDesc::orig), with the same FP64 arithmetic as the
// per-particle origin it replaces: o + (double)i * w, no contraction.
__global__ void k_origins(double ox, double wx, int nbx, double oy, double wy, int ny, double oz, double wz, int nz,
                          double *orig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nbx) orig[i] = ox + (i * DS_XB) * wx;
  else if (i < nbx + ny) orig[i] = oy + (i - nbx) * wy;
  else if (i < nbx + ny + nz) orig[i] = oz + (i - nbx - ny) * wz;
}

// ---------------------------------------------------------------------------
// List reuse: the test, at the start of a step, of whether a tube's recorded
// lists still hold every pair within its cut-off.  The lists of particle i
// hold every j with |x0_i - x0_j| < rc_ij = 2 max(h_i, h_j) + skin (x0: the
// positions when they were recorded).  With d the displacements since then, a
// pair now within 2 max(h_i, h_j) that is not listed has |d_i - d_j| > skin.
// Per cell c of the recording sort: m_c, the mean displacement of its
// particles, and dev_c, the largest |d_i - m_c| in it.  For i in c, j in c',
// |d_i - d_j| <= dev_c + dev_c' + |m_c - m_c'| (the triangle inequality).
//   * c' within r_c + 1 cells of c (r_c: the cells the recording walk of c
//     searched, r_c w >= rc_ij, w the least cell width): the tube keeps its
//     lists only while dev_c + dev_c' + |m_c - m_c'| < skin for all of them.
//   * c' further (along some axis more than r_c + 1 cells): the pair was more
//     than (r_c + 1) w >= rc_ij + w apart, so it is within its cut-off now
//     only if |d_i - d_j| > skin + w; bounded by 2 G + |M|, G the tube's
//     largest dev_c and |M| the diagonal of the box holding every m_c.  The
//     tube keeps its lists only while 2 G + |M| < skin + w.
// A particle outside the grid (its own bucket, no cell) makes its tube
// re-sort every step.  The values are the FP32 offsets the screens use; the
// decision keeps 0.1 % of each threshold for their rounding.
// ---------------------------------------------------------------------------

// order-preserving map of a float to an unsigned (for atomicMin / atomicMax)
__device__ __forceinline__ unsigned ord_bits(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord_float(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Combine v into *p with one atomic per group of lanes naming the same p
// (p == nullptr: nothing).  Every lane of the warp calls it.
__device__ __forceinline__ void warp_atomic_max(unsigned *p, unsigned v) {
  const unsigned grp = __match_any_sync(0xffffffffu, (unsigned long long)p);
  const unsigned m = __reduce_max_sync(grp, v);
  if (p && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(p, m);
}
__device__ __forceinline__ void warp_atomic_min(unsigned *p, unsigned v) {
  const unsigned grp = __match_any_sync(0xffffffffu, (unsigned long long)p);
  const unsigned m = __reduce_min_sync(grp, v);
  if (p && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMin(p, m);
}

// the FP32 offset of a position from the cell (ix, iy, iz) of the FP32 path
// (x from the cell's x-block origin), periodic axes to the nearest image
__device__ __forceinline__ float4 list_offset(const TubeDesc &T, int ix, int iy, int iz, double x, double y, double z) {
  double dy = y - T.orig[T.nbx + iy], dz = z - T.orig[T.nbx + T.ny + iz];
  if (T.mode & M_PER_Y) dy += dy > 0.5 * T.Ly ? -T.Ly : (dy < -0.5 * T.Ly ? T.Ly : 0.0);
  if (T.mode & M_PER_Z) dz += dz > 0.5 * T.Lz ? -T.Lz : (dz < -0.5 * T.Lz ? T.Lz : 0.0);
  return make_float4(ds_d2f(x - T.orig[ix >> DS_XB_LOG]), ds_d2f(dy), ds_d2f(dz), 0.0f);
}

// displacement of every gas slot of a reusing tube since its lists were
// recorded; a slot outside the grid marks its tube (re-sort)
//
// slot_pid (a step on bound host arrays): st holds the host's state in caller
// order and slot q of the recorded order holds particle slot_pid[q]; res is the
// resident state the lists were recorded on (slot order).  A particle whose h
// or Ind the host has changed makes its tube re-sort: the lists' cut-offs and
// membership assume both.
__global__ void k_list_disp(const TubeDesc *tubes, TubeState *ts, const Chunk *chunks, int nchunks, DevState st,
                            const uint32_t *skey, const float4 *pos_ref, float4 *disp, const int *force,
                            const int *slot_pid, DevState res) {
  if (*force) return;
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const Chunk ch = chunks[c];
    const int q = ch.begin + threadIdx.x;
    if (q >= ch.end) continue;
    const TubeDesc &T = tubes[ch.tube];
    if (!(T.skin > 0.0) || !ts[ch.tube].built) continue;
    const int j = slot_pid ? T.seg_begin[ch.species] + slot_pid[q] : q;
    if (slot_pid && (dbl_bits(st.h[j]) != dbl_bits(res.h[q]) || st.ind[j] != res.ind[q]))
      atomicMax(&ts[ch.tube].disp_bits, 0x7f800000u);  // +inf: re-sort
    const int local = (int)(skey[q] >> T.xl) - T.key_base[ch.species];
    float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
    if (local >= 0 && local < T.ncells) {
      const int ix = local % T.nx, iy = (local / T.nx) % T.ny, iz = local / (T.nx * T.ny);
      const float4 o = list_offset(T, ix, iy, iz, st.x[j], st.y[j], st.z[j]);
      const float4 r = pos_ref[q];
      d = make_float4(o.x - r.x, o.y - r.y, o.z - r.z, 0.0f);
    } else {
      atomicMax(&ts[ch.tube].disp_bits, 0x7f800000u);  // +inf: re-sort
    }
    disp[q] = d;
  }
}

// per gas cell of a reusing tube: mean displacement (xyz) and the largest
// distance of a displacement from it (w; -1 for an empty cell); per tube the
// largest of those distances and the box of the means
__global__ void k_list_cellstat(const TubeDesc *tubes, TubeState *ts, const int *nseg_key0, const int *nseg_tube,
                                const int *nseg_species, int nseg, int nkeys, const int *cell_start, int xl,
                                const float4 *disp, float4 *stat, const int *force) {
  if (*force) return;  // uniform over the grid
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  bool act = key < nkeys;
  int t = 0;
  if (act) {
    const int sg = find_seg(nseg_key0, nseg, key);
    t = nseg_tube[sg];
    act = nseg_species[sg] == 0 && tubes[t].skin > 0.0 && ts[t].built && key - tubes[t].key_base[0] < tubes[t].ncells;
  }
  float4 out = make_float4(0.f, 0.f, 0.f, -1.f);
  if (act) {
    const int a = cell_start[key << xl], b = cell_start[(key + 1) << xl];
    if (b > a) {
      float sx = 0.f, sy = 0.f, sz = 0.f;
      for (int j = a; j < b; j++) {
        const float4 d = disp[j];
        sx += d.x; sy += d.y; sz += d.z;
      }
      const float inv = 1.0f / (float)(b - a);
      const float mx = sx * inv, my = sy * inv, mz = sz * inv;
      float dev2 = 0.f;
      bool bad = !(fabsf(mx) <= 3.0e38f && fabsf(my) <= 3.0e38f && fabsf(mz) <= 3.0e38f);
      for (int j = a; j < b; j++) {
        const float4 d = disp[j];
        const float ex = d.x - mx, ey = d.y - my, ez = d.z - mz;
        const float e2 = ex * ex + ey * ey + ez * ez;
        bad |= !(e2 <= 3.0e38f);
        dev2 = fmaxf(dev2, e2);
      }
      out = make_float4(mx, my, mz, bad ? __int_as_float(0x7f800000) : sqrtf(dev2));
    }
    stat[key] = out;
  }
  const bool full = act && out.w >= 0.0f;
  TubeState *S = full ? ts + t : nullptr;
  warp_atomic_max(S ? &S->gdev_bits : nullptr, full ? __float_as_uint(out.w) : 0u);
  warp_atomic_min(S ? &S->mlo[0] : nullptr, full ? ord_bits(out.x) : 0xffffffffu);
  warp_atomic_min(S ? &S->mlo[1] : nullptr, full ? ord_bits(out.y) : 0xffffffffu);
  warp_atomic_min(S ? &S->mlo[2] : nullptr, full ? ord_bits(out.z) : 0xffffffffu);
  warp_atomic_max(S ? &S->mhi[0] : nullptr, full ? ord_bits(out.x) : 0u);
  warp_atomic_max(S ? &S->mhi[1] : nullptr, full ? ord_bits(out.y) : 0u);
  warp_atomic_max(S ? &S->mhi[2] : nullptr, full ? ord_bits(out.z) : 0u);
}

// (c + k) mod n for any offset k, n >= 1
__device__ __forceinline__ int wrap_index(int c, int n) {
  c %= n;
  return c < 0 ? c + n : c;
}

// per gas cell c of a reusing tube: the largest dev_c + dev_c' + |m_c - m_c'|
// over the non-empty cells c' within r_c + 1 cells (each unordered pair once:
// c' after c in the (z, y, x) order of the offsets), max-reduced per tube into
// disp_bits (a float >= 0 as bits; not finite -> +inf).  One warp per cell,
// its lanes over the offsets (the offsets after (0, 0, 0) in that order are
// the cube indices after its centre); the block's warps combine their maxima
// in shared memory for the tube of the block's first cell, so that the tube's
// one address takes one atomic per block, not one per cell.
#define DS_BOUND_WARPS 16
__global__ void __launch_bounds__(32 * DS_BOUND_WARPS)
    k_list_bound(const TubeDesc *tubes, TubeState *ts, const int *nseg_key0, const int *nseg_tube,
                 const int *nseg_species, int nseg, int nkeys, const unsigned char *krad, const float4 *stat,
                 const int *force) {
  if (*force) return;  // uniform over the grid
  const unsigned FULL = 0xffffffffu;
  __shared__ unsigned s_acc;
  __shared__ int s_tube, s_any;
  const int lane = (int)(threadIdx.x & 31);
  const int kfirst = (int)blockIdx.x * DS_BOUND_WARPS;
  const int key = kfirst + (int)(threadIdx.x >> 5);  // one per warp
  if (threadIdx.x == 0) {
    s_acc = 0u;
    s_any = 0;
    s_tube = nseg_tube[find_seg(nseg_key0, nseg, kfirst < nkeys ? kfirst : nkeys - 1)];
  }
  __syncthreads();
  bool act = key < nkeys;
  int t = 0;
  if (act) {
    const int sg = find_seg(nseg_key0, nseg, key);
    t = nseg_tube[sg];
    act = nseg_species[sg] == 0 && tubes[t].skin > 0.0 && ts[t].built && key - tubes[t].key_base[0] < tubes[t].ncells;
  }
  float m = 0.0f;
  bool bad = false;
  const float4 a = act ? stat[key] : make_float4(0.f, 0.f, 0.f, -1.f);
  act = act && a.w >= 0.0f;  // uniform over the warp
  if (act) {
    const TubeDesc &T = tubes[t];
    const int kb = T.key_base[0];
    const int local = key - kb;
    const int ix = local % T.nx, iy = (local / T.nx) % T.ny, iz = local / (T.nx * T.ny);
    int r = T.stencil == 1 ? 1 : (int)krad[key];
    r = (r < 1 ? 1 : (r > T.stencil ? T.stencil : r)) + 1;
    if (lane == 0) {
      m = 2.0f * a.w;  // two particles of the cell itself
      bad = !(a.w <= 3.0e38f);
    }
    // cube index idx = ((g + r) w + l + r) w + k + r; a lane starts at the
    // centre + 1 + lane and steps by 32, its (g, l, k) advanced with carries
    // (no division in the loop); |offsets| <= r < a periodic axis's cells, so
    // one wrap brings a periodic index back
    const int w = 2 * r + 1, n3 = w * w * w;
    int idx = n3 / 2 + 1 + lane;
    int k = idx % w - r, l = (idx / w) % w - r, g = idx / (w * w) - r;  // g >= 0 after the centre
    const int sk = 32 % w, sl = (32 / w) % w, sg = 32 / (w * w);
    for (; idx < n3; idx += 32) {
      int cz = iz + g, cy = iy + l;
      const int cx = ix + k;
      if (T.mode & M_PER_Z) cz += cz < 0 ? T.nz : (cz >= T.nz ? -T.nz : 0);
      if (T.mode & M_PER_Y) cy += cy < 0 ? T.ny : (cy >= T.ny ? -T.ny : 0);
      if (cz < T.nz && cy >= 0 && cy < T.ny && cx >= 0 && cx < T.nx) {
        const float4 b = stat[kb + cx + cy * T.sy + cz * T.sz];
        if (b.w >= 0.0f) {
          const float ex = a.x - b.x, ey = a.y - b.y, ez = a.z - b.z;
          const float bound = a.w + b.w + sqrtf(ex * ex + ey * ey + ez * ez);
          bad |= !(bound <= 3.0e38f);
          m = fmaxf(m, bound);
        }
      }
      k += sk;
      l += sl;
      g += sg;
      if (k > r) { k -= w; ++l; }
      if (l > r) { l -= w; ++g; }
    }
  }
  // m >= 0: its bits order as the floats do
  const unsigned mb = __reduce_max_sync(FULL, __float_as_uint(m));
  const unsigned v = __any_sync(FULL, bad) ? 0x7f800000u : mb;
  if (act && lane == 0) {
    if (t == s_tube) {
      atomicMax(&s_acc, v);
      atomicOr(&s_any, 1);
    } else {
      atomicMax(&ts[t].disp_bits, v);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_any) atomicMax(&ts[s_tube].disp_bits, s_acc);
}

// per tube: re-sort and record this step, or keep the lists; *any: some tube
// re-sorts (the sort and the cell tables run); *force: every tube re-sorts
// (the state was replaced or re-ordered since the last step), then cleared.
// Resets the tube's statistics for the next test.
__global__ void k_list_decide(const TubeDesc *tubes, TubeState *ts, int ntubes, int *force, int *any) {
  __shared__ int s_any;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  const int f = *force;
  for (int t = threadIdx.x; t < ntubes; t += blockDim.x) {
    const TubeDesc &T = tubes[t];
    TubeState &S = ts[t];
    int rb = 1;
    if (T.skin > 0.0 && !f && S.built) {
      const float skin = (float)T.skin;
      const float wmin = (float)fmin(T.wx, fmin(T.wy, T.wz));
      const float local = __uint_as_float(S.disp_bits);
      float far = 2.0f * __uint_as_float(S.gdev_bits);
      if (S.mhi[0] >= S.mlo[0]) {  // some cell has particles
        const float ex = ord_float(S.mhi[0]) - ord_float(S.mlo[0]);
        const float ey = ord_float(S.mhi[1]) - ord_float(S.mlo[1]);
        const float ez = ord_float(S.mhi[2]) - ord_float(S.mlo[2]);
        far += sqrtf(ex * ex + ey * ey + ez * ez);
      }
      rb = (local < 0.999f * skin && far < 0.999f * (skin + wmin)) ? 0 : 1;
    }
    S.rebuild = rb;
    S.disp_bits = 0u;
    S.gdev_bits = 0u;
    for (int a = 0; a < 3; a++) { S.mlo[a] = 0xffffffffu; S.mhi[a] = 0u; }
    if (rb) {
      S.built = T.skin > 0.0 ? 1 : 0;
      S.nrebuild++;
      s_any = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *any = s_any;
    *force = 0;
  }
}

// Split step: the density and pressure of listed gas particles (caller
// indices, slots through inv) set from outside between the two parts of a
// step, with what the density sweep derives from them for the force sweep --
// the same expressions as its epilogues (FP64: c_s, p / rho^2 and their FP32
// copies; FP32: the FP32 inputs, 1/h of the particle).
__global__ void k_set_hydro(const TubeDesc *tubes, int tube, int n, const int *idx, const double *val,
                            const int *inv, DevState st, double *cs64, double *pt64, float4 *hyd32,
                            const float4 *pos32, int fp32, int hpp) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const TubeDesc &T = tubes[tube];
  const int q = inv[T.seg_begin[0] + idx[k]];
  const double rho = val[k], p = val[n + k];
  st.rho[q] = rho;
  st.p[q] = p;
  if (fp32) {
    const float rhof = (float)rho, pf = (float)p;
    const float csf = sqrtf((float)T.gam * pf / rhof);
    const float hown = hpp ? pos32[q].w : (float)T.h;
    hyd32[q] = make_float4(csf, pf / (rhof * rhof), rhof, 1.0f / hown);
  } else {
    const double cs = sqrt(T.gam * p / rho);
    const double pt = p / (rho * rho);
    cs64[q] = cs;
    pt64[q] = pt;
    hyd32[q] = make_float4((float)cs, (float)pt, (float)rho, 0.0f);
  }
}

__global__ void k_fill(double *a, int n, double v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

__global__ void k_iota(int *a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers (ds_kernels.cuh)
// ---------------------------------------------------------------------------
static inline int blocks_for(int n, int b) { return (n + b - 1) / b; }

void ds_launch_step_begin(const TubeDesc *tubes, TubeState *ts, int ntubes, int *work, cudaStream_t s) {
  const int n = ntubes > DS_NSWEEP ? ntubes : DS_NSWEEP;
  k_step_begin<<<blocks_for(n, 64), 64, 0, s>>>(tubes, ts, ntubes, work);
}
void ds_launch_keys(const TubeDesc *tubes, const Chunk *chunks, int nchunks, DevState st, uint32_t *kin,
                    uint32_t *vin, bool fast, cudaStream_t s, const TubeState *reuse_ts, const uint32_t *prev_skey,
                    const int *slot_pid) {
  if (!nchunks) return;
  if (fast)
    k_keys<true><<<nchunks, DS_CHUNK, 0, s>>>(tubes, chunks, nchunks, st, kin, vin, reuse_ts, prev_skey, slot_pid);
  else
    k_keys<false><<<nchunks, DS_CHUNK, 0, s>>>(tubes, chunks, nchunks, st, kin, vin, nullptr, nullptr, nullptr);
}
void ds_launch_reorder(const TubeDesc *tubes, const Chunk *chunks, int nchunks, const uint32_t *order,
                       const uint32_t *skey, DevState src, DevState dst, float4 *pos32, float4 *vm32, int *idic_local,
                       uint32_t *ikin, uint32_t *ivin, int *slot_of_pid, int *ind_of_pid, int *flags, bool fast,
                       cudaStream_t s, const TubeState *reuse_ts, float4 *pos_ref, const int *slot_pid,
                       float4 *pm32) {
  if (!nchunks) return;
  if (fast)
    k_reorder<true><<<nchunks, DS_CHUNK, 0, s>>>(tubes, chunks, nchunks, order, skey, src, dst, pos32, vm32,
                                                 idic_local, ikin, ivin, slot_of_pid, ind_of_pid, flags, reuse_ts,
                                                 pos_ref, slot_pid, pm32);
  else
    k_reorder<false><<<nchunks, DS_CHUNK, 0, s>>>(tubes, chunks, nchunks, order, skey, src, dst, pos32, vm32,
                                                  idic_local, ikin, ivin, slot_of_pid, ind_of_pid, flags, nullptr,
                                                  nullptr, nullptr, nullptr);
}
void ds_launch_early_fp32(const TubeDesc *tubes, const Chunk *gas_chunks, int ngas_chunks, const TubeState *ts,
                          const uint32_t *skey, DevState cs, const int *slot_pid, float4 *pos32, float4 *pm32,
                          cudaStream_t s) {
  if (ngas_chunks)
    k_early_fp32<<<ngas_chunks, DS_CHUNK, 0, s>>>(tubes, gas_chunks, ngas_chunks, ts, skey, cs, slot_pid, pos32, pm32);
}
void ds_launch_cell_start(const uint32_t *skey, int n, int nkeys, int *cell_start, cudaStream_t s,
                          const int *run_if) {
  k_cell_start<<<blocks_for(n + 1, 256), 256, 0, s>>>(skey, n, nkeys, cell_start, run_if);
}
void ds_launch_list_test(const TubeDesc *tubes, TubeState *ts, int ntubes, const Chunk *gas_chunks,
                         int ngas_chunks, DevState st, const uint32_t *skey, const float4 *pos_ref, float4 *disp,
                         const int *nseg_key0, const int *nseg_tube, const int *nseg_species, int nseg, int nkeys,
                         const int *cell_start, int xl, const unsigned char *krad, float4 *cellstat, int *force,
                         int *any, cudaStream_t s, const int *slot_pid, DevState res) {
  if (ngas_chunks)
    k_list_disp<<<ngas_chunks, DS_CHUNK, 0, s>>>(tubes, ts, gas_chunks, ngas_chunks, st, skey, pos_ref, disp, force,
                                                 slot_pid, res);
  if (nkeys > 0) {
    const int b = blocks_for(nkeys, 128);
    k_list_cellstat<<<b, 128, 0, s>>>(tubes, ts, nseg_key0, nseg_tube, nseg_species, nseg, nkeys, cell_start, xl,
                                      disp, cellstat, force);
    k_list_bound<<<blocks_for(nkeys, DS_BOUND_WARPS), 32 * DS_BOUND_WARPS, 0, s>>>(
        tubes, ts, nseg_key0, nseg_tube, nseg_species, nseg, nkeys, krad, cellstat, force);
  }
  k_list_decide<<<1, 256, 0, s>>>(tubes, ts, ntubes, force, any);
}
void ds_launch_set_hydro(const TubeDesc *tubes, int tube, int n, const int *idx, const double *val, const int *inv,
                         DevState st, double *cs64, double *pt64, float4 *hyd32, const float4 *pos32, bool fp32,
                         bool hpp, cudaStream_t s) {
  if (n > 0)
    k_set_hydro<<<blocks_for(n, 256), 256, 0, s>>>(tubes, tube, n, idx, val, inv, st, cs64, pt64, hyd32, pos32,
                                                   fp32 ? 1 : 0, hpp ? 1 : 0);
}
void ds_launch_list_decide(const TubeDesc *tubes, TubeState *ts, int ntubes, int *force, int *any, cudaStream_t s) {
  k_list_decide<<<1, 256, 0, s>>>(tubes, ts, ntubes, force, any);
}
// FP32 path: lanes per IDIC key of the cell sums, 2, 4 or 8 (an autotuner
// choice; 4 measured fastest on the 720k tube)
template <int LANES>
static void launch_idic_split(const uint32_t *islot, int nikeys, const int *seg_key0, const int *seg_species,
                              const int *seg_orphan, int nseg, DevState st, CellArrays ca, cudaStream_t s) {
  k_idic_reduce_split<LANES><<<(int)(((long long)LANES * nikeys + 127) / 128), 128, 0, s>>>(
      islot, nikeys, seg_key0, seg_species, seg_orphan, nseg, st, ca);
}
void ds_launch_idic_reduce(const uint32_t *ikey, const uint32_t *islot, int n, int nikeys, const int *seg_key0,
                           const int *seg_species, const int *seg_orphan, int nseg, DevState st, CellArrays ca,
                           bool fast, cudaStream_t s, int lanes) {
  if (nikeys <= 0) return;
  k_cell_start<<<blocks_for(n + 1, 256), 256, 0, s>>>(ikey, n, nikeys, ca.start, nullptr);
  if (fast && lanes == 2)
    launch_idic_split<2>(islot, nikeys, seg_key0, seg_species, seg_orphan, nseg, st, ca, s);
  else if (fast && lanes == 8)
    launch_idic_split<8>(islot, nikeys, seg_key0, seg_species, seg_orphan, nseg, st, ca, s);
  else if (fast)
    launch_idic_split<4>(islot, nikeys, seg_key0, seg_species, seg_orphan, nseg, st, ca, s);
  else
    k_idic_reduce<<<blocks_for(nikeys, 128), 128, 0, s>>>(islot, nikeys, seg_key0, seg_species, seg_orphan, nseg,
                                                          st, ca);
}
void ds_launch_idic_solve(const TubeDesc *tubes, const TubeState *ts, const int *tube_cell0, int ntubes,
                          int ncell_total, CellArrays ca, bool fast, cudaStream_t s) {
  if (!ncell_total) return;
  if (fast)
    k_idic_solve<true><<<blocks_for(ncell_total, 128), 128, 0, s>>>(tubes, ts, tube_cell0, ntubes, ncell_total, ca);
  else
    k_idic_solve<false><<<blocks_for(ncell_total, 128), 128, 0, s>>>(tubes, ts, tube_cell0, ntubes, ncell_total, ca);
}
void ds_launch_relax_move(const TubeDesc *tubes, const TubeState *ts, const Chunk *chunks, int nchunks,
                          DevState st, const int *idic_local, const double *edot, CellArrays ca, int *flags,
                          bool fast, cudaStream_t s) {
  if (!nchunks) return;
  if (fast)
    k_relax_move<true><<<nchunks, DS_CHUNK, 0, s>>>(tubes, ts, chunks, nchunks, st, idic_local, edot, ca, flags);
  else
    k_relax_move<false><<<nchunks, DS_CHUNK, 0, s>>>(tubes, ts, chunks, nchunks, st, idic_local, edot, ca, flags);
}
void ds_launch_tstop(const TubeDesc *tubes, const TubeState *ts, const Chunk *chunks, int nchunks, DevState st,
                     const int *gas_slot_of_pid, int *flags, cudaStream_t s) {
  if (nchunks) k_tstop<<<nchunks, DS_CHUNK, 0, s>>>(tubes, ts, chunks, nchunks, st, gas_slot_of_pid, flags);
}
void ds_launch_dt(const TubeDesc *tubes, TubeState *ts, int ntubes, cudaStream_t s) {
  k_dt<<<blocks_for(ntubes, 64), 64, 0, s>>>(tubes, ts, ntubes);
}
void ds_launch_step_end(TubeState *ts, int ntubes, cudaStream_t s) {
  k_step_end<<<blocks_for(ntubes, 64), 64, 0, s>>>(ts, ntubes);
}
void ds_launch_conservation(const TubeDesc *tubes, int tube, DevState st, double *out, cudaStream_t s) {
  k_conservation<<<1, 256, 0, s>>>(tubes, tube, st, out);
}
void ds_launch_debug_lists(const TubeDesc *tubes, int tube, int species, int nseg_particles, int ncells,
                           DevState st, const int *cell_start, int xl, int *head, int *next, int *rawkey,
                           cudaStream_t s) {
  int n = nseg_particles > ncells + 1 ? nseg_particles : ncells + 1;
  k_debug_lists<<<blocks_for(n, 256), 256, 0, s>>>(tubes, tube, species, st, cell_start, xl, head, next, rawkey);
}
void ds_launch_origins(const TubeDesc &T, double *orig, cudaStream_t s) {
  const int n = T.nbx + T.ny + T.nz;
  if (n > 0) k_origins<<<blocks_for(n, 256), 256, 0, s>>>(T.ox, T.wx, T.nbx, T.oy, T.wy, T.ny, T.oz, T.wz, T.nz, orig);
}
void ds_launch_fill(double *a, int n, double v, cudaStream_t s) {
  if (n > 0) k_fill<<<blocks_for(n, 256), 256, 0, s>>>(a, n, v);
}
void ds_launch_iota(int *a, int n, cudaStream_t s) {
  if (n > 0) k_iota<<<blocks_for(n, 256), 256, 0, s>>>(a, n);
}
void ds_launch_cell_radius(const TubeDesc *tubes, const int *cell_start, int nkeys, int xl, const double *h,
                           double *wa, double *wb, const int *nseg_key0, const int *nseg_tube,
                           const int *nseg_species, int nseg, unsigned char *krad, cudaStream_t s,
                           const int *run_if) {
  if (nkeys <= 0) return;
  const int b = blocks_for(nkeys, 256);
  k_cell_hmax<<<b, 256, 0, s>>>(cell_start, nkeys, xl, h, wa, run_if);
  k_cell_window<0><<<b, 256, 0, s>>>(tubes, nseg_key0, nseg_tube, nseg_species, nseg, nkeys, wa, wb, krad, run_if);
  k_cell_window<1><<<b, 256, 0, s>>>(tubes, nseg_key0, nseg_tube, nseg_species, nseg, nkeys, wb, wa, krad, run_if);
  k_cell_window<2><<<b, 256, 0, s>>>(tubes, nseg_key0, nseg_tube, nseg_species, nseg, nkeys, wa, nullptr, krad,
                                     run_if);
}
