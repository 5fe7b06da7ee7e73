// ds_sweep64.cu -- FP64 neighbour sweeps in the reference's operation order.
//
// Compiled with -fmad=false.  For each particle the neighbour cells are
// visited in the reference's launch order (k, l, g; kernel.cu:2014-2016,
// 2259-2262) and each cell's particles in ascending caller index (the sorted
// slots), so every sum is formed in the reference's order and the results
// equal the reference's CPU build bit for bit (the distance uses the correctly
// rounded sqrt where the reference writes pow(r^2, 0.5), IDIC.h:37, 219).
//
// Work split: one thread per particle, 128 particles of one segment per block
// (chunk table), cell ranges from cell_start[] of the sorted arrays.
//
// GB300 issues FP64 at ~1/64 of its FP32 rate.  Two things keep the FP64 work
// to the pairs that contribute:
//  * each candidate is first screened in FP32 (packed float4 positions); a
//    candidate whose FP32 distance exceeds the cut-off by more than the
//    rounding bound cannot contribute (W = 0 beyond 2h, the force needs
//    r < 2h) and is dropped; the screen never drops a pair the FP64 test
//    accepts, so results are unchanged;
//  * survivors go to a per-thread list in shared memory (ds_walk) and the
//    FP64 work runs over the lists, so a warp's lanes all do pair work
//    together instead of idling while one lane meets a neighbour.
// With 125-cell stencils (cells of half the width) a particle whose cut-off
// fits the 27 inner cells walks only those: the outer cells hold no partner
// within the cut-off, so the sums are unchanged.
#include <cuda_runtime.h>

#include "ds_common.cuh"
#include "ds_kernels.cuh"

namespace {

__device__ __forceinline__ float pre_cut2(float two_h, float slack) {
  float r = two_h * 1.00001f + slack;
  return r * r;
}

// what: 0 gas density + EOS + per-particle force inputs, 1 dust self-density.
template <bool HPP, int WHAT>
// FP64 pair work is heavy, so the lists are longer: flushes are rarer and the
// lanes' lists are fuller when they run.
#define DS_LIST_CAP64 64

__global__ void __launch_bounds__(DS_SWEEP_THREADS) k_density64(SweepArgs a) {
  __shared__ uint32_t lst[DS_LIST_CAP64 * DS_SWEEP_THREADS];
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    const bool valid = i < ch.end && (a.all_tubes || a.tstate[ch.tube].active);
    const TubeDesc &T = a.tubes[ch.tube];
    const int s = ch.species;
    const int ind = valid ? a.st.ind[i] : 1;
    const bool upd = valid && ind == 0;
    bool zero = upd;
    if (valid && WHAT == 1 && (T.mode & M_REF_COUPLING)) {
      // Rho_InitKernel_IDIC zeroes dust rho by the GAS Ind at the same index (IDIC.h:8)
      const int q = a.st.pid[i];
      const int ng = T.seg_end[0] - T.seg_begin[0];
      zero = q < ng && a.gas_ind_pid[T.seg_begin[0] + q] == 0;
    }
    double rho = valid ? a.st.rho[i] : 0.0;
    if (zero) rho = 0.0;
    const double xi = upd ? a.st.x[i] : 0.0, yi = upd ? a.st.y[i] : 0.0, zi = upd ? a.st.z[i] : 0.0;
    const double hi = upd ? (HPP ? a.st.h[i] : T.h) : T.h;
    const float4 pi = upd ? a.pos32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float cut2 = pre_cut2(2.0f * (float)hi, T.pre_abs);
    Stencil S;
    ds_stencil_init(T, xi, yi, zi, S);
    const int r = hi <= T.r1_hmax ? 1 : T.stencil;
    double rho_tmp = 0.0;
    int cur_o = -1;
    const double wn = ds_W_norm(hi);
    ds_walk<DS_LIST_CAP64>(
        T, S, upd, r, T.key_base[s], T.seg_begin[s], a.cell_start, pi, lst + threadIdx.x,
        [&](int j, float ox, float oy, float oz) {
          const float4 pj = a.pos32[j];
          const float fx = pj.x + ox, fy = pj.y + oy, fz = pj.z + oz;
          return fx * fx + fy * fy + fz * fz <= cut2;  // beyond: W = 0
        },
        [&](int j, int o5) {
          // one partial sum per neighbour cell, added as the reference does
          if (o5 != cur_o) {
            rho = rho + rho_tmp;
            rho_tmp = 0.0;
            cur_o = o5;
          }
          int k, l, g;
          ds_decode_ofs(o5, k, l, g);
          double shy, shz;
          ds_wrap_shift(T, S, l, g, shy, shz);
          const double dx = a.st.x[j] - xi;
          const double dy = ds_diff(a.st.y[j], shy, yi);
          const double dz = ds_diff(a.st.z[j], shz, zi);
          const double d = sqrt(dx * dx + dy * dy + dz * dz);
          rho_tmp = rho_tmp + a.st.m[j] * ds_W_n(d, hi, wn);
        });
    rho = rho + rho_tmp;
    unsigned long long dtb = ~0ull;  // CFL bound as double bits (positive doubles order as unsigned)
    if (valid && (zero || upd)) a.st.rho[i] = rho;
    if (valid && WHAT == 0) {
      // PKernel (kernel.cu:107-123) and per-particle quantities of the force sweep
      double p = a.st.p[i];
      if (upd) {
        p = ds_eq_state(rho, a.st.e[i], T.type_of_state, T.gam, T.cs);
        a.st.p[i] = p;
      }
      const double cs = sqrt(T.gam * p / rho);
      const double pt = p / (rho * rho);
      a.cs64[i] = cs;
      a.pt64[i] = pt;
      a.dwn64[i] = ds_dW_norm(HPP ? a.st.h[i] : T.h);
      a.hyd32[i] = make_float4((float)cs, (float)pt, (float)rho, 0.0f);
      if (upd && (T.mode & M_CFL)) {
        const double vx = a.st.vx[i], vy = a.st.vy[i], vz = a.st.vz[i];
        const double v = sqrt(vx * vx + vy * vy + vz * vz);
        const double hh = HPP ? a.st.h[i] : T.h;
        const double dt = hh / (cs + v);
        dtb = (unsigned long long)__double_as_longlong(dt);
      }
    }
    // one atomic per warp on the tube's CFL minimum (a warp's lanes share a tube)
    for (int k = 16; k > 0; k >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, dtb, k);
      dtb = o < dtb ? o : dtb;
    }
    if (WHAT == 0 && (threadIdx.x & 31) == 0 && dtb != ~0ull) atomicMin(&a.tstate_rw[ch.tube].dtmin_bits, dtb);
  }
}

// ForceKernel_IDIC (IDIC.h:198-260): A_i and the energy rate, accumulated per
// neighbour in the reference's order from zero (Force_InitKernel_IDIC,
// EnergyInitKernel_IDIC).
template <bool HPP>
__global__ void __launch_bounds__(DS_SWEEP_THREADS) k_force64(SweepArgs a) {
  __shared__ uint32_t lst[DS_LIST_CAP64 * DS_SWEEP_THREADS];
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    const TubeDesc &T = a.tubes[ch.tube];
    const bool act = i < ch.end && a.tstate[ch.tube].active && a.st.ind[i] == 0;
    const int s = ch.species;
    const double xi = act ? a.st.x[i] : 0.0, yi = act ? a.st.y[i] : 0.0, zi = act ? a.st.z[i] : 0.0;
    const double hi = act ? (HPP ? a.st.h[i] : T.h) : T.h;
    const float4 pi = act ? a.pos32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const double vxi = act ? a.st.vx[i] : 0.0, vyi = act ? a.st.vy[i] : 0.0, vzi = act ? a.st.vz[i] : 0.0;
    const double rhoi = act ? a.st.rho[i] : 1.0, mi = act ? a.st.m[i] : 0.0;
    const double pti = act ? a.pt64[i] : 0.0, csi = act ? a.cs64[i] : 0.0;
    const double mpi = mi * (act ? a.st.p[i] : 0.0) / (rhoi * rhoi);
    const double alpha = T.alpha, beta = T.beta, eps = T.eps;
    double Ax = 0.0, Ay = 0.0, Az = 0.0, et = 0.0;
    Stencil S;
    ds_stencil_init(T, xi, yi, zi, S);
    const int r = (T.stencil == 1 || !act) ? 1 : (int)a.krad[a.skey[i]];
    const float hif = (float)hi;
    const double dni = act ? a.dwn64[i] : 0.0;
    ds_walk<DS_LIST_CAP64>(
        T, S, act, r, T.key_base[s], T.seg_begin[s], a.cell_start, pi, lst + threadIdx.x,
        [&](int j, float ox, float oy, float oz) {
          const float4 pj = a.pos32[j];
          const float fx = pj.x + ox, fy = pj.y + oy, fz = pj.z + oz;
          const float hcf = HPP ? fmaxf(hif, pj.w) : hif;
          return fx * fx + fy * fy + fz * fz <= pre_cut2(2.0f * hcf, T.pre_abs);
        },
        [&](int j, int o5) {
          int k, l, g;
          ds_decode_ofs(o5, k, l, g);
          double shy, shz;
          ds_wrap_shift(T, S, l, g, shy, shz);
          const double dxj = a.st.x[j] - xi;
          const double dyj = ds_diff(a.st.y[j], shy, yi);
          const double dzj = ds_diff(a.st.z[j], shz, zi);
          const double dist = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
          const double hj = HPP ? a.st.h[j] : hi;
          const double hcut = HPP ? (hi > hj ? hi : hj) : hi;
          if (!((dist < 2 * hcut) && (dist > 0))) return;
          // x_i - x_j with the neighbour's image shift
          const double xij = xi - a.st.x[j];
          const double yij = shy != 0.0 ? yi - (a.st.y[j] + shy) : yi - a.st.y[j];
          const double zij = shz != 0.0 ? zi - (a.st.z[j] + shz) : zi - a.st.z[j];
          const double hh = HPP ? 0.5 * (hi + hj) : hi;
          const double rhoj = a.st.rho[j];
          double F_nu = 0;
          const double nu1x = (vxi - a.st.vx[j]) * xij;
          const double nu1y = (vyi - a.st.vy[j]) * yij;
          const double nu1z = (vzi - a.st.vz[j]) * zij;
          double nu_temp = nu1x + nu1y + nu1z;
          if (nu_temp < 0.0) {
            const double Cnu = 0.5 * (csi + a.cs64[j]);
            nu_temp = hh * nu_temp / (dist * dist + eps * hh * hh);
            F_nu = (-alpha * Cnu * nu_temp + beta * nu_temp * nu_temp) / (0.5 * (rhoi + rhoj));
          }
          const double dWr =
              HPP ? 0.5 * (ds_dW_n(dist, hi, dni) + ds_dW_n(dist, hj, a.dwn64[j])) : ds_dW_n(dist, hi, dni);
          et = et + (mpi + mi * F_nu / 2.0) * (nu1x + nu1y + nu1z) * dWr / dist;
          const double A = a.st.m[j] * (pti + a.pt64[j] + F_nu) * dWr;
          Ax = Ax + dxj * A / dist;
          Ay = Ay + dyj * A / dist;
          Az = Az + dzj * A / dist;
        });
    if (!act) continue;
    a.st.ax[i] = Ax;
    a.st.ay[i] = Ay;
    a.st.az[i] = Az;
    a.edot[i] = et;
  }
}

// Parity hook: candidates over the full stencil and those with 0 < r < 2h
// (IDIC.h:219-220), for every particle, no physics.
template <bool HPP>
__global__ void __launch_bounds__(DS_SWEEP_THREADS) k_counts64(SweepArgs a) {
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    const TubeDesc &T = a.tubes[ch.tube];
    const int s = ch.species;
    const double xi = a.st.x[i], yi = a.st.y[i], zi = a.st.z[i];
    const double hi = HPP ? a.st.h[i] : T.h;
    Stencil S;
    ds_stencil_init(T, xi, yi, zi, S);
    const int r = T.stencil;
    const int nofs = (2 * r + 1) * (2 * r + 1) * (2 * r + 1);
    const int kb = T.key_base[s];
    int ncand = 0, nnb = 0;
    for (int o = 0; o < nofs; o++) {
      double shy, shz;
      int k, l, g;
      const int cell = ds_stencil_cell(T, S, r, o, shy, shz, k, l, g);
      if (cell < 0) continue;
      const int j0 = a.cell_start[kb + cell], j1 = a.cell_start[kb + cell + 1];
      ncand += j1 - j0;
      for (int j = j0; j < j1; j++) {
        const double dxj = a.st.x[j] - xi;
        const double dyj = ds_diff(a.st.y[j], shy, yi);
        const double dzj = ds_diff(a.st.z[j], shz, zi);
        const double dist = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
        const double hj = HPP ? a.st.h[j] : hi;
        const double hcut = HPP ? (hi > hj ? hi : hj) : hi;
        if ((dist < 2 * hcut) && (dist > 0)) nnb++;
      }
    }
    const int q = T.seg_begin[s] + a.st.pid[i];
    a.ncand[q] = ncand;
    a.nnb[q] = nnb;
  }
}

}  // namespace

void ds_launch_density64(const SweepArgs &a, bool hpp, bool proper, int what, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (what == 0) {
    if (hpp) k_density64<true, 0><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
    else k_density64<false, 0><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
  } else {
    if (hpp) k_density64<true, 1><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
    else k_density64<false, 1><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
  }
}

void ds_launch_force64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (hpp) k_force64<true><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
  else k_force64<false><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
}

void ds_launch_counts64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (hpp) k_counts64<true><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
  else k_counts64<false><<<a.nchunks, DS_SWEEP_THREADS, 0, s>>>(a);
}
