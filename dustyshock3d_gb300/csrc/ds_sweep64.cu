// ds_sweep64.cu -- FP64 neighbour sweeps in the reference's operation order.
//
// Compiled with -fmad=false.  For each particle the 27 neighbour cells are
// visited in the reference's launch order (k, l, g; kernel.cu:2014-2016,
// 2259-2262) and each cell's particles in ascending caller index (the sorted
// slots), so every sum is formed in the reference's order and the results
// equal the reference's CPU build bit for bit (the distance uses the correctly
// rounded sqrt where the reference writes pow(r^2, 0.5), IDIC.h:37, 219).
//
// Work split: one thread per particle, 128 particles of one segment per block
// (chunk table), cell ranges from cell_start[] of the sorted arrays.  Threads of
// a warp hold neighbouring particles of the same or adjacent cells, so they
// walk nearly the same neighbour slots in lockstep and the loads broadcast
// from L1.
//
// GB300's FP64 rate is ~1/64 of its FP32 rate, so each candidate is first
// screened in FP32 (packed float4 positions): a candidate whose FP32 distance
// exceeds the cut-off by more than the rounding bound cannot contribute
// (W = 0 beyond 2h; the force needs r < 2h) and is skipped; the FP64 test and
// arithmetic run only for the rest.  The screen never rejects a pair the FP64
// test accepts, so results are unchanged.
#include <cuda_runtime.h>

#include "ds_common.cuh"
#include "ds_kernels.cuh"

namespace {

// FP32 shift that brings a neighbour cell's coordinates into ours.
__device__ __forceinline__ void pre_shift(const TubeDesc &T, int o, double shy, double shz, float &sx, float &sy,
                                          float &sz) {
  if (T.cellrel) {
    const int k = o / 9 - 1, l = (o / 3) % 3 - 1, g = o % 3 - 1;
    sx = (float)(k * T.wx);
    sy = (float)(l * T.wy);
    sz = (float)(g * T.wz);
  } else {
    sx = 0.0f;
    sy = (float)shy;
    sz = (float)shz;
  }
}

__device__ __forceinline__ float pre_cut2(float two_h, float slack) {
  float r = two_h * 1.00001f + slack;
  return r * r;
}

// what: 0 gas density + EOS + derived quantities, 1 dust self-density.
template <bool HPP, int WHAT>
__global__ void __launch_bounds__(DS_CHUNK) k_density64(SweepArgs a) {
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    if (!a.tstate[ch.tube].active) continue;
    const TubeDesc &T = a.tubes[ch.tube];
    const int s = ch.species;
    const int ind = a.st.ind[i];
    const bool upd = ind == 0;
    bool zero = upd;
    if (WHAT == 1 && (T.mode & M_REF_COUPLING)) {
      // Rho_InitKernel_IDIC zeroes dust rho by the GAS Ind at the same index (IDIC.h:8)
      const int q = a.st.pid[i];
      const int ng = T.seg_end[0] - T.seg_begin[0];
      zero = q < ng && a.gas_ind_pid[T.seg_begin[0] + q] == 0;
    }
    double rho = a.st.rho[i];
    if (zero) rho = 0.0;
    if (upd) {
      const double xi = a.st.x[i], yi = a.st.y[i], zi = a.st.z[i];
      const double hi = HPP ? a.st.h[i] : T.h;
      const float4 pi = a.pos32[i];
      const float cut2 = pre_cut2(2.0f * (float)hi, T.pre_abs);
      Stencil S;
      ds_stencil_init(T, xi, yi, zi, S);
      const int kb = T.key_base[s];
      for (int o = 0; o < 27; o++) {
        double shy, shz;
        const int cell = ds_stencil_cell(T, S, o, shy, shz);
        if (cell < 0) continue;
        float sx, sy, sz;
        pre_shift(T, o, shy, shz, sx, sy, sz);
        const int j1 = a.cell_start[kb + cell + 1];
        double rho_tmp = 0.0;
        for (int j = a.cell_start[kb + cell]; j < j1; j++) {
          const float4 pj = a.pos32[j];
          const float fx = pj.x + sx - pi.x, fy = pj.y + sy - pi.y, fz = pj.z + sz - pi.z;
          if (fx * fx + fy * fy + fz * fz > cut2) continue;  // W = 0 there
          const double dx = a.st.x[j] - xi;
          const double dy = ds_diff(a.st.y[j], shy, yi);
          const double dz = ds_diff(a.st.z[j], shz, zi);
          const double d = sqrt(dx * dx + dy * dy + dz * dz);
          rho_tmp = rho_tmp + a.st.m[j] * ds_W(d, hi);
        }
        rho = rho + rho_tmp;
      }
    }
    if (zero || upd) a.st.rho[i] = rho;
    if (WHAT == 0) {
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
      a.hyd32[i] = make_float4((float)cs, (float)pt, (float)rho, 0.0f);
      if (upd && (T.mode & M_CFL)) {
        const double vx = a.st.vx[i], vy = a.st.vy[i], vz = a.st.vz[i];
        const double v = sqrt(vx * vx + vy * vy + vz * vz);
        const double hh = HPP ? a.st.h[i] : T.h;
        const double dt = hh / (cs + v);
        atomicMin(&a.tstate_rw[ch.tube].dtmin_bits, (unsigned long long)__double_as_longlong(dt));
      }
    }
  }
}

// ForceKernel_IDIC (IDIC.h:198-260): A_i and the energy rate, accumulated per
// neighbour in the reference's order from zero (Force_InitKernel_IDIC,
// EnergyInitKernel_IDIC).  COUNT_ONLY: the parity hook's candidate and
// in-range counts, for every particle, no physics.
template <bool HPP, bool COUNT_ONLY>
__global__ void __launch_bounds__(DS_CHUNK) k_force64(SweepArgs a) {
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    if (i >= ch.end) continue;
    if (!COUNT_ONLY) {
      if (!a.tstate[ch.tube].active) continue;
      if (a.st.ind[i] != 0) continue;
    }
    const TubeDesc &T = a.tubes[ch.tube];
    const int s = ch.species;
    const double xi = a.st.x[i], yi = a.st.y[i], zi = a.st.z[i];
    const double hi = HPP ? a.st.h[i] : T.h;
    const float4 pi = a.pos32[i];
    double vxi = 0, vyi = 0, vzi = 0, rhoi = 0, mi = 0, pti = 0, csi = 0, mpi = 0;
    if (!COUNT_ONLY) {
      vxi = a.st.vx[i]; vyi = a.st.vy[i]; vzi = a.st.vz[i];
      rhoi = a.st.rho[i]; mi = a.st.m[i];
      pti = a.pt64[i]; csi = a.cs64[i];
      mpi = mi * a.st.p[i] / (rhoi * rhoi);
    }
    const double Gam_g = T.gam, alpha = T.alpha, beta = T.beta, eps = T.eps;
    (void)Gam_g;
    double Ax = 0.0, Ay = 0.0, Az = 0.0, et = 0.0;
    int ncand = 0, nnb = 0;
    Stencil S;
    ds_stencil_init(T, xi, yi, zi, S);
    const int kb = T.key_base[s];
    const float hif = (float)hi;
    for (int o = 0; o < 27; o++) {
      double shy, shz;
      const int cell = ds_stencil_cell(T, S, o, shy, shz);
      if (cell < 0) continue;
      float sx, sy, sz;
      pre_shift(T, o, shy, shz, sx, sy, sz);
      const int j0 = a.cell_start[kb + cell], j1 = a.cell_start[kb + cell + 1];
      if (COUNT_ONLY) ncand += j1 - j0;
      for (int j = j0; j < j1; j++) {
        const float4 pj = a.pos32[j];
        const float fx = pj.x + sx - pi.x, fy = pj.y + sy - pi.y, fz = pj.z + sz - pi.z;
        const float hcf = HPP ? fmaxf(hif, pj.w) : hif;
        if (fx * fx + fy * fy + fz * fz > pre_cut2(2.0f * hcf, T.pre_abs)) continue;
        const double dxj = a.st.x[j] - xi;
        const double dyj = ds_diff(a.st.y[j], shy, yi);
        const double dzj = ds_diff(a.st.z[j], shz, zi);
        const double dist = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
        const double hj = HPP ? a.st.h[j] : hi;
        const double hcut = HPP ? (hi > hj ? hi : hj) : hi;
        if ((dist < 2 * hcut) && (dist > 0)) {
          if (COUNT_ONLY) {
            nnb++;
            continue;
          }
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
          const double dWr = HPP ? 0.5 * (ds_dW(dist, hi) + ds_dW(dist, hj)) : ds_dW(dist, hi);
          et = et + (mpi + mi * F_nu / 2.0) * (nu1x + nu1y + nu1z) * dWr / dist;
          const double A = a.st.m[j] * (pti + a.pt64[j] + F_nu) * dWr;
          Ax = Ax + dxj * A / dist;
          Ay = Ay + dyj * A / dist;
          Az = Az + dzj * A / dist;
        }
      }
    }
    if (COUNT_ONLY) {
      const int q = T.seg_begin[s] + a.st.pid[i];
      a.ncand[q] = ncand;
      a.nnb[q] = nnb;
    } else {
      a.st.ax[i] = Ax;
      a.st.ay[i] = Ay;
      a.st.az[i] = Az;
      a.edot[i] = et;
    }
  }
}

inline int grid_for(int nchunks) { return nchunks; }

}  // namespace

void ds_launch_density64(const SweepArgs &a, bool hpp, bool proper, int what, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (what == 0) {
    if (hpp) k_density64<true, 0><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
    else k_density64<false, 0><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
  } else {
    if (hpp) k_density64<true, 1><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
    else k_density64<false, 1><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
  }
}

void ds_launch_force64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (hpp) k_force64<true, false><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
  else k_force64<false, false><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
}

void ds_launch_counts64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s) {
  (void)proper;
  if (!a.nchunks) return;
  if (hpp) k_force64<true, true><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
  else k_force64<false, true><<<grid_for(a.nchunks), DS_CHUNK, 0, s>>>(a);
}
