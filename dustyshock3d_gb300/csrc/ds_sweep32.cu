// ds_sweep32.cu -- FP32 neighbour sweeps with Kahan-compensated sums.
//
// Same traversal as ds_sweep64.cu (stencil cells in the reference's order,
// one thread per particle, screened candidates listed in shared memory), but every per-pair quantity is FP32: positions are FP32
// offsets from the particle's own cell origin (proper grid; a neighbour cell's
// offsets are shifted by whole cell widths, which also applies the periodic
// image), velocities/masses come from packed float4 copies, and each sum is
// Kahan-compensated.  The kernel normalisation 1/(pi h^3) is applied once per
// particle in FP64.  State, the IDIC exchange and the conservation sums stay
// FP64 (ds_cells.cu).  GB300 issues FP32 at ~64x its FP64 rate, which is what
// this path is for; its error against the FP64 path is measured, not assumed.
#include <cuda_runtime.h>

#include "ds_common.cuh"
#include "ds_kernels.cuh"

namespace {

struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// This file is compiled without multiply-add contraction (-fmad=false): every
// fused multiply-add below is written out (__fmaf_rn), so that the same pair
// gives the same bits in every kernel that evaluates it (the recording walk and
// the streamed lists, the force walk and the force lists), whatever registers
// and schedule each kernel gets.

// M4 shape without normalisation, q = r/h >= 0 (kernel.cu:18-20):
// 1 - 1.5 q^2 + 0.75 q^3 = 1 + q^2 (0.75 q - 1.5), and 0.25 (2 - q)^3
__device__ __forceinline__ float w_shape(float q) {
  if (q < 1.0f) return __fmaf_rn(q * q, __fmaf_rn(0.75f, q, -1.5f), 1.0f);
  if (q <= 2.0f) {
    const float t = 2.0f - q;
    return (0.25f * t) * (t * t);
  }
  return 0.0f;
}

// derivative shape, q >= 0 (kernel.cu:34-36): -3 q + 2.25 q^2 = q (2.25 q - 3),
// and -0.75 (2 - q)^2
__device__ __forceinline__ float dw_shape(float q) {
  if (q <= 1.0f) return q * __fmaf_rn(2.25f, q, -3.0f);
  if (q <= 2.0f) {
    const float t = 2.0f - q;
    return -0.75f * (t * t);
  }
  return 0.0f;
}

// Squared distance with explicit roundings (no contraction chosen by the
// compiler), so the density sweep's screen, the force sweep's screen and the
// pair work all see the same value for the same pair.
__device__ __forceinline__ float r2_of(float dx, float dy, float dz) {
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// After the density sum of particle i: the density (kernel normalisation in
// FP64), the EOS, and the force sweep's FP32 inputs.  Returns the particle's
// CFL bound h / (c_s + |v|) as FP32 bits, or ~0u when it has none.
template <bool HPP, int WHAT>
__device__ __forceinline__ unsigned density_epilogue(const SweepArgs &a, const TubeDesc &T, const Chunk &ch, int i,
                                                     bool upd, bool zero, double rho, double hd, float hf,
                                                     const Kahan &sum) {
  unsigned dtb = ~0u;
  if (upd) rho = rho + (((double)1 / (DS_PI_REF)) / (hd * hd * hd)) * sum.value();
  if (zero || upd) a.st.rho[i] = rho;
  if (WHAT == 0) {
    double p = a.st.p[i];
    if (upd) {
      p = ds_eq_state(rho, a.st.e[i], T.type_of_state, T.gam, T.cs);
      a.st.p[i] = p;
    }
    // force inputs and the CFL bound in FP32 (the force sweep is FP32)
    const float rhof = (float)rho, pf = (float)p;
    const float csf = sqrtf((float)T.gam * pf / rhof);
    // .w: 1/h of the particle (frozen ones too: they are force partners)
    const float hown = HPP ? a.pos32[i].w : (float)T.h;
    a.hyd32[i] = make_float4(csf, pf / (rhof * rhof), rhof, 1.0f / hown);
    if (upd && (T.mode & M_CFL)) {
      const float vx = (float)a.st.vx[i], vy = (float)a.st.vy[i], vz = (float)a.st.vz[i];
      const float dt = hf / (csf + sqrtf(vx * vx + vy * vy + vz * vz));
      dtb = __float_as_uint(dt);
    }
  }
  return dtb;
}

// The CFL minimum of a tube: the smallest bound of the warp's particles (FP32
// bits: positive floats order as unsigned, NaN and negative values above
// them), then one atomic per warp, as a double -- the value a per-particle
// atomic would leave, with 1/32 of the atomics on the tube's one address
// (per-particle atomics there serialised and took a large part of the sweep).
// Every lane of the warp calls it (a warp's lanes share their chunk's tube).
__device__ __forceinline__ void cfl_min_warp(const SweepArgs &a, int tube, unsigned dtb) {
  const unsigned m = __reduce_min_sync(0xffffffffu, dtb);
  if ((threadIdx.x & 31) == 0 && m != ~0u)
    atomicMin(&a.tstate_rw[tube].dtmin_bits, (unsigned long long)__double_as_longlong((double)__uint_as_float(m)));
}

// The chunks a block takes: blockIdx.x, then every gridDim.x-th (one block per
// chunk), or, with a work counter (a persistent grid), the next unclaimed one
// each time, so that blocks that finish early take more.  Every thread of the
// block calls it once per chunk (it holds two block barriers).
__device__ __forceinline__ int claim_chunk(int *work, int *claim) {
  __syncthreads();  // the previous claim is read by every thread
  if (threadIdx.x == 0) *claim = atomicAdd(work, 1);
  __syncthreads();
  return *claim;
}
__device__ __forceinline__ int first_chunk(const SweepArgs &a, int *claim) {
  return a.work ? claim_chunk(a.work, claim) : (int)blockIdx.x;
}
__device__ __forceinline__ int next_chunk(const SweepArgs &a, int c, int *claim) {
  return a.work ? claim_chunk(a.work, claim) : c + (int)gridDim.x;
}

// The 4 warp flags of a chunk as one word (nbl_walk is 4-byte aligned per chunk).
__device__ __forceinline__ uint32_t chunk_walk_flags(const SweepArgs &a, int c) {
  return *reinterpret_cast<const uint32_t *>(a.nbl_walk + (size_t)c * (DS_SWEEP_THREADS / 32));
}

// LIST: the gas density sweep also records the force sweep's neighbours.  It
// then walks the force sweep's stencil and screens with its cut-off
// 2 max(h_i, h_j) (a superset of its own 2 h_i: the density adds only pairs
// within 2 h_i, so its sum is unchanged), and writes every candidate that
// passes (the particle itself too, which the force sweep's screen r > 0
// drops) -- the pairs the force sweep's own walk would accept, in its visiting
// order.  A warp with a particle beyond nbl_cap entries is flagged (one flag
// per warp, no block barrier); the force sweep walks that warp's particles.
// With list reuse (a.reuse) the recorded cut-off is 2 max(h_i, h_j) + skin,
// and a tube that keeps its lists this step (TubeState::rebuild 0) neither
// walks nor records here: k_density32_lst streams its lists, and only its
// flagged warps walk (with its last re-sort's cells, which the skin covers),
// recording nothing.
#ifndef DS_DENS_LIST_MINB
#define DS_DENS_LIST_MINB 6  // blocks per SM the list-recording density sweep is built for
#endif
template <bool HPP, int WHAT, int CAP, bool LIST>
__global__ void __launch_bounds__(DS_SWEEP_THREADS, LIST ? DS_DENS_LIST_MINB : (WHAT ? 9 : 8)) k_density32(SweepArgs a) {
  __shared__ uint32_t lst[CAP * DS_SWEEP_THREADS];
  __shared__ float4 shtab[DS_NOFS32];
  __shared__ int claim;
  for (int c = first_chunk(a, &claim); c < a.nchunks; c = next_chunk(a, c, &claim)) {
    const Chunk ch = a.chunks[c];
    const bool record = !LIST || !a.reuse || a.tstate[ch.tube].rebuild;
    if (LIST && !record && chunk_walk_flags(a, c) == 0u) continue;  // uniform per block: the lists serve it
    const bool mine = record || a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)];
    const int i = ch.begin + threadIdx.x;
    const bool valid = mine && i < ch.end && (a.all_tubes || a.tstate[ch.tube].active);
    const TubeDesc &T = a.tubes[ch.tube];
    __syncthreads();  // the previous chunk's table is no longer read
    ds_fill_shift_table32(T, shtab);
    __syncthreads();
    const int s = ch.species;
    const int ind = valid ? a.st.ind[i] : 1;
    const bool upd = valid && ind == 0;
    bool zero = upd;
    if (valid && WHAT == 1 && (T.mode & M_REF_COUPLING)) {
      const int q = a.st.pid[i];
      const int ng = T.seg_end[0] - T.seg_begin[0];
      zero = q < ng && a.gas_ind_pid[T.seg_begin[0] + q] == 0;
    }
    double rho = valid ? a.st.rho[i] : 0.0;
    if (zero) rho = 0.0;
    const double hd = upd ? (HPP ? a.st.h[i] : T.h) : T.h;
    const float4 pi = upd ? a.pos32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float hf = (float)hd, inv_h = 1.0f / hf, cut2 = 4.0f * hf * hf;
    const float skin = LIST ? (float)T.skin : 0.0f;
    Stencil S{0, 0, 0, 0};
    const int own = upd ? (int)(a.skey[i] >> T.xl) : 0;  // own cell key
    if (upd) ds_stencil_from_key(T, own - T.key_base[s], a.st.x[i], a.st.y[i], a.st.z[i], S);
    const int r = LIST ? ((T.stencil == 1 || !upd) ? 1 : (int)a.krad[own]) : ds_radius(T, 2.0 * hd);
    // x reach of the partners: r cells (every partner lies within them) or 2 h
    const float cutx = LIST ? (float)r * (float)T.wx : 2.0f * hf;
    const int sb = T.seg_begin[s];
    uint32_t *nl = LIST ? a.nbl + (size_t)c * a.nbl_cap * DS_SWEEP_THREADS + threadIdx.x : nullptr;
    int cnt = 0;
    Kahan sum;
    ds_walk_rows<CAP>(
        T, S, upd, r, T.key_base[s], sb, a.cell_start, pi, cutx, shtab, lst + threadIdx.x,
        [&](int j, float ox, float oy, float oz) {
          const float4 pj = a.pos32[j];
          const float r2 = r2_of(pj.x + ox, pj.y + oy, pj.z + oz);
          if (LIST) {
            const float rc = 2.0f * (HPP ? fmaxf(hf, pj.w) : hf) + skin;
            return r2 < rc * rc;
          }
          return r2 < cut2;
        },
        [&](int j, int o5) {
          const float4 sh = shtab[o5];
          const float4 pj = a.pos32[j];
          const float r2 = r2_of(pj.x + (sh.x - pi.x), pj.y + (sh.y - pi.y), pj.z + (sh.z - pi.z));
          if (!LIST || r2 < cut2) {
            const float q = r2 > 0.0f ? r2 * rsqrtf(r2) * inv_h : 0.0f;
            sum.add(a.vm32[j].w * w_shape(q));
          }
          if (LIST && record) {
            if (cnt < a.nbl_cap)
              nl[(size_t)cnt * DS_SWEEP_THREADS] = ((uint32_t)o5 << DS_OFS32_SHIFT) | (uint32_t)(j - sb);
            cnt++;
          }
        });
    if (LIST && record) {
      const unsigned over = __ballot_sync(0xffffffffu, cnt > a.nbl_cap);
      if ((threadIdx.x & 31) == 0) a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)] = over != 0u;
      if (i < ch.end) a.nbl_cnt[i] = cnt;
    }
    const unsigned dtb = valid ? density_epilogue<HPP, WHAT>(a, T, ch, i, upd, zero, rho, hd, hf, sum) : ~0u;
    if (WHAT == 0) cfl_min_warp(a, ch.tube, dtb);
  }
}

// The gas density of a tube that keeps its lists this step: its recorded
// entries (the particle itself among them) in the recording walk's order, each
// added when within 2 h_i now -- the pairs and the order a walk of the same
// cells would take, so the sum equals the walk's bit for bit; no walk, no
// screen of candidates.  Warps flagged as overflowed are left to the walk
// (k_density32), tubes that re-sort to the recording walk.
#ifndef DS_DPIECE
#define DS_DPIECE 4  // list entries per pipeline stage of the density stream (measured: 4 beats 2 and 8;
                     // a piece-ahead prefetch as in the force list sweep measured 2 % slower here)
#endif
//
// MODE 0: the whole sweep (sums, then density, EOS, force inputs, CFL bound).
// MODE 1 and 2 split it for a step on bound host arrays, so that the sums run
// while the host's other fields are still on their way: MODE 1 (before the
// reorder) reads a slot's own Ind and h from the host's state in caller order
// (cs; slot i holds particle slot_pid[i]) and the FP32 copies of the early
// pass, and stores each slot's Kahan pair in dsum; MODE 2 (after the reorder)
// finishes from dsum exactly as MODE 0 does after its loop.
template <bool HPP, int MODE>
__global__ void __launch_bounds__(DS_SWEEP_THREADS)
    k_density32_lst(SweepArgs a, DevState cs, const int *slot_pid, float2 *dsum) {
  const unsigned FULL = 0xffffffffu;
  __shared__ float4 shtab[DS_NOFS32];
  __shared__ int claim;
  for (int c = first_chunk(a, &claim); c < a.nchunks; c = next_chunk(a, c, &claim)) {
    const Chunk ch = a.chunks[c];
    if (a.tstate[ch.tube].rebuild || chunk_walk_flags(a, c) == 0x01010101u) continue;  // uniform per block
    const int i = ch.begin + threadIdx.x;
    const TubeDesc &T = a.tubes[ch.tube];
    __syncthreads();
    ds_fill_shift_table32(T, shtab);
    __syncthreads();
    const int sb = T.seg_begin[ch.species];
    const bool listed = !a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)];
    const bool valid = listed && i < ch.end && (a.all_tubes || a.tstate[ch.tube].active);
    const int jo = (MODE == 1 && valid) ? sb + slot_pid[i] : i;  // the slot's own particle in cs
    const bool upd = valid && (MODE == 1 ? cs.ind[jo] : a.st.ind[i]) == 0;
    double rho = 0.0;
    if (MODE != 1) {
      rho = valid ? a.st.rho[i] : 0.0;
      if (upd) rho = 0.0;
    }
    const double hd = upd ? (HPP ? (MODE == 1 ? cs.h[jo] : a.st.h[i]) : T.h) : T.h;
    const float4 pi = upd ? a.pos32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float hf = (float)hd, inv_h = 1.0f / hf, cut2 = 4.0f * hf * hf;
    Kahan sum;
    if (MODE == 2) {
      if (upd) {
        const float2 k = dsum[i];
        sum.s = k.x;
        sum.c = k.y;
      }
    } else {
      const int cnt = upd ? a.nbl_cnt[i] : 0;
      const int cnt_w = __reduce_max_sync(FULL, cnt);
      const uint32_t *nl = a.nbl + (size_t)c * a.nbl_cap * DS_SWEEP_THREADS + threadIdx.x;
      uint32_t ent[DS_DPIECE];
#pragma unroll
      for (int t = 0; t < DS_DPIECE; t++) ent[t] = t < cnt ? __ldcs(nl + (size_t)t * DS_SWEEP_THREADS) : 0u;
      for (int e = 0; e < cnt_w; e += DS_DPIECE) {
        float4 pj[DS_DPIECE];
        float mj[DS_DPIECE];
#pragma unroll
        for (int t = 0; t < DS_DPIECE; t++)
          if (e + t < cnt) {
            const int j = sb + (int)(ent[t] & DS_SLOT32_MASK);
            if (a.pm32) {  // coordinates and mass in one 16-byte record (measured: 0.496 -> 0.482 ms per step)
              pj[t] = a.pm32[j];
              mj[t] = pj[t].w;
            } else {
              pj[t] = a.pos32[j];
              mj[t] = a.vm32[j].w;
            }
          }
        uint32_t nxt[DS_DPIECE];
#pragma unroll
        for (int t = 0; t < DS_DPIECE; t++) {
          const int q = e + DS_DPIECE + t;
          nxt[t] = q < cnt ? __ldcs(nl + (size_t)q * DS_SWEEP_THREADS) : 0u;
        }
#pragma unroll
        for (int t = 0; t < DS_DPIECE; t++)
          if (e + t < cnt) {
            const float4 sh = shtab[ent[t] >> DS_OFS32_SHIFT];
            const float r2 = r2_of(pj[t].x + (sh.x - pi.x), pj[t].y + (sh.y - pi.y), pj[t].z + (sh.z - pi.z));
            if (r2 < cut2) {
              const float q = r2 > 0.0f ? r2 * rsqrtf(r2) * inv_h : 0.0f;
              sum.add(mj[t] * w_shape(q));
            }
          }
#pragma unroll
        for (int t = 0; t < DS_DPIECE; t++) ent[t] = nxt[t];
      }
    }
    if (MODE == 1) {
      if (valid) dsum[i] = make_float2(sum.s, sum.c);
      continue;
    }
    const unsigned dtb = valid ? density_epilogue<HPP, 0>(a, T, ch, i, upd, upd, rho, hd, hf, sum) : ~0u;
    cfl_min_warp(a, ch.tube, dtb);
  }
}

// Per-particle state and pair work of the force sweep (ForceKernel_IDIC,
// IDIC.h:198-260, in FP32 with Kahan sums).
template <bool HPP>
struct ForceSum {
  float4 pi, vmi;
  float hi, inv_hi, ni, mi, rhoi, pti, csi, mpi, alpha, beta, eps;
  Kahan Ax, Ay, Az, et;

  __device__ __forceinline__ ForceSum(const SweepArgs &a, const TubeDesc &T, int i, bool act) {
    pi = act ? a.pos32[i] : make_float4(0.f, 0.f, 0.f, 1.f);
    vmi = act ? a.vm32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 hyi = act ? a.hyd32[i] : make_float4(0.f, 0.f, 1.f, 1.f);
    hi = HPP ? pi.w : (float)T.h;
    inv_hi = hyi.w;
    ni = (float)(1.0 / 3.14159265) * inv_hi * inv_hi * inv_hi * inv_hi;
    mi = vmi.w;
    rhoi = hyi.z;
    pti = hyi.y;
    csi = hyi.x;
    mpi = mi * pti;  // m_i p_i / rho_i^2
    alpha = (float)T.alpha;
    beta = (float)T.beta;
    eps = (float)T.eps;
  }

  // the force sweep's screen: 0 < r < 2 max(h_i, h_j)
  __device__ __forceinline__ bool screen(const float4 &pj, float ox, float oy, float oz) const {
    const float r2 = r2_of(pj.x + ox, pj.y + oy, pj.z + oz);
    const float hc = HPP ? fmaxf(hi, pj.w) : hi;
    return (r2 < 4.0f * hc * hc) && (r2 > 0.0f);
  }

  // sh: the FP32 shift of the entry's cell (shift table), as the screen saw it
  __device__ __forceinline__ void pair(const SweepArgs &a, const float4 &sh, int j) {
    pair(sh, a.pos32[j], a.vm32[j], a.hyd32[j]);
  }

  // the same with the neighbour's pos32, vm32, hyd32 already loaded
  __device__ __forceinline__ void pair(const float4 &sh, const float4 &pj, const float4 &vmj, const float4 &hyj) {
    const float dx = pj.x + (sh.x - pi.x), dy = pj.y + (sh.y - pi.y), dz = pj.z + (sh.z - pi.z);
    const float r2 = r2_of(dx, dy, dz);
    const float inv_d = rsqrtf(r2);
    const float dist = r2 * inv_d;
    const float hh = HPP ? 0.5f * (hi + pj.w) : hi;
    const float nu = __fmaf_rn(vmi.z - vmj.z, -dz, __fmaf_rn(vmi.y - vmj.y, -dy, (vmi.x - vmj.x) * (-dx)));
    float F = 0.0f;
    if (nu < 0.0f) {
      const float Cnu = 0.5f * (csi + hyj.x);
      const float mu = __fdividef(hh * nu, __fmaf_rn(eps * hh, hh, r2));
      F = __fdividef(__fmaf_rn(beta * mu, mu, (-alpha * Cnu) * mu), 0.5f * (rhoi + hyj.z));
    }
    float dWr = ni * dw_shape(dist * inv_hi);
    if (HPP) {
      const float inv_hj = hyj.w;
      const float nj = (float)(1.0 / 3.14159265) * inv_hj * inv_hj * inv_hj * inv_hj;
      dWr = 0.5f * __fmaf_rn(nj, dw_shape(dist * inv_hj), dWr);
    }
    const float gd = dWr * inv_d;
    et.add((__fmaf_rn(mi * F, 0.5f, mpi) * nu) * gd);
    const float A = vmj.w * (pti + hyj.y + F) * gd;
    Ax.add(dx * A);
    Ay.add(dy * A);
    Az.add(dz * A);
  }

  __device__ __forceinline__ void store(const SweepArgs &a, int i) const {
    a.st.ax[i] = Ax.value();
    a.st.ay[i] = Ay.value();
    a.st.az[i] = Az.value();
    a.edot[i] = et.value();
  }
};

// Force sweep by walking the stencil.  With recorded lists it runs only the
// warps flagged as overflowed.
template <bool HPP, int CAP>
__global__ void __launch_bounds__(DS_SWEEP_THREADS) k_force32(SweepArgs a) {
  __shared__ uint32_t lst[CAP * DS_SWEEP_THREADS];
  __shared__ float4 shtab[DS_NOFS32];
  __shared__ int claim;
  for (int c = first_chunk(a, &claim); c < a.nchunks; c = next_chunk(a, c, &claim)) {
    if (a.nbl && chunk_walk_flags(a, c) == 0u) continue;  // uniform per block
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    const TubeDesc &T = a.tubes[ch.tube];
    __syncthreads();
    ds_fill_shift_table32(T, shtab);
    __syncthreads();
    const bool mine = !a.nbl || a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)];
    const bool act = mine && i < ch.end && a.tstate[ch.tube].active && a.st.ind[i] == 0;
    const int s = ch.species;
    ForceSum<HPP> F(a, T, i, act);
    Stencil S{0, 0, 0, 0};
    const int own = act ? (int)(a.skey[i] >> T.xl) : 0;  // own cell key
    if (act) ds_stencil_from_key(T, own - T.key_base[s], a.st.x[i], a.st.y[i], a.st.z[i], S);
    const int r = (T.stencil == 1 || !act) ? 1 : (int)a.krad[own];
    ds_walk_rows<CAP>(
        T, S, act, r, T.key_base[s], T.seg_begin[s], a.cell_start, F.pi, (float)r * (float)T.wx, shtab,
        lst + threadIdx.x,
        [&](int j, float ox, float oy, float oz) { return F.screen(a.pos32[j], ox, oy, oz); },
        [&](int j, int o5) { F.pair(a, shtab[o5], j); });
    if (act) F.store(a, i);
  }
}

// Force sweep over the recorded lists: no cell walk; entries in the walk's
// order, each tested against its exact cut-off, so the sums equal the walk's.
// Measured on the 720k tube: the one-entry-deep prefetch took the force phase
// from 0.548 to 0.478 ms per step with a 0.15 h skin (0.468 -> 0.421 ms
// without), against the earlier two-entry pieces whose partner data loaded
// only at the top of each piece; with it the kernel runs best unconstrained
// (93 registers, 5 blocks per SM) -- built for 7 or 8 blocks per SM it spills
// and measured 0.497 and 0.529 ms.
template <bool HPP>
__global__ void __launch_bounds__(DS_SWEEP_THREADS) k_force32_list(SweepArgs a) {
  const unsigned FULL = 0xffffffffu;
  __shared__ float4 shtab[DS_NOFS32];
  __shared__ int claim;
  for (int c = first_chunk(a, &claim); c < a.nchunks; c = next_chunk(a, c, &claim)) {
    if (chunk_walk_flags(a, c) == 0x01010101u) continue;  // every warp walks instead; uniform per block
    const Chunk ch = a.chunks[c];
    const int i = ch.begin + threadIdx.x;
    const TubeDesc &T = a.tubes[ch.tube];
    __syncthreads();
    ds_fill_shift_table32(T, shtab);
    __syncthreads();
    const bool listed = !a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)];
    const bool act = listed && i < ch.end && a.tstate[ch.tube].active && a.st.ind[i] == 0;
    const int sb = T.seg_begin[ch.species];
    ForceSum<HPP> F(a, T, i, act);
    const int cnt = act ? a.nbl_cnt[i] : 0;
    const int cnt_w = __reduce_max_sync(FULL, cnt);
    const uint32_t *nl = a.nbl + (size_t)c * a.nbl_cap * DS_SWEEP_THREADS + threadIdx.x;
    // software pipeline, one entry deep: while entry e's pair work runs, the
    // partner data of entry e + 1 and the index of entry e + 2 are in flight
    // (pairs still summed in list order)
    {
      uint32_t e0 = 0u < (unsigned)cnt ? __ldcs(nl) : 0u;
      uint32_t e1 = 1 < cnt ? __ldcs(nl + DS_SWEEP_THREADS) : 0u;
      float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), v0 = p0, y0 = p0;
      if (0 < cnt) {
        const int j = sb + (int)(e0 & DS_SLOT32_MASK);
        p0 = a.pos32[j];
        v0 = a.vm32[j];
        y0 = a.hyd32[j];
      }
      for (int e = 0; e < cnt_w; e++) {
        float4 p1 = p0, v1 = v0, y1 = y0;
        if (e + 1 < cnt) {
          const int j = sb + (int)(e1 & DS_SLOT32_MASK);
          p1 = a.pos32[j];
          v1 = a.vm32[j];
          y1 = a.hyd32[j];
        }
        const uint32_t e2 = e + 2 < cnt ? __ldcs(nl + (size_t)(e + 2) * DS_SWEEP_THREADS) : 0u;
        if (e < cnt) {
          const float4 sh = shtab[e0 >> DS_OFS32_SHIFT];
          if (F.screen(p0, sh.x - F.pi.x, sh.y - F.pi.y, sh.z - F.pi.z)) F.pair(sh, p0, v0, y0);
        }
        e0 = e1;
        e1 = e2;
        p0 = p1;
        v0 = v1;
        y0 = y1;
      }
    }
    if (act) F.store(a, i);
  }
}

// Parity hook: the recorded force lists of one tube's gas, by caller index.
// count[i]: entries recorded for particle i, or -1 when its warp walks (an
// entry beyond the lists' capacity); nbr[i * cap + k]: the caller index of its
// k-th entry (k < min(count[i], cap)).
__global__ void k_debug_force_lists(SweepArgs a, int tube, int cap, int *count, int *nbr) {
  __shared__ int claim;
  for (int c = first_chunk(a, &claim); c < a.nchunks; c = next_chunk(a, c, &claim)) {
    const Chunk ch = a.chunks[c];
    const int q = ch.begin + threadIdx.x;
    if (ch.tube != tube || q >= ch.end) continue;
    const int pi = a.st.pid[q];
    if (a.nbl_walk[c * (DS_SWEEP_THREADS / 32) + (threadIdx.x >> 5)]) {
      count[pi] = -1;
      continue;
    }
    const int n = a.nbl_cnt[q];
    count[pi] = n;
    const int sb = a.tubes[ch.tube].seg_begin[ch.species];
    const uint32_t *nl = a.nbl + (size_t)c * a.nbl_cap * DS_SWEEP_THREADS + threadIdx.x;
    for (int e = 0; e < n && e < cap && e < a.nbl_cap; e++)
      nbr[(size_t)pi * cap + e] = a.st.pid[sb + (int)(nl[(size_t)e * DS_SWEEP_THREADS] & DS_SLOT32_MASK)];
  }
}

}  // namespace

// One sweep launch: one block per chunk, or (with work counters) a
// persistent grid of nsm x bps[k] blocks claiming chunks from counter k.
template <class Kernel, class... Extra>
static void launch_sweep(Kernel kern, const SweepArgs &a, int k, cudaStream_t s, Extra... extra) {
  SweepArgs b = a;
  int n = a.nchunks;
  if (b.work) {
    b.work += k;
    const long long g = (long long)(a.bps[k] > 0 ? a.bps[k] : 1) * (a.nsm > 0 ? a.nsm : 1);
    n = (int)(g < n ? g : n);
  }
  kern<<<n, DS_SWEEP_THREADS, 0, s>>>(b, extra...);
}

template <int CAP>
static void launch_density32(const SweepArgs &a, bool hpp, int what, cudaStream_t s) {
  if (what == 0 && a.nbl) {
    if (hpp) launch_sweep(k_density32<true, 0, CAP, true>, a, DS_SW_DENSITY, s);
    else launch_sweep(k_density32<false, 0, CAP, true>, a, DS_SW_DENSITY, s);
  } else if (what == 0) {
    if (hpp) launch_sweep(k_density32<true, 0, CAP, false>, a, DS_SW_DENSITY, s);
    else launch_sweep(k_density32<false, 0, CAP, false>, a, DS_SW_DENSITY, s);
  } else {
    if (hpp) launch_sweep(k_density32<true, 1, CAP, false>, a, DS_SW_DUST_DENSITY, s);
    else launch_sweep(k_density32<false, 1, CAP, false>, a, DS_SW_DUST_DENSITY, s);
  }
}

template <class Kernel>
static int fit(Kernel kern) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, DS_SWEEP_THREADS, 0) != cudaSuccess) b = 1;
  return b < 1 ? 1 : b;
}

template <int CAP>
static void fit_all(bool hpp, bool list, int *bps) {
  if (hpp) {
    bps[DS_SW_DENSITY] = list ? fit(k_density32<true, 0, CAP, true>) : fit(k_density32<true, 0, CAP, false>);
    bps[DS_SW_DENSITY_LST] = fit(k_density32_lst<true, 0>);
    bps[DS_SW_DUST_DENSITY] = fit(k_density32<true, 1, CAP, false>);
    bps[DS_SW_FORCE_LIST] = fit(k_force32_list<true>);
    bps[DS_SW_FORCE_WALK] = fit(k_force32<true, CAP>);
  } else {
    bps[DS_SW_DENSITY] = list ? fit(k_density32<false, 0, CAP, true>) : fit(k_density32<false, 0, CAP, false>);
    bps[DS_SW_DENSITY_LST] = fit(k_density32_lst<false, 0>);
    bps[DS_SW_DUST_DENSITY] = fit(k_density32<false, 1, CAP, false>);
    bps[DS_SW_FORCE_LIST] = fit(k_force32_list<false>);
    bps[DS_SW_FORCE_WALK] = fit(k_force32<false, CAP>);
  }
}

void ds_sweep32_blocks_per_sm(bool hpp, int depth, bool list, int *bps) {
  if (depth >= 64) fit_all<64>(hpp, list, bps);
  else fit_all<32>(hpp, list, bps);
}

void ds_launch_density32(const SweepArgs &a, bool hpp, int what, int depth, cudaStream_t s) {
  if (!a.nchunks) return;
  if (depth >= 64) launch_density32<64>(a, hpp, what, s);
  else launch_density32<32>(a, hpp, what, s);
}

void ds_launch_density32_lst(const SweepArgs &a, bool hpp, cudaStream_t s) {
  if (!a.nchunks || !a.nbl || !a.reuse) return;
  const DevState none{};
  if (hpp) launch_sweep(k_density32_lst<true, 0>, a, DS_SW_DENSITY_LST, s, none, nullptr, nullptr);
  else launch_sweep(k_density32_lst<false, 0>, a, DS_SW_DENSITY_LST, s, none, nullptr, nullptr);
}

// The same split for a step on bound host arrays: the sums before the
// reorder (cs: the host's state in caller order, slot i holding particle
// slot_pid[i]), the rest after it.  One block per chunk.
void ds_launch_density32_lst_sums(const SweepArgs &a, bool hpp, DevState cs, const int *slot_pid, float2 *dsum,
                                  cudaStream_t s) {
  if (!a.nchunks || !a.nbl || !a.reuse) return;
  SweepArgs b = a;
  b.work = nullptr;
  if (hpp) k_density32_lst<true, 1><<<b.nchunks, DS_SWEEP_THREADS, 0, s>>>(b, cs, slot_pid, dsum);
  else k_density32_lst<false, 1><<<b.nchunks, DS_SWEEP_THREADS, 0, s>>>(b, cs, slot_pid, dsum);
}
void ds_launch_density32_lst_finish(const SweepArgs &a, bool hpp, float2 *dsum, cudaStream_t s) {
  if (!a.nchunks || !a.nbl || !a.reuse) return;
  SweepArgs b = a;
  b.work = nullptr;
  const DevState none{};
  if (hpp) k_density32_lst<true, 2><<<b.nchunks, DS_SWEEP_THREADS, 0, s>>>(b, none, nullptr, dsum);
  else k_density32_lst<false, 2><<<b.nchunks, DS_SWEEP_THREADS, 0, s>>>(b, none, nullptr, dsum);
}

void ds_launch_debug_force_lists(const SweepArgs &a, int tube, int cap, int *count, int *nbr, cudaStream_t s) {
  if (!a.nchunks || !a.nbl) return;
  SweepArgs b = a;
  b.work = nullptr;  // one block per chunk
  k_debug_force_lists<<<b.nchunks, DS_SWEEP_THREADS, 0, s>>>(b, tube, cap, count, nbr);
}

// With recorded lists: the list kernel, then the walk over overflowed chunks.
void ds_launch_force32(const SweepArgs &a, bool hpp, int depth, cudaStream_t s) {
  ds_launch_force32_list(a, hpp, s);
  ds_launch_force32_walk(a, hpp, depth, s);
}

// The list kernel alone (no-op without recorded lists).
void ds_launch_force32_list(const SweepArgs &a, bool hpp, cudaStream_t s) {
  if (!a.nchunks || !a.nbl) return;
  if (hpp) launch_sweep(k_force32_list<true>, a, DS_SW_FORCE_LIST, s);
  else launch_sweep(k_force32_list<false>, a, DS_SW_FORCE_LIST, s);
}

// The walk: every particle without recorded lists, else only the warps the
// density sweep flagged as overflowed (disjoint from the list kernel's, so the
// two may run concurrently).
void ds_launch_force32_walk(const SweepArgs &a, bool hpp, int depth, cudaStream_t s) {
  if (!a.nchunks) return;
  if (depth >= 64) {
    if (hpp) launch_sweep(k_force32<true, 64>, a, DS_SW_FORCE_WALK, s);
    else launch_sweep(k_force32<false, 64>, a, DS_SW_FORCE_WALK, s);
  } else {
    if (hpp) launch_sweep(k_force32<true, 32>, a, DS_SW_FORCE_WALK, s);
    else launch_sweep(k_force32<false, 32>, a, DS_SW_FORCE_WALK, s);
  }
}
