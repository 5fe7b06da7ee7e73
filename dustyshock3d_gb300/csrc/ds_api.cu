// ds_api.cu -- the C ABI (include/dustyshock3d_gb300.h): contexts, resident
// device state, the step sequence and its CUDA graphs.
//
// The reference runs each step as ~120 launches with a device sync after each
// and ~35 blocking copies (kernel.cu:1929-2566), building cell lists and doing
// the IDIC cell algebra on the host.  Here one step is ~25 launches on one
// stream with no host work and no copies; the sequence is captured once into a
// CUDA graph per buffer parity and replayed.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // driver types only (CUcontext, CUresult); libcuda is not linked
#include <cuda_runtime.h>

#include "../../include/dustyshock3d_gb300.h"
#include "ds_common.cuh"
#include "ds_ic.cuh"
#include "ds_inittxt.cuh"
#include "ds_kernels.cuh"
#include "ds_sort.cuh"

#define DS_VERSION "dustyshock3d_gb300 1.0 (sm_103a)"

namespace {

struct HostSpecies {
  int n = -1;
  std::vector<double> f[15];  // x y z vx vy vz ax ay az rho p e m h ts
  std::vector<int> ind;
  std::shared_ptr<IcPlan> gen;  // generated on the device instead (ds_init_tube)
};

enum { FX, FY, FZ, FVX, FVY, FVZ, FAX, FAY, FAZ, FRHO, FP, FE, FM, FH, FTS, NF };

// Host arrays bound to one species for ds_step_host: device addresses of
// mapped host arrays (nullptr: field not bound), read by the kernels at run
// time, so rebinding needs no new graph.
struct BoundSeg {
  double *f[NF];
  int *ind;
  int bound;     // 0: the segment is carried over from the resident state
  int out_mask;  // fields written back after the step (bit f)
};

struct Buffers {
  double *f[NF] = {};
  int *ind = nullptr, *pid = nullptr;
  DevState view() const {
    DevState s;
    s.x = f[FX]; s.y = f[FY]; s.z = f[FZ]; s.vx = f[FVX]; s.vy = f[FVY]; s.vz = f[FVZ];
    s.ax = f[FAX]; s.ay = f[FAY]; s.az = f[FAZ]; s.rho = f[FRHO]; s.p = f[FP]; s.e = f[FE];
    s.m = f[FM]; s.h = f[FH]; s.ts = f[FTS]; s.ind = ind; s.pid = pid;
    return s;
  }
};

}  // namespace

struct ds_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int ntubes = 0;
  std::vector<ds_params> params;
  std::vector<std::vector<HostSpecies>> host;  // [tube][species]
  std::vector<std::pair<ds_ctx *, int>> dev_src;  // per tube: resident tube to copy from (ds_copy_tube)
  std::vector<std::pair<bool, std::pair<double, long long>>> clock_set;  // per tube: clock to start from
  bool finalized = false;
  std::string msg;
  // sizes
  int N = 0;
  int nkeys = 0, key_bits = 0, nikeys = 0, ikey_bits = 0, ncell_total = 0, nseg = 0, nnseg = 0;
  int xl = 0;  // FP32 path: sub-cell x bits below the cell in the sort keys
  int last_xl = 0;  // x bits of the keys of the last sort (0 after an exact-order sort)
  std::vector<TubeDesc> tdesc;
  std::vector<Chunk> ch_all, ch_gas, ch_dust;
  // device
  std::vector<void *> allocs;
  long long bytes = 0;
  Buffers buf[2];
  int parity = 0;
  TubeDesc *d_tubes = nullptr;
  TubeState *d_tstate = nullptr;
  Chunk *d_ch_all = nullptr, *d_ch_gas = nullptr, *d_ch_dust = nullptr;
  int *d_seg_key0 = nullptr, *d_seg_species = nullptr, *d_seg_orphan = nullptr, *d_tube_cell0 = nullptr;
  int *d_nseg_key0 = nullptr, *d_nseg_tube = nullptr, *d_nseg_species = nullptr;
  double *cwa = nullptr, *cwb = nullptr;  // stencil-radius passes (h maxima per key)
  unsigned char *krad = nullptr;
  double *origins = nullptr;  // FP32 path: TubeDesc::orig of every tube
  const uint32_t *skey = nullptr;  // sorted neighbour keys of the current order
  bool any_stencil2 = false;
  float4 *pos32 = nullptr, *vm32 = nullptr, *hyd32 = nullptr;
  float4 *pm32 = nullptr;  // with list reuse: coordinates and mass in one record (the density stream)
  float2 *dsum = nullptr;  // with list reuse: a bound step's early density sums (Kahan pairs)
  bool dens_split = false;  // set while a bound step with list reuse is enqueued
  double *cs64 = nullptr, *pt64 = nullptr, *dwn64 = nullptr, *edot = nullptr;
  uint32_t *nbl = nullptr;  // FP32 force neighbour lists, nbl_cap entries per gas slot of each chunk
  int *nbl_cnt = nullptr;
  unsigned char *nbl_walk = nullptr;
  int nbl_cap = 0;
  // list reuse (some tube with a skin): FP32 offsets at each tube's last
  // re-sort, displacements, per-key statistics, and the device flags of the
  // start-of-step test (force: every tube re-sorts; any: some tube re-sorts)
  bool reuse = false;
  float4 *pos_ref = nullptr, *disp = nullptr, *cellstat = nullptr;
  // split step (ds_step_density .. ds_step_complete): 1 between the parts;
  // ialt: the IDIC key sort's result is in the alternate buffers
  int split = 0;
  bool ialt = false;
  // persistent FP32 sweeps (ds_params.persistent of tube 0): work counters,
  // SMs, blocks per SM of each sweep
  bool persistent = false;
  int *d_work = nullptr;
  int nsm = 0;
  int bps[DS_NSWEEP] = {0};
  int idic_lanes = 4;     // FP32 path: threads per IDIC key in the cell sums
  int *hy_idx = nullptr;       // ds_set_gas_hydro: caller indices, rho, p on the device
  double *hy_val = nullptr;
  int hy_cap = 0;
  int *d_force = nullptr, *d_any = nullptr;
  uint32_t *kin = nullptr, *vin = nullptr, *kalt = nullptr, *valt = nullptr;
  uint32_t *ikin = nullptr, *ivin = nullptr, *ikalt = nullptr, *ivalt = nullptr;
  uint32_t *rs_scratch = nullptr;
  int *slot_of_pid = nullptr, *ind_of_pid = nullptr, *idic_local = nullptr, *cell_start = nullptr;
  int *ncand = nullptr, *nnb = nullptr, *dbg_head = nullptr, *dbg_next = nullptr, *dbg_key = nullptr;
  double *stage = nullptr;  // N doubles, download/upload staging
  double *d_cons = nullptr;
  int *d_flags = nullptr;
  CellArrays ca{};
  bool any_hpp = false, any_proper = false, any_dust_rho = false, any_fp32 = false;
  // graphs
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  // host arrays bound to the step (ds_bind_host / ds_step_host)
  std::vector<BoundSeg> hbound;  // [tube * DS_MAXS + species]
  BoundSeg *d_bound = nullptr;
  int *inv = nullptr;            // slot of each particle (absolute), all segments
  bool any_bound = false;
  cudaStream_t stream2 = nullptr;
  // FP32 path with force lists: the overflow walk of the force sweep runs on
  // its own stream beside the list kernel (they write disjoint particles)
  cudaStream_t wstream = nullptr;
  cudaEvent_t e_wfork = nullptr, e_wjoin = nullptr;
  cudaEvent_t e_fork = nullptr, e_up = nullptr, e_dens = nullptr, e_force = nullptr, e_join = nullptr;
  cudaGraphExec_t hgraph[2] = {nullptr, nullptr};
  int side_blocks = 0;  // grid of the transfers overlapped with the step
  // timing
  cudaEvent_t ev[DS_NPHASE + 1] = {};
  std::vector<cudaEvent_t> tev;
};

static_assert(DS_CHUNK == DS_SWEEP_THREADS, "one sweep thread per particle of a chunk");

#ifndef DS_XL_MAX
#define DS_XL_MAX 4  // x bins per cell on the FP32 path: at most 2^DS_XL_MAX (measured: 16 bins beat 8, 32, 64)
#endif

namespace {

ds_status fail(ds_ctx *c, ds_status st, const std::string &m) {
  if (c) c->msg = m;
  return st;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(c, e_ == cudaErrorMemoryAllocation ? DS_ERR_NOMEM : DS_ERR_CUDA,            \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                        \
  } while (0)

template <class T> ds_status dalloc(ds_ctx *c, T **p, size_t count) {
  size_t bytes = sizeof(T) * (count ? count : 1);
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return fail(c, DS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back(q);
  c->bytes += (long long)bytes;
  *p = (T *)q;
  return DS_OK;
}

// Temporary device buffers of one call, freed when the call returns, on an
// early error return too (cudaFree waits for the device).
struct ScratchDev {
  std::vector<void *> held;
  ~ScratchDev() {
    for (void *q : held) cudaFree(q);
  }
  template <class T> cudaError_t alloc(T **out, size_t count) {
    const cudaError_t e = cudaMalloc((void **)out, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) held.push_back(*out);
    return e;
  }
};

#define DA(ptr, count)                         \
  do {                                         \
    ds_status s_ = dalloc(c, &(ptr), (count)); \
    if (s_ != DS_OK) return s_;                \
  } while (0)

int bits_for(long long n) {
  int b = 1;
  while ((1LL << b) < n) b++;
  return b;
}

// FP32 path index maps (TubeDesc::kxa ...) for the tube's x bits xl: scaling
// by 2^xl is exact, so the fine x index's top bits are the x cell.
void set_index_maps(TubeDesc &T) {
  T.kxa = std::ldexp(T.inv_wx, T.xl); T.kxb = -T.ox * T.kxa;
  T.kya = T.inv_wy; T.kyb = -T.oy * T.inv_wy;
  T.kza = T.inv_wz; T.kzb = -T.oz * T.inv_wz;
  T.iaa = T.inv_aw;
  T.iab[0] = -T.ox * T.inv_aw; T.iab[1] = -T.oy * T.inv_aw; T.iab[2] = -T.oz * T.inv_aw;
  T.wrap_key[0] = ds_order_key(T.oy); T.wrap_key[1] = ds_order_key(T.ymax);
  T.wrap_key[2] = ds_order_key(T.oz); T.wrap_key[3] = ds_order_key(T.zmax);
}

// Tube constants from its parameters; grid sizes follow kernel.cu:1767-1778
// and kernel.cu:1577-1582 with the same arithmetic.
void build_desc(const ds_params &P, TubeDesc &T) {
  memset(&T, 0, sizeof(T));
  T.mode = P.mode;
  T.ox = P.X_min; T.oy = P.Y_min; T.oz = P.Z_min;
  const bool proper = (P.mode & DS_MODE_GRID_PROPER) != 0;
  // list reuse (FP32 path with force lists): record 2 max(h_i, h_j) + skin and
  // widen the cells by the skin, so that every cell's walk keeps its radius
  // (a cut-off c within r cells of width w: c + skin within r cells of w + skin)
  const bool reuse = P.list_skin > 0 && P.precision == DS_PRECISION_FP32 && P.force_list != -1 && proper &&
                     !(P.mode & DS_MODE_DUST_RHO);
  T.skin = reuse ? P.list_skin * P.h : 0.0;
  const double w = (P.cell_w > 0 ? P.cell_w : 2.0 * P.h) + T.skin;
  T.Cnx = (int)((P.X_max - P.X_min) / w);
  T.Cny = (int)((P.Y_max - P.Y_min) / w);
  T.Cnz = (int)((P.Z_max - P.Z_min) / w);
  T.Ly = P.Y_max - P.Y_min;
  T.Lz = P.Z_max - P.Z_min;
  T.ymax = P.Y_max; T.zmax = P.Z_max;
  T.wx = T.wy = T.wz = w;
  if (!proper) {
    T.sy = T.Cnx;
    T.sz = T.Cnx * T.Cny;
    T.ncells = (T.Cnx + 1) * (T.Cny + 1) * (T.Cnz + 1);
    T.nx = T.Cnx + 1; T.ny = T.Cny + 1; T.nz = T.Cnz + 1;
  } else {
    T.nx = T.Cnx + 1;
    T.ny = (P.mode & DS_MODE_PERIODIC_Y) ? (int)(T.Ly / w) : T.Cny + 1;
    T.nz = (P.mode & DS_MODE_PERIODIC_Z) ? (int)(T.Lz / w) : T.Cnz + 1;
    if (T.ny < 1) T.ny = 1;
    if (T.nz < 1) T.nz = 1;
    if (P.mode & DS_MODE_PERIODIC_Y) T.wy = T.Ly / T.ny;
    if (P.mode & DS_MODE_PERIODIC_Z) T.wz = T.Lz / T.nz;
    T.sy = T.nx;
    T.sz = T.nx * T.ny;
    T.ncells = T.nx * T.ny * T.nz;
  }
  T.aw = P.idic_w > 0 ? P.idic_w : P.Coeff_h_dust_cell * P.h;
  T.Nax = (int)((P.X_max - P.X_min) / T.aw);
  T.Nay = (int)((P.Y_max - P.Y_min) / T.aw);
  T.Naz = (int)((P.Z_max - P.Z_min) / T.aw);
  T.n_idic = (T.Nax + 1) * (T.Nay + 1) * (T.Naz + 1);
  T.anx = T.Nax + 1; T.any_ = T.Nay + 1; T.anz = T.Naz + 1;
  if (P.mode & DS_MODE_IDIC_PROPER) {
    T.asy = T.anx;
    T.asz = T.anx * T.any_;
  } else {
    T.asy = T.Nax;
    T.asz = T.Nax * T.Nay;
  }
  T.h = P.h; T.alpha = P.alpha; T.beta = P.beta; T.eps = P.eps; T.gam = P.Gam_g;
  T.cs = P.Speed_of_sound_gas; T.tau = P.tau; T.cfl = P.cfl; T.t_end = P.T_end; T.t_empty = P.t_empty;
  T.type_of_state = P.Type_of_state; T.n_dust = P.n_dust; T.precision = P.precision;
  for (int k = 0; k < DS_MAXD; k++) {
    T.mass_ratio[k] = P.mass_ratio[k]; T.R_dust[k] = P.R_dust[k];
    T.t_stop_const[k] = P.t_stop_const[k]; T.eps_empty[k] = P.eps_empty[k];
  }
  T.fx = 0.5 * (P.X_min + P.X_max);
  T.fy = 0.5 * (P.Y_min + P.Y_max);
  T.fz = 0.5 * (P.Z_min + P.Z_max);
  T.cellrel = proper ? 1 : 0;
  double L = fmax(P.X_max - P.X_min, fmax(P.Y_max - P.Y_min, P.Z_max - P.Z_min));
  double wmax = fmax(T.wx, fmax(T.wy, T.wz));
  // FP32 screen slack: rounding of |coordinate| <= L (or <= 2 cell widths when
  // cell-relative) in each of the two operands, with a 5x margin
  T.pre_abs = (float)(1e-6 * (proper ? 4.0 * wmax : L));
  T.stencil = proper && P.stencil > 1 ? P.stencil : 1;
  const double wmin = fmin(T.wx, fmin(T.wy, T.wz));
  T.r1_hmax = T.stencil >= 2 ? 0.5 * wmin * (1.0 - 1e-9) : 1e300;
  T.rw = 1.0 / (wmin * (1.0 - 1e-9));
  T.reach_hmax = proper ? 0.5 * (T.stencil * wmin - T.skin) * (1.0 + 1e-9) : 1e300;
  T.inv_wx = 1.0 / T.wx; T.inv_wy = 1.0 / T.wy; T.inv_wz = 1.0 / T.wz; T.inv_aw = 1.0 / T.aw;
  set_index_maps(T);
}

ds_status check_params(ds_ctx *c, const ds_params &P) {
  if (P.n_dust < 1 || P.n_dust > DS_MAX_DUST) return fail(c, DS_ERR_ARG, "n_dust must be 1..4");
  if (!(P.h > 0)) return fail(c, DS_ERR_ARG, "h must be positive");
  if (P.Type_of_state != 0 && P.Type_of_state != 1) return fail(c, DS_ERR_ARG, "Type_of_state must be 0 or 1");
  if (P.precision != DS_PRECISION_FP64 && P.precision != DS_PRECISION_FP32)
    return fail(c, DS_ERR_ARG, "precision must be 0 (fp64) or 1 (fp32)");
  if ((P.precision == DS_PRECISION_FP32) && !(P.mode & DS_MODE_GRID_PROPER))
    return fail(c, DS_ERR_UNSUPPORTED, "the fp32 path needs the proper cell grid (DS_MODE_GRID_PROPER)");
  if (((P.mode & (DS_MODE_PERIODIC_Y | DS_MODE_PERIODIC_Z)) != 0) && !(P.mode & DS_MODE_GRID_PROPER))
    return fail(c, DS_ERR_UNSUPPORTED, "periodic axes need the proper cell grid (DS_MODE_GRID_PROPER)");
  if (!(P.list_skin >= 0 && P.list_skin <= 4)) return fail(c, DS_ERR_ARG, "list_skin must be in [0, 4]");
  if (P.persistent != 0 && P.persistent != 1) return fail(c, DS_ERR_ARG, "persistent must be 0 or 1");
  if (P.idic_lanes != 0 && P.idic_lanes != 2 && P.idic_lanes != 4 && P.idic_lanes != 8)
    return fail(c, DS_ERR_ARG, "idic_lanes must be 0, 2, 4 or 8");
  {  // the grid sizes in double first: the int conversions and products of build_desc must not overflow
    const double w = P.cell_w > 0 ? P.cell_w : 2.0 * P.h;  // list reuse only widens it: fewer cells
    const double aw = P.idic_w > 0 ? P.idic_w : P.Coeff_h_dust_cell * P.h;
    if (!(w > 0) || !(aw > 0) || !std::isfinite(w) || !std::isfinite(aw))
      return fail(c, DS_ERR_ARG, "cell widths must be positive and finite");
    const double ext[3] = {P.X_max - P.X_min, P.Y_max - P.Y_min, P.Z_max - P.Z_min};
    double cells = 1.0, icells = 1.0;
    for (double l : ext) {
      if (!std::isfinite(l) || l < 0) return fail(c, DS_ERR_ARG, "box extent must be finite and positive");
      cells *= std::floor(l / w) + 1.0;
      icells *= std::floor(l / aw) + 1.0;
    }
    if (!(cells <= (double)(1 << 28))) return fail(c, DS_ERR_ARG, "neighbour grid too large");
    if (!(icells <= (double)(1 << 28))) return fail(c, DS_ERR_ARG, "IDIC grid too large");
  }
  TubeDesc T;
  build_desc(P, T);
  if (T.Cnx < 0 || T.Cny < 0 || T.Cnz < 0) return fail(c, DS_ERR_ARG, "box extent must be positive");
  if (T.ncells <= 0 || T.ncells > (1 << 28)) return fail(c, DS_ERR_ARG, "neighbour grid too large");
  if (T.n_idic <= 0 || T.n_idic > (1 << 28)) return fail(c, DS_ERR_ARG, "IDIC grid too large");
  if (P.stencil < 0 || P.stencil > 4) return fail(c, DS_ERR_ARG, "stencil must be 1..4");
  if (P.stencil > 2 && P.precision != DS_PRECISION_FP32)
    return fail(c, DS_ERR_UNSUPPORTED, "stencils wider than 2 cells need the fp32 path");
  if (P.list_depth != 0 && P.list_depth != 32 && P.list_depth != 64)
    return fail(c, DS_ERR_ARG, "list_depth must be 0, 32 or 64");
  if (P.force_list < -1 || P.force_list > 4096) return fail(c, DS_ERR_ARG, "force_list must be -1, 0 or 1..4096");
  if (P.stencil >= 2 && !(P.mode & DS_MODE_GRID_PROPER))
    return fail(c, DS_ERR_UNSUPPORTED, "stencils of 2+ cells need the proper cell grid (DS_MODE_GRID_PROPER)");
  const int need = 2 * T.stencil + 1;  // a periodic axis must not alias its own stencil
  if ((P.mode & DS_MODE_PERIODIC_Y) && T.ny < need) return fail(c, DS_ERR_ARG, "too few cells across periodic y");
  if ((P.mode & DS_MODE_PERIODIC_Z) && T.nz < need) return fail(c, DS_ERR_ARG, "too few cells across periodic z");
  return DS_OK;
}

void add_chunks(std::vector<Chunk> &v, int tube, int s, int b, int e) {
  for (int q = b; q < e; q += DS_CHUNK) v.push_back(Chunk{tube, s, q, q + DS_CHUNK < e ? q + DS_CHUNK : e});
}

template <class T> ds_status upload_vec(ds_ctx *c, T **dptr, const std::vector<T> &v) {
  DA(*dptr, v.size());
  if (!v.empty()) CK(cudaMemcpy(*dptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return DS_OK;
}

SweepArgs sweep_args(ds_ctx *c, const Chunk *chunks, int nchunks) {
  SweepArgs a;
  a.tubes = c->d_tubes;
  a.tstate = c->d_tstate;
  a.chunks = chunks;
  a.nchunks = nchunks;
  a.st = c->buf[c->parity].view();
  a.cell_start = c->cell_start;
  a.pos32 = c->pos32;
  a.vm32 = c->vm32;
  a.pm32 = c->pm32;
  a.hyd32 = c->hyd32;
  a.cs64 = c->cs64;
  a.pt64 = c->pt64;
  a.dwn64 = c->dwn64;
  a.edot = c->edot;
  a.ncand = c->ncand;
  a.nnb = c->nnb;
  a.skey = c->skey;
  a.krad = c->krad;
  a.gas_slot_of_pid = c->slot_of_pid;
  a.gas_ind_pid = c->ind_of_pid;
  a.tstate_rw = c->d_tstate;
  a.flags = c->d_flags;
  a.all_tubes = 0;
  a.nbl = nullptr;
  a.nbl_cnt = nullptr;
  a.nbl_walk = nullptr;
  a.nbl_cap = 0;
  a.reuse = 0;
  a.work = nullptr;
  a.nsm = 0;
  for (int k = 0; k < DS_NSWEEP; k++) a.bps[k] = 0;
  return a;
}

// The step's sweeps: with persistent sweeps, the work counters (zeroed by
// k_step_begin) and the grid sizes.
SweepArgs step_sweep_args(ds_ctx *c, SweepArgs a) {
  if (c->persistent && c->d_work) {
    a.work = c->d_work;
    a.nsm = c->nsm;
    for (int k = 0; k < DS_NSWEEP; k++) a.bps[k] = c->bps[k];
  }
  return a;
}

// The gas sweeps' arguments, with the recorded force lists when there are any.
SweepArgs gas_sweep_args(ds_ctx *c) {
  SweepArgs ag = sweep_args(c, c->d_ch_gas, (int)c->ch_gas.size());
  if (c->nbl) {
    ag.nbl = c->nbl;
    ag.nbl_cnt = c->nbl_cnt;
    ag.nbl_walk = c->nbl_walk;
    ag.nbl_cap = c->nbl_cap;
    ag.reuse = c->reuse ? 1 : 0;
  }
  return ag;
}

// The sorted keys' buffer of the FP32 path's sorts (a fixed number of passes).
const uint32_t *fast_skey(const ds_ctx *c) {
  return (ds_radix_passes(c->key_bits + c->xl) & 1) ? c->kalt : c->kin;
}

// Sort + reorder + cell ranges for the particles' current positions; flips
// parity.  exact_order: cells list their particles in caller-index order even
// on the FP32 path (the parity hook's lists).  reuse: the step's list-reuse
// decisions apply (TubeState::rebuild, set by the start-of-step test); any
// other sort of a list-reuse context re-orders every tube, so the next step
// must re-sort and record (the force flag).  slot_pid (FP32 path, a step on
// bound host arrays with list reuse): the current buffer holds the host's
// state in caller order and slot i of the previous order held particle
// slot_pid[i]; the sort starts from the previous order, as a resident step's.
void enqueue_sort(ds_ctx *c, bool exact_order = false, cudaEvent_t before_reorder = nullptr, bool reuse = false,
                  const int *slot_pid = nullptr) {
  cudaStream_t s = c->stream;
  DevState src = c->buf[c->parity].view();
  DevState dst = c->buf[c->parity ^ 1].view();
  const bool fast = c->any_fp32 && !exact_order;
  const int xl = fast ? c->xl : 0;  // fast keys carry the x bin below the cell
  const bool ru = reuse && c->reuse && fast;
  const TubeState *rts = ru ? c->d_tstate : nullptr;
  const int *run_if = ru ? c->d_any : nullptr;
  c->last_xl = xl;
  const int *sp = (ru && slot_pid) ? slot_pid : nullptr;
  ds_launch_keys(c->d_tubes, c->d_ch_all, (int)c->ch_all.size(), src, c->kin, c->vin, fast, s, rts,
                 ru ? fast_skey(c) : nullptr, sp);
  bool alt = false;
  ds_radix_sort(c->kin, c->vin, c->kalt, c->valt, c->N, c->key_bits + xl, c->rs_scratch, s, &alt, run_if);
  const uint32_t *skey = alt ? c->kalt : c->kin;
  const uint32_t *sval = alt ? c->valt : c->vin;
  if (before_reorder) cudaStreamWaitEvent(s, before_reorder, 0);  // fields still arriving from the host
  ds_launch_reorder(c->d_tubes, c->d_ch_all, (int)c->ch_all.size(), sval, skey, src, dst, c->pos32, c->vm32,
                    c->idic_local, c->ikin, c->ivin, c->slot_of_pid, c->ind_of_pid, c->d_flags, fast, s, rts,
                    (c->reuse && fast) ? c->pos_ref : nullptr, sp, fast ? c->pm32 : nullptr);
  ds_launch_cell_start(skey, c->N, c->nkeys << xl, c->cell_start, s, run_if);
  c->skey = skey;
  if (c->any_stencil2)
    ds_launch_cell_radius(c->d_tubes, c->cell_start, c->nkeys, xl, dst.h, c->cwa, c->cwb, c->d_nseg_key0, c->d_nseg_tube,
                          c->d_nseg_species, c->nnseg, c->krad, s, run_if);
  if (c->reuse && !ru) cudaMemsetAsync(c->d_force, 1, sizeof(int), s);
  c->parity ^= 1;
}

// The step after the sort, first part: the IDIC key sort and the densities
// (with the EOS and the force sweep's per-particle inputs).  ev: optional
// phase events.
void enqueue_density(ds_ctx *c, cudaEvent_t *ev) {
  cudaStream_t s = c->stream;
  bool alt = false;
  ds_radix_sort(c->ikin, c->ivin, c->ikalt, c->ivalt, c->N, c->ikey_bits, c->rs_scratch, s, &alt);
  c->ialt = alt;
  if (ev) cudaEventRecord(ev[1], s);
  const bool fp32 = c->any_fp32;
  SweepArgs ag = step_sweep_args(c, gas_sweep_args(c));
  SweepArgs ad = step_sweep_args(c, sweep_args(c, c->d_ch_dust, (int)c->ch_dust.size()));
  const int depth = c->params[0].list_depth;
  if (fp32) ds_launch_density32(ag, c->any_hpp, 0, depth, s);
  else ds_launch_density64(ag, c->any_hpp, c->any_proper, 0, s);
  if (fp32 && c->reuse) {  // tubes keeping their lists
    if (c->dens_split) ds_launch_density32_lst_finish(ag, c->any_hpp, c->dsum, s);  // sums taken before the reorder
    else ds_launch_density32_lst(ag, c->any_hpp, s);
  }
  if (c->any_dust_rho) {
    if (fp32) ds_launch_density32(ad, c->any_hpp, 1, depth, s);
    else ds_launch_density64(ad, c->any_hpp, c->any_proper, 1, s);
  }
  if (ev) cudaEventRecord(ev[2], s);
}

// The rest of the step: t_stop, the step size, the force, the IDIC cell sums
// and solve, the update and the clock.
void enqueue_rest(ds_ctx *c, cudaEvent_t *ev, cudaEvent_t after_density = nullptr,
                  cudaEvent_t after_force = nullptr) {
  cudaStream_t s = c->stream;
  const bool fp32 = c->any_fp32;
  SweepArgs ag = step_sweep_args(c, gas_sweep_args(c));
  const int depth = c->params[0].list_depth;
  if (after_density) cudaEventRecord(after_density, s);
  if (fp32 && c->wstream) {  // the overflow walk beside t_stop, dt and the list kernel
    cudaEventRecord(c->e_wfork, s);
    cudaStreamWaitEvent(c->wstream, c->e_wfork, 0);
    ds_launch_force32_walk(ag, c->any_hpp, depth, c->wstream);
    cudaEventRecord(c->e_wjoin, c->wstream);
  }
  DevState st = c->buf[c->parity].view();
  ds_launch_tstop(c->d_tubes, c->d_tstate, c->d_ch_dust, (int)c->ch_dust.size(), st, c->slot_of_pid, c->d_flags, s);
  ds_launch_dt(c->d_tubes, c->d_tstate, c->ntubes, s);
  if (fp32 && c->wstream) {
    ds_launch_force32_list(ag, c->any_hpp, s);
    cudaStreamWaitEvent(s, c->e_wjoin, 0);
  } else if (fp32) {
    ds_launch_force32(ag, c->any_hpp, depth, s);
  } else {
    ds_launch_force64(ag, c->any_hpp, c->any_proper, s);
  }
  if (ev) cudaEventRecord(ev[3], s);
  if (after_force) cudaEventRecord(after_force, s);
  const uint32_t *ik = c->ialt ? c->ikalt : c->ikin;
  const uint32_t *iv = c->ialt ? c->ivalt : c->ivin;
  ds_launch_idic_reduce(ik, iv, c->N, c->nikeys, c->d_seg_key0, c->d_seg_species, c->d_seg_orphan, c->nseg, st,
                        c->ca, fp32, s, c->idic_lanes);
  ds_launch_idic_solve(c->d_tubes, c->d_tstate, c->d_tube_cell0, c->ntubes, c->ncell_total, c->ca, fp32, s);
  ds_launch_relax_move(c->d_tubes, c->d_tstate, c->d_ch_all, (int)c->ch_all.size(), st, c->idic_local, c->edot,
                       c->ca, c->d_flags, fp32, s);
  ds_launch_step_end(c->d_tstate, c->ntubes, s);
}

// The step after the sort: sweeps, IDIC, update.  ev: optional phase events.
void enqueue_physics(ds_ctx *c, cudaEvent_t *ev, cudaEvent_t after_density = nullptr,
                     cudaEvent_t after_force = nullptr) {
  enqueue_density(c, ev);
  enqueue_rest(c, ev, after_density, after_force);
}

// The start of a step: the clocks and, with list reuse, which tubes keep
// their lists; then the sort.
void enqueue_step_begin(ds_ctx *c) {
  ds_launch_step_begin(c->d_tubes, c->d_tstate, c->ntubes, c->d_work, c->stream);
  if (c->reuse)  // which tubes keep their lists this step
    ds_launch_list_test(c->d_tubes, c->d_tstate, c->ntubes, c->d_ch_gas, (int)c->ch_gas.size(),
                        c->buf[c->parity].view(), fast_skey(c), c->pos_ref, c->disp, c->d_nseg_key0, c->d_nseg_tube,
                        c->d_nseg_species, c->nnseg, c->nkeys, c->cell_start, c->xl, c->krad, c->cellstat,
                        c->d_force, c->d_any, c->stream);
  enqueue_sort(c, false, nullptr, true);
}

void enqueue_step(ds_ctx *c, cudaEvent_t *ev) {
  if (ev) cudaEventRecord(ev[0], c->stream);
  enqueue_step_begin(c);
  enqueue_physics(c, ev);
  if (ev) cudaEventRecord(ev[4], c->stream);
}

// ---------------------------------------------------------------------------
// A step on bound host arrays (ds_step_host): the bound fields come in from the
// host at the start, the changed ones go back as soon as the step has made
// them final, on a second stream, overlapped with the step's own kernels.
// ---------------------------------------------------------------------------

// inv[seg_begin + pid[i]] = i: the slot of every particle, all segments
__global__ void k_inverse(const Chunk *chunks, const TubeDesc *tubes, const int *pid, int *inv) {
  const Chunk ch = chunks[blockIdx.x];
  const int i = ch.begin + (int)threadIdx.x;
  if (i >= ch.end) return;
  inv[tubes[ch.tube].seg_begin[ch.species] + pid[i]] = i;
}

// Into the other buffer set in caller order (slot seg_begin + p = particle p):
// bound fields from the host, unbound ones gathered from the resident state;
// segments without host arrays carried over slot for slot.  PART 0: x, y, z
// and pid (what the cell keys read), and with EARLY also h, the mass and Ind
// (what the list-reuse test and the early density sums read); PART 1: the
// other fields.
template <bool EARLY>
__host__ __device__ constexpr int bound_part(int f) {
  return (f == FX || f == FY || f == FZ || (EARLY && (f == FH || f == FM))) ? 0 : 1;
}
template <int PART, bool EARLY>
__device__ __forceinline__ void bound_in_chunk(const Chunk &ch, const TubeDesc *tubes, const BoundSeg *bs,
                                               const int *inv, DevState src, DevState dst) {
  constexpr bool IND = (PART == 0) == EARLY;  // Ind travels in this part
  const int i = ch.begin + (int)threadIdx.x;
  if (i >= ch.end) return;
  const BoundSeg &B = bs[ch.tube * DS_MAXS + ch.species];
  const double *sf[NF] = {src.x, src.y, src.z, src.vx, src.vy, src.vz, src.ax, src.ay, src.az,
                          src.rho, src.p, src.e, src.m, src.h, src.ts};
  double *df[NF] = {dst.x, dst.y, dst.z, dst.vx, dst.vy, dst.vz, dst.ax, dst.ay, dst.az,
                    dst.rho, dst.p, dst.e, dst.m, dst.h, dst.ts};
  // a segment without host arrays keeps its slot order, except with list reuse
  // (EARLY), whose test and sort read every segment in caller order
  if (!B.bound && !EARLY) {
#pragma unroll
    for (int f = 0; f < NF; f++)
      if (bound_part<EARLY>(f) == PART) df[f][i] = sf[f][i];
    if (PART == 0) dst.pid[i] = src.pid[i];
    if (IND) dst.ind[i] = src.ind[i];
    return;
  }
  const int p = i - tubes[ch.tube].seg_begin[ch.species];
  const int q = inv[i];  // the resident slot of particle p
  double v[NF];          // every load before any store: the link's latency is paid once
  // (a segment without host arrays has no host fields: every one from q)
#pragma unroll
  for (int f = 0; f < NF; f++)
    if (bound_part<EARLY>(f) == PART) v[f] = B.f[f] ? B.f[f][p] : sf[f][q];
  int k = 0;
  if (IND) k = B.ind ? B.ind[p] : src.ind[q];
#pragma unroll
  for (int f = 0; f < NF; f++)
    if (bound_part<EARLY>(f) == PART) df[f][i] = v[f];
  if (PART == 0) dst.pid[i] = p;
  if (IND) dst.ind[i] = k;
}
template <int PART, bool EARLY>
__global__ void k_bound_in(const Chunk *chunks, int nchunks, const TubeDesc *tubes, const BoundSeg *bs,
                           const int *inv, DevState src, DevState dst) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
    bound_in_chunk<PART, EARLY>(chunks[c], tubes, bs, inv, src, dst);
}

// The bound fields a step has made final, back to the host in caller order:
// PART 0 after the density sweeps (rho, p), 1 after the force sweep (ax, ay,
// az, t_stop), 2 at the end (x, y, z, vx, vy, vz, e).
template <int PART>
__device__ __forceinline__ void bound_out_chunk(const Chunk &ch, const TubeDesc *tubes, const BoundSeg *bs,
                                                const int *inv, DevState st) {
  constexpr int NOUT = PART == 0 ? 2 : (PART == 1 ? 4 : 7);
  constexpr int fl0[2] = {FRHO, FP}, fl1[4] = {FAX, FAY, FAZ, FTS};
  constexpr int fl2[7] = {FX, FY, FZ, FVX, FVY, FVZ, FE};
  const int i = ch.begin + (int)threadIdx.x;
  if (i >= ch.end) return;
  const BoundSeg &B = bs[ch.tube * DS_MAXS + ch.species];
  if (!B.bound) return;
  const double *sf[NF] = {st.x, st.y, st.z, st.vx, st.vy, st.vz, st.ax, st.ay, st.az,
                          st.rho, st.p, st.e, st.m, st.h, st.ts};
  const int p = i - tubes[ch.tube].seg_begin[ch.species];
  const int q = inv[i];  // the slot of particle p after this step's sort
  double v[NOUT];
#pragma unroll
  for (int k = 0; k < NOUT; k++) {
    const int f = PART == 0 ? fl0[k] : (PART == 1 ? fl1[k] : fl2[k]);
    v[k] = sf[f][q];
  }
#pragma unroll
  for (int k = 0; k < NOUT; k++) {
    const int f = PART == 0 ? fl0[k] : (PART == 1 ? fl1[k] : fl2[k]);
    if (B.f[f] && (B.out_mask >> f & 1)) B.f[f][p] = v[k];
  }
}

template <int PART>
__global__ void k_bound_out(const Chunk *chunks, int nchunks, const TubeDesc *tubes, const BoundSeg *bs,
                            const int *inv, DevState st) {
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) bound_out_chunk<PART>(chunks[c], tubes, bs, inv, st);
}

void enqueue_bound_step(ds_ctx *c) {
  cudaStream_t s = c->stream, s2 = c->stream2;
  const int nch = (int)c->ch_all.size();
  const int P0 = c->parity;
  DevState old = c->buf[P0].view(), neu = c->buf[P0 ^ 1].view();
  k_inverse<<<nch, DS_CHUNK, 0, s>>>(c->d_ch_all, c->d_tubes, old.pid, c->inv);
  cudaEventRecord(c->e_fork, s);
  cudaStreamWaitEvent(s2, c->e_fork, 0);
  // The second stream's transfers run on a small grid: the link needs few
  // loads in flight, and a grid of every chunk would take all the SMs' slots
  // from the sort and the sweeps they are meant to overlap.
  const int nside = nch < c->side_blocks ? nch : c->side_blocks;
  // with list reuse the start-of-step test reads h and Ind too: they come
  // with the positions, on the first stream
  const bool ru = c->reuse && c->any_fp32;
  if (ru) {
    k_bound_in<0, true><<<nch, DS_CHUNK, 0, s>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, old, neu);
    k_bound_in<1, true><<<nside, DS_CHUNK, 0, s2>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, old, neu);
  } else {
    k_bound_in<0, false><<<nch, DS_CHUNK, 0, s>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, old, neu);
    k_bound_in<1, false><<<nside, DS_CHUNK, 0, s2>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, old, neu);
  }
  cudaEventRecord(c->e_up, s2);
  c->parity = P0 ^ 1;  // the caller-order state; the sort brings it back to P0
  ds_launch_step_begin(c->d_tubes, c->d_tstate, c->ntubes, c->d_work, s);
  if (ru) {
    // List reuse: the test measures the host's positions against the recorded
    // ones slot by slot (slot q of the resident order holds particle
    // old.pid[q]); a tube that keeps its lists keeps its slot order, and one
    // that re-sorts starts from it, as a step on the resident state does.
    ds_launch_list_test(c->d_tubes, c->d_tstate, c->ntubes, c->d_ch_gas, (int)c->ch_gas.size(), neu, fast_skey(c),
                        c->pos_ref, c->disp, c->d_nseg_key0, c->d_nseg_tube, c->d_nseg_species, c->nnseg, c->nkeys,
                        c->cell_start, c->xl, c->krad, c->cellstat, c->d_force, c->d_any, s, old.pid, old);
    // the tubes that keep their lists take their density sums now, from the
    // positions, h and masses already here, while the second stream still
    // brings the other fields; the rest of the sweep follows the reorder
    ds_launch_early_fp32(c->d_tubes, c->d_ch_gas, (int)c->ch_gas.size(), c->d_tstate, fast_skey(c), neu, old.pid,
                         c->pos32, c->pm32, s);
    ds_launch_density32_lst_sums(gas_sweep_args(c), c->any_hpp, neu, old.pid, c->dsum, s);
    c->dens_split = true;
    enqueue_sort(c, false, c->e_up, true, old.pid);
  } else {
    enqueue_sort(c, false, c->e_up);  // the host's arrays: every tube re-sorts
  }
  k_inverse<<<nch, DS_CHUNK, 0, s>>>(c->d_ch_all, c->d_tubes, c->buf[c->parity].pid, c->inv);
  enqueue_physics(c, nullptr, c->e_dens, c->e_force);
  c->dens_split = false;
  DevState st = c->buf[c->parity].view();
  cudaStreamWaitEvent(s2, c->e_dens, 0);
  k_bound_out<0><<<nside, DS_CHUNK, 0, s2>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, st);
  cudaStreamWaitEvent(s2, c->e_force, 0);
  k_bound_out<1><<<nside, DS_CHUNK, 0, s2>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, st);
  k_bound_out<2><<<nch, DS_CHUNK, 0, s>>>(c->d_ch_all, nch, c->d_tubes, c->d_bound, c->inv, st);
  cudaEventRecord(c->e_join, s2);
  cudaStreamWaitEvent(s, c->e_join, 0);
}

ds_status finalize(ds_ctx *c) {
  if (c->finalized) return DS_OK;
  CK(cudaSetDevice(c->device));
  // segments, keys
  c->tdesc.assign(c->ntubes, TubeDesc{});
  std::vector<int> seg_key0, seg_species, seg_orphan, tube_cell0, nseg_key0, nseg_tube, nseg_species;
  int N = 0;
  long long nkeys = 0, nikeys = 0, ncell = 0;
  for (int t = 0; t < c->ntubes; t++) {
    const ds_params &P = c->params[t];
    TubeDesc &T = c->tdesc[t];
    build_desc(P, T);
    const int ns = 1 + P.n_dust;
    for (int s = 0; s < ns; s++) {
      const HostSpecies &H = c->host[t][s];
      if (H.n < 0)
        return fail(c, DS_ERR_STATE, "tube " + std::to_string(t) + " species " + std::to_string(s) + " not set");
      T.seg_begin[s] = N;
      N += H.n;
      T.seg_end[s] = N;
      T.key_base[s] = (int)nkeys;
      nseg_key0.push_back((int)nkeys);
      nseg_tube.push_back(t);
      nseg_species.push_back(s);
      nkeys += T.ncells + 2;
      T.idic_base[s] = (int)nikeys;
      seg_key0.push_back((int)nikeys);
      seg_species.push_back(s);
      seg_orphan.push_back((int)nikeys + T.n_idic + 1);
      nikeys += T.n_idic + 2;
      add_chunks(c->ch_all, t, s, T.seg_begin[s], T.seg_end[s]);
      add_chunks(s == 0 ? c->ch_gas : c->ch_dust, t, s, T.seg_begin[s], T.seg_end[s]);
    }
    tube_cell0.push_back((int)ncell);
    ncell += T.n_idic + 1;
    if (P.mode & DS_MODE_H_PER_PARTICLE) c->any_hpp = true;
    if (P.mode & DS_MODE_GRID_PROPER) c->any_proper = true;
    if (P.mode & DS_MODE_DUST_RHO) c->any_dust_rho = true;
    if (P.precision == DS_PRECISION_FP32) c->any_fp32 = true;
    if (T.stencil >= 2) c->any_stencil2 = true;
  }
  if (nkeys >= (1LL << 31) || nikeys >= (1LL << 31)) return fail(c, DS_ERR_ARG, "key space too large");
  for (const auto &T : c->tdesc)
    for (int s = 0; s < DS_MAXS; s++)
      if (T.seg_end[s] - T.seg_begin[s] >= (T.precision == DS_PRECISION_FP32 ? (1 << 24) : (1 << 25)))
        return fail(c, DS_ERR_UNSUPPORTED, "more particles in one species of a tube than a list entry holds "
                                           "(2^24 on the fp32 path, 2^25 on the fp64 path)");
  // one kernel variant per batch: the mode bits that select templates must agree
  for (int t = 1; t < c->ntubes; t++) {
    const ds_params &P = c->params[t];
    if (((P.mode & DS_MODE_H_PER_PARTICLE) != 0) != c->any_hpp || ((P.mode & DS_MODE_GRID_PROPER) != 0) != c->any_proper ||
        (P.precision == DS_PRECISION_FP32) != c->any_fp32 || ((P.mode & DS_MODE_DUST_RHO) != 0) != c->any_dust_rho)
      return fail(c, DS_ERR_UNSUPPORTED, "tubes of one batch must share h mode, grid kind, dust-rho mode and precision");
  }
  c->N = N;
  c->nkeys = (int)nkeys;
  c->key_bits = bits_for(nkeys);
  // FP32 path: up to 2^DS_XL_MAX x bins per cell, as long as the start table stays
  // within ~8 entries per particle and the keys within 31 bits
  c->xl = 0;
  if (c->any_fp32 && c->any_proper) {
    c->xl = DS_XL_MAX;
    while (c->xl > 0 && ((nkeys << c->xl) > 8LL * N + 4096 || c->key_bits + c->xl > 31)) c->xl--;
  }
  for (auto &T : c->tdesc) {
    T.xl = c->xl;
    set_index_maps(T);
  }
  c->nikeys = (int)nikeys;
  c->ikey_bits = bits_for(nikeys);
  c->ncell_total = (int)ncell;
  c->nseg = (int)seg_key0.size();
  // device memory
  for (int b = 0; b < 2; b++) {
    for (int f = 0; f < NF; f++) DA(c->buf[b].f[f], N);
    DA(c->buf[b].ind, N);
    DA(c->buf[b].pid, N);
  }
  DA(c->pos32, N); DA(c->vm32, N); DA(c->hyd32, N);
  DA(c->cs64, N); DA(c->pt64, N); DA(c->dwn64, N); DA(c->edot, N);
  DA(c->kin, N); DA(c->vin, N); DA(c->kalt, N); DA(c->valt, N);
  DA(c->ikin, N); DA(c->ivin, N); DA(c->ikalt, N); DA(c->ivalt, N);
  DA(c->rs_scratch, ds_radix_scratch_words(N));
  DA(c->slot_of_pid, N); DA(c->ind_of_pid, N); DA(c->idic_local, N);
  DA(c->cell_start, ((size_t)nkeys << c->xl) + 1);
  DA(c->ncand, N); DA(c->nnb, N);
  DA(c->cwa, (size_t)nkeys);
  DA(c->cwb, (size_t)nkeys);
  DA(c->krad, (size_t)nkeys);
  CK(cudaMemsetAsync(c->krad, 1, (size_t)nkeys, c->stream));
  DA(c->stage, (size_t)NF * N + (N + 1) / 2 + 1);  // download staging: every field, then Ind
  if (c->any_fp32 && c->params[0].force_list != -1 && !c->ch_gas.empty()) {
    // the force sweep's neighbours, recorded by the gas density sweep
    // default capacity: 256 entries (interior gas has ~80 partners within
    // 2 max(h_i, h_j), shocked gas more); 512 when lists are recorded with a
    // skin, whose shell adds partners
    bool skin = false;
    for (const auto &T : c->tdesc) skin = skin || T.skin > 0.0;
    c->nbl_cap = c->params[0].force_list > 0 ? c->params[0].force_list : (skin ? 512 : 256);
    DA(c->nbl, c->ch_gas.size() * (size_t)c->nbl_cap * DS_CHUNK);
    DA(c->nbl_cnt, N);
    DA(c->nbl_walk, c->ch_gas.size() * (DS_SWEEP_THREADS / 32));
    CK(cudaStreamCreateWithFlags(&c->wstream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->e_wfork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->e_wjoin, cudaEventDisableTiming));
    for (const auto &T : c->tdesc) c->reuse = c->reuse || T.skin > 0.0;
    if (c->reuse) {
      DA(c->pm32, N);  // the streamed density gathers one 16-byte record per partner
      DA(c->dsum, N);
    }
  }
  c->persistent = c->any_fp32 && c->params[0].persistent != 0;
  DA(c->d_work, DS_NSWEEP);
  CK(cudaMemsetAsync(c->d_work, 0, sizeof(int) * DS_NSWEEP, c->stream));
  if (c->persistent) {
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
    ds_sweep32_blocks_per_sm(c->any_hpp, c->params[0].list_depth, c->nbl != nullptr, c->bps);
    CK(cudaGetLastError());
  }
  {
    const int l = c->params[0].idic_lanes;
    c->idic_lanes = (l == 2 || l == 8) ? l : 4;
  }
  if (c->reuse) {
    DA(c->pos_ref, N); DA(c->disp, N); DA(c->cellstat, (size_t)nkeys);
    DA(c->d_force, 1); DA(c->d_any, 1);
    CK(cudaMemsetAsync(c->d_force, 1, sizeof(int), c->stream));  // the first step sorts and records
    CK(cudaMemsetAsync(c->d_any, 1, sizeof(int), c->stream));
  }
  DA(c->d_cons, 8);
  DA(c->d_flags, 1);
  DA(c->ca.cnt, nikeys);
  DA(c->ca.start, (size_t)nikeys + 1);
  double **cd[] = {&c->ca.vx, &c->ca.vy, &c->ca.vz, &c->ca.a0, &c->ca.a1, &c->ca.a2, &c->ca.nvx, &c->ca.nvy,
                   &c->ca.nvz, &c->ca.px, &c->ca.py, &c->ca.pz, &c->ca.q0, &c->ca.q1};
  for (double **p : cd) DA(*p, nikeys);
  CK(cudaMemsetAsync(c->ca.cnt, 0, sizeof(int) * (size_t)nikeys, c->stream));
  for (double **p : cd) CK(cudaMemsetAsync(*p, 0, sizeof(double) * (size_t)nikeys, c->stream));
  CK(cudaMemsetAsync(c->edot, 0, sizeof(double) * (size_t)(N ? N : 1), c->stream));
  CK(cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
  // FP32 path: FP64 origins of every tube's x-blocks and y, z cells
  if (c->any_fp32) {
    size_t norig = 0;
    for (auto &T : c->tdesc) {
      T.nbx = (T.nx + DS_XB - 1) / DS_XB;
      norig += (size_t)T.nbx + T.ny + T.nz;
    }
    DA(c->origins, norig);
    size_t o = 0;
    for (auto &T : c->tdesc) {
      double *d = c->origins + o;
      T.orig = d;
      ds_launch_origins(T, d, c->stream);
      o += (size_t)T.nbx + T.ny + T.nz;
    }
    CK(cudaGetLastError());
  }
  // tables
  ds_status st;
  if ((st = upload_vec(c, &c->d_tubes, c->tdesc)) != DS_OK) return st;
  std::vector<TubeState> ts(c->ntubes);
  for (auto &x : ts) memset(&x, 0, sizeof(x));
  if ((st = upload_vec(c, &c->d_tstate, ts)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_ch_all, c->ch_all)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_ch_gas, c->ch_gas)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_ch_dust, c->ch_dust)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_seg_key0, seg_key0)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_seg_species, seg_species)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_seg_orphan, seg_orphan)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_tube_cell0, tube_cell0)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_nseg_key0, nseg_key0)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_nseg_tube, nseg_tube)) != DS_OK) return st;
  if ((st = upload_vec(c, &c->d_nseg_species, nseg_species)) != DS_OK) return st;
  c->nnseg = (int)nseg_key0.size();
  // particles: slot = segment begin + caller index
  c->parity = 0;
  for (int t = 0; t < c->ntubes; t++)
    for (int s = 0; s <= c->params[t].n_dust; s++) {
      if (c->dev_src[t].first) continue;  // copied from a resident tube below
      HostSpecies &H = c->host[t][s];
      const int b = c->tdesc[t].seg_begin[s];
      if (H.gen) {  // on the device, in caller order
        ds_launch_ic(*H.gen, s, c->buf[0].view(), b, c->stream);
        CK(cudaGetLastError());
        H.gen.reset();
        continue;
      }
      for (int f = 0; f < NF; f++)
        if (H.n) CK(cudaMemcpy(c->buf[0].f[f] + b, H.f[f].data(), sizeof(double) * H.n, cudaMemcpyHostToDevice));
      std::vector<int> pid(H.n);
      for (int i = 0; i < H.n; i++) pid[i] = i;
      if (H.n) {
        CK(cudaMemcpy(c->buf[0].ind + b, H.ind.data(), sizeof(int) * H.n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->buf[0].pid + b, pid.data(), sizeof(int) * H.n, cudaMemcpyHostToDevice));
      }
      for (int f = 0; f < NF; f++) { std::vector<double>().swap(H.f[f]); }
      std::vector<int>().swap(H.ind);
    }
  // tubes carried over from another context: state and clock, device to device
  for (int t = 0; t < c->ntubes; t++) {
    ds_ctx *src = c->dev_src[t].first;
    if (!src) continue;
    const int st_ = c->dev_src[t].second;
    CK(cudaStreamSynchronize(src->stream));
    const TubeDesc &S = src->tdesc[st_];
    const Buffers &B = src->buf[src->parity];
    for (int s = 0; s <= c->params[t].n_dust; s++) {
      const int n = S.seg_end[s] - S.seg_begin[s], sb = S.seg_begin[s], db = c->tdesc[t].seg_begin[s];
      if (n == 0) continue;
      for (int f = 0; f < NF; f++)
        CK(cudaMemcpyAsync(c->buf[0].f[f] + db, B.f[f] + sb, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
      CK(cudaMemcpyAsync(c->buf[0].ind + db, B.ind + sb, sizeof(int) * n, cudaMemcpyDeviceToDevice, c->stream));
      CK(cudaMemcpyAsync(c->buf[0].pid + db, B.pid + sb, sizeof(int) * n, cudaMemcpyDeviceToDevice, c->stream));
    }
    CK(cudaMemcpyAsync(c->d_tstate + t, src->d_tstate + st_, sizeof(TubeState), cudaMemcpyDeviceToDevice, c->stream));
  }
  // clocks set before the first step (a resumed checkpoint)
  for (int t = 0; t < c->ntubes; t++)
    if (!c->clock_set.empty() && c->clock_set[t].first) {
      TubeState ts;
      memset(&ts, 0, sizeof(ts));
      ts.Tm = c->clock_set[t].second.first;
      ts.nstep = c->clock_set[t].second.second;
      CK(cudaMemcpy(c->d_tstate + t, &ts, sizeof(ts), cudaMemcpyHostToDevice));
    }
  for (int k = 0; k <= DS_NPHASE; k++) CK(cudaEventCreate(&c->ev[k]));
  CK(cudaStreamSynchronize(c->stream));
  c->finalized = true;
  return DS_OK;
}

ds_status capture_graph(ds_ctx *c, int parity) {
  if (c->graph[parity]) return DS_OK;
  const int saved = c->parity;
  c->parity = parity;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step(c, nullptr);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->parity = saved;
  if (e != cudaSuccess) return fail(c, DS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&c->graph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(c, DS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return DS_OK;
}

ds_status capture_bound_graph(ds_ctx *c, int parity) {
  if (c->hgraph[parity]) return DS_OK;
  const int saved = c->parity;
  c->parity = parity;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_bound_step(c);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  const int after = c->parity;
  c->parity = saved;
  if (e != cudaSuccess) return fail(c, DS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  if (after != parity) {
    cudaGraphDestroy(g);
    return fail(c, DS_ERR_STATE, "bound step: buffer parity not restored");
  }
  e = cudaGraphInstantiate(&c->hgraph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(c, DS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return DS_OK;
}

ds_status check_flags(ds_ctx *c) {
  int f = 0;
  CK(cudaMemcpy(&f, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
  // DS_FLAG_NONFINITE is reported, not an error: the reference's own runs can
  // turn NaN (its eps guard, kernel.cu:2203) and go on
  if (f & ~DS_FLAG_NONFINITE) return fail(c, DS_ERR_DEVICE, "device flags set: " + std::to_string(f));
  return DS_OK;
}

// Host buffers that kernels may read or write in place: pinned and mapped
// (cudaMallocHost, ds_host_alloc, cudaHostAlloc, mapped cudaHostRegister).
// Their device address, else nullptr (pageable memory goes through the copy
// engines).  On GB300 kernels reach such buffers over NVLink-C2C with many
// loads in flight, well above what the copy engines give for many arrays.
template <class T> T *mapped_ptr(const T *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear: an unknown pointer is simply not mapped
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? (T *)a.devicePointer : nullptr;
}

struct HostFields {
  const double *src[NF];  // device addresses of mapped host arrays (nullptr: absent field)
};

// Upload of one segment straight from mapped host arrays, caller order (slot
// b + p holds particle p; the next step sorts); absent fields: h the tube's h,
// others zero.
__global__ void k_upload_mapped(HostFields hf, const int *ind, int n, double hdef, DevState dst, int b) {
  double *d[NF] = {dst.x, dst.y, dst.z, dst.vx, dst.vy, dst.vz, dst.ax, dst.ay, dst.az,
                   dst.rho, dst.p, dst.e, dst.m, dst.h, dst.ts};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    // every load issued before any store: the link's latency is paid once
    double v[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) v[f] = hf.src[f] ? hf.src[f][p] : (f == FH ? hdef : 0.0);
    const int k = ind[p];
#pragma unroll
    for (int f = 0; f < NF; f++) d[f][b + p] = v[f];
    dst.ind[b + p] = k;
    dst.pid[b + p] = p;
  }
}

ds_status set_species(ds_ctx *c, int tube, int s, int n, const double *const *fields, const int *ind) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c) return DS_ERR_ARG;
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  if (s < 0 || s > c->params[tube].n_dust) return fail(c, DS_ERR_ARG, "bad species index");
  if (n < 0) return fail(c, DS_ERR_ARG, "negative particle count");
  if (s == 0 && n > c->params[tube].Maximum_particle && c->params[tube].Maximum_particle > 0)
    return fail(c, DS_ERR_ARG, "gas count exceeds Maximum_particle (kernel.cu:1751)");
  const int req[] = {FX, FY, FZ, FVX, FVY, FVZ, FRHO, FM};
  for (int f : req)
    if (n > 0 && !fields[f]) return fail(c, DS_ERR_ARG, "required array is NULL");
  if (n > 0 && !ind) return fail(c, DS_ERR_ARG, "ind is NULL");
  if (!c->finalized) {
    c->dev_src[tube] = std::make_pair((ds_ctx *)nullptr, 0);
    HostSpecies &H = c->host[tube][s];
    H.n = n;
    H.gen.reset();
    for (int f = 0; f < NF; f++) {
      if (fields[f]) H.f[f].assign(fields[f], fields[f] + n);
      else if (f == FH) H.f[f].assign(n, c->params[tube].h);
      else H.f[f].assign(n, 0.0);
    }
    H.ind.assign(ind, ind + n);
    return DS_OK;
  }
  // resident state: overwrite this segment in caller order (the next step sorts)
  const TubeDesc &T = c->tdesc[tube];
  if (n != T.seg_end[s] - T.seg_begin[s]) return fail(c, DS_ERR_STATE, "particle count differs from the resident state");
  CK(cudaSetDevice(c->device));
  Buffers &B = c->buf[c->parity];
  const int b = T.seg_begin[s];
  {  // every given array mapped: one kernel reads them in place
    HostFields hf;
    bool all = n > 0;
    for (int f = 0; f < NF && all; f++) {
      hf.src[f] = mapped_ptr(fields[f]);
      all = !fields[f] || hf.src[f];
    }
    const int *dind = all ? mapped_ptr(ind) : nullptr;
    if (all && dind) {
      k_upload_mapped<<<(n + 255) / 256, 256, 0, c->stream>>>(hf, dind, n, c->params[tube].h, B.view(), b);
      CK(cudaGetLastError());
      if (c->reuse) CK(cudaMemsetAsync(c->d_force, 1, sizeof(int), c->stream));  // caller order: re-sort
      return DS_OK;
    }
  }
  for (int f = 0; f < NF; f++) {
    if (fields[f]) {
      CK(cudaMemcpyAsync(B.f[f] + b, fields[f], sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    } else if (f == FH) {
      ds_launch_fill(B.f[f] + b, n, c->params[tube].h, c->stream);
      CK(cudaGetLastError());
    } else {
      CK(cudaMemsetAsync(B.f[f] + b, 0, sizeof(double) * n, c->stream));  // absent field: zero
    }
  }
  CK(cudaMemcpyAsync(B.ind + b, ind, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
  ds_launch_iota(B.pid + b, n, c->stream);  // caller order: slot b + p holds particle p
  CK(cudaGetLastError());
  if (c->reuse) CK(cudaMemsetAsync(c->d_force, 1, sizeof(int), c->stream));  // the next step re-sorts
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

// Download straight into mapped host arrays, written in caller order
// (coalesced over the link): inv[p] = slot of particle p, then each thread p
// reads its particle's slot.
__global__ void k_slot_of(const int *pid, int b, int n, int *inv) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) inv[pid[b + q]] = q;
}
struct HostOut {
  double *dst[NF];
  const double *src[NF];
  int nf;
};
__global__ void k_download_mapped(HostOut ho, const int *ind, int *ind_out, const int *inv, int b, int n) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int q = b + inv[p];
    double v[NF];  // every load before any store
#pragma unroll
    for (int k = 0; k < NF; k++) v[k] = k < ho.nf ? ho.src[k][q] : 0.0;
    const int i = ind_out ? ind[q] : 0;
#pragma unroll
    for (int k = 0; k < NF; k++)
      if (k < ho.nf) ho.dst[k][p] = v[k];
    if (ind_out) ind_out[p] = i;
  }
}

// Every requested field of one segment back into caller order in one pass:
// field k of the request (src[k]) to stage[k * n + pid], Ind to istage[pid].
struct FieldSet {
  const double *src[NF];
  int nf;
};
__global__ void k_to_caller_order(FieldSet fs, const int *ind, const int *pid, int b, int n, double *stage,
                                  int *istage) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int p = pid[b + q];
  for (int k = 0; k < fs.nf; k++) stage[(size_t)k * n + p] = fs.src[k][b + q];
  if (istage) istage[p] = ind[b + q];
}

ds_status get_species(ds_ctx *c, int tube, int s, double *const *out, int *ind_out) {
  if (!c) return DS_ERR_ARG;
  if (!c->finalized) {  // the particles as set: build the resident state now
    const ds_status st = finalize(c);
    if (st != DS_OK) return st;
  }
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  if (s < 0 || s > c->params[tube].n_dust) return fail(c, DS_ERR_ARG, "bad species index");
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  const int b = T.seg_begin[s], n = T.seg_end[s] - b;
  if (n == 0) return DS_OK;
  Buffers &B = c->buf[c->parity];
  {  // every output mapped: write them in place
    HostOut ho;
    ho.nf = 0;
    bool all = true;
    for (int f = 0; f < NF && all; f++)
      if (out[f]) {
        ho.dst[ho.nf] = mapped_ptr(out[f]);
        ho.src[ho.nf] = B.f[f];
        all = ho.dst[ho.nf++] != nullptr;
      }
    int *dind = ind_out ? mapped_ptr(ind_out) : nullptr;
    if (all && (!ind_out || dind)) {
      int *inv = reinterpret_cast<int *>(c->stage + (size_t)NF * c->N);
      k_slot_of<<<(n + 255) / 256, 256, 0, c->stream>>>(B.pid, b, n, inv);
      k_download_mapped<<<(n + 255) / 256, 256, 0, c->stream>>>(ho, B.ind, dind, inv, b, n);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(c->stream));
      return DS_OK;
    }
  }
  // one gather of every requested field into its own stage region, then the
  // copies back to back (the copy engine streams without kernels in between)
  FieldSet fs;
  int map[NF];
  fs.nf = 0;
  for (int f = 0; f < NF; f++)
    if (out[f]) {
      map[fs.nf] = f;
      fs.src[fs.nf++] = B.f[f];
    }
  int *istage = ind_out ? reinterpret_cast<int *>(c->stage + (size_t)NF * c->N) : nullptr;
  k_to_caller_order<<<(n + 255) / 256, 256, 0, c->stream>>>(fs, B.ind, B.pid, b, n, c->stage, istage);
  CK(cudaGetLastError());
  for (int k = 0; k < fs.nf; k++)
    CK(cudaMemcpyAsync(out[map[k]], c->stage + (size_t)k * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                       c->stream));
  if (ind_out) CK(cudaMemcpyAsync(ind_out, istage, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}


}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *ds_version(void) { return DS_VERSION; }

ds_status ds_params_init(ds_params *p) {
  if (!p) return DS_ERR_ARG;
  memset(p, 0, sizeof(*p));
  // Init.txt as shipped (Init.txt:2-18)
  p->X_min = -2.0; p->X_max = 2.0; p->Y_min = -2.0; p->Y_max = 2.0; p->Z_min = -2.0; p->Z_max = 2.0;
  p->Type_of_state = 0; p->Maximum_particle = 1000000; p->Particle_on_length = 40; p->h = 0.1;
  p->Coeff_h_dust_cell = 0.5; p->tau = 5.0e-3; p->T_end = 0.2; p->T_out = 0.1;
  p->alpha = 1.0; p->beta = 2.0; p->eps = 0.01;
  p->Gam_g = 1.4;               // data.h:7
  p->Speed_of_sound_gas = 1.0;  // kernel.cu:1744
  p->n_dust = 2;
  p->mode = DS_MODE_REFERENCE;
  p->precision = DS_PRECISION_FP64;
  p->stencil = 1;  // the reference's 27 cells
  p->cfl = 0.3;
  p->t_empty = 1.0;  // kernel.cu:2160
  p->mass_ratio[0] = 0.75; p->mass_ratio[1] = 0.5;   // kernel.cu:1499-1502
  p->R_dust[0] = 0.01; p->R_dust[1] = 1.0;
  p->t_stop_const[0] = p->t_stop_const[1] = 1e-3;
  p->eps_empty[0] = 0.5; p->eps_empty[1] = 0.33;     // kernel.cu:2200, 2209
  return DS_OK;
}

ds_status ds_params_read_init_txt(const char *path, ds_params *p) {
  if (!path || !p) return DS_ERR_ARG;
  return ds_read_init_txt_file(path, p);
}

ds_status ds_create_batch(int ntubes, const ds_params *p, ds_ctx **out) {
  if (!out || !p || ntubes <= 0) return DS_ERR_ARG;
  *out = nullptr;
  ds_ctx *c = new ds_ctx();
  for (int t = 0; t < ntubes; t++) {
    ds_status st = check_params(c, p[t]);
    if (st != DS_OK) { delete c; return st; }
  }
  c->ntubes = ntubes;
  c->params.assign(p, p + ntubes);
  c->host.resize(ntubes);
  for (int t = 0; t < ntubes; t++) c->host[t].resize(1 + p[t].n_dust);
  c->dev_src.assign(ntubes, std::make_pair((ds_ctx *)nullptr, 0));
  if (cudaGetDevice(&c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return DS_ERR_CUDA;
  }
  *out = c;
  return DS_OK;
}

ds_status ds_create(const ds_params *p, ds_ctx **out) { return ds_create_batch(1, p, out); }

ds_status ds_set_gas(ds_ctx *c, int tube, int n, const double *x, const double *y, const double *z,
                     const double *vx, const double *vy, const double *vz, const double *ax, const double *ay,
                     const double *az, const double *rho, const double *p, const double *e, const double *mas,
                     const double *h, const int *ind) {
  const double *f[NF] = {x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, mas, h, nullptr};
  if (!c) return DS_ERR_ARG;
  if (n > 0 && (!p || !e)) return fail(c, DS_ERR_ARG, "gas p and e are required");
  return set_species(c, tube, 0, n, f, ind);
}

ds_status ds_set_dust(ds_ctx *c, int tube, int species, int n, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, const double *rho, const double *mas,
                      const double *t_stop, const double *h, const int *ind) {
  if (!c) return DS_ERR_ARG;
  if (species < 1) return fail(c, DS_ERR_ARG, "dust species are numbered from 1");
  if (n > 0 && !t_stop) return fail(c, DS_ERR_ARG, "dust t_stop is required");
  const double *f[NF] = {x, y, z, vx, vy, vz, nullptr, nullptr, nullptr, rho, nullptr, nullptr, mas, h, t_stop};
  return set_species(c, tube, species, n, f, ind);
}

ds_status ds_copy_tube(ds_ctx *dst, int dst_tube, ds_ctx *src, int src_tube) {
  if (!dst || !src || dst == src) return DS_ERR_ARG;
  ds_ctx *c = dst;
  if (dst->finalized) return fail(c, DS_ERR_STATE, "ds_copy_tube: destination already holds its state");
  if (!src->finalized) return fail(c, DS_ERR_STATE, "ds_copy_tube: source has no resident state");
  if (dst_tube < 0 || dst_tube >= dst->ntubes || src_tube < 0 || src_tube >= src->ntubes)
    return fail(c, DS_ERR_ARG, "ds_copy_tube: bad tube index");
  if (dst->device != src->device) return fail(c, DS_ERR_UNSUPPORTED, "ds_copy_tube: contexts on different devices");
  const int nd = dst->params[dst_tube].n_dust;
  if (nd != src->params[src_tube].n_dust) return fail(c, DS_ERR_ARG, "ds_copy_tube: species counts differ");
  const TubeDesc &S = src->tdesc[src_tube];
  for (int s = 0; s <= nd; s++) {
    HostSpecies &H = dst->host[dst_tube][s];
    H.n = S.seg_end[s] - S.seg_begin[s];
    for (int f = 0; f < NF; f++) std::vector<double>().swap(H.f[f]);
    std::vector<int>().swap(H.ind);
    H.gen.reset();
  }
  dst->dev_src[dst_tube] = std::make_pair(src, src_tube);
  return DS_OK;
}

ds_status ds_ic_init(ds_ic *ic, int kind) {
  if (!ic) return DS_ERR_ARG;
  if (kind != DS_IC_SOD_X_DUST && kind != DS_IC_SOD_X_MAS && kind != DS_IC_DUSTY_SOD) return DS_ERR_ARG;
  memset(ic, 0, sizeof(*ic));
  ic->kind = kind;
  // the dusty Sod tube's defaults: classical Sod states, one dust species
  ic->eps = 1.0;
  ic->t_s = 1e-3;
  ic->rho_L = 1.0;
  ic->p_L = 1.0;
  ic->rho_R = 0.125;
  ic->p_R = 0.1;
  ic->gamma = 1.4;
  ic->h_factor = 1.3;
  ic->x0 = -0.5;
  ic->x1 = 0.5;
  ic->wall = 2.5;
  ic->lattice_offset = 0.25;
  ic->t_end = 0.2;
  ic->cfl = 0.3;
  ic->alpha = 1.0;
  ic->beta = 2.0;
  ic->av_eps = 0.01;
  ic->idic_cells = 2.0;
  return DS_OK;
}

ds_status ds_ic_read_init_txt(const char *path, ds_ic *ic) {
  if (!path || !ic) return DS_ERR_ARG;
  return ds_read_ic_txt_file(path, ic);
}

ds_status ds_ic_plan(const ds_ic *ic, const ds_params *init, ds_params *out, int *counts) {
  if (!ic || !out || !counts) return DS_ERR_ARG;
  IcPlan plan;
  std::string err;
  const ds_status st = ds_ic_make_plan(*ic, init, plan, err);
  if (st != DS_OK) return st;
  if (check_params(nullptr, plan.params) != DS_OK) return DS_ERR_ARG;
  *out = plan.params;
  for (int s = 0; s < plan.nspecies; s++) counts[s] = (int)plan.count[s];
  return DS_OK;
}

ds_status ds_init_tube(ds_ctx *c, int tube, const ds_ic *ic) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c || !ic) return DS_ERR_ARG;
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  auto plan = std::make_shared<IcPlan>();
  std::string err;
  ds_status st = ds_ic_make_plan(*ic, &c->params[tube], *plan, err);
  if (st != DS_OK) return fail(c, st, "ds_init_tube: " + err);
  const ds_params &P = c->params[tube];
  if (plan->nspecies != 1 + P.n_dust)
    return fail(c, DS_ERR_ARG, "ds_init_tube: the generator's species count differs from the tube's n_dust");
  if (P.Maximum_particle > 0 && plan->count[0] > P.Maximum_particle)
    return fail(c, DS_ERR_ARG, "gas count exceeds Maximum_particle (kernel.cu:1751)");
  if (!c->finalized) {
    c->dev_src[tube] = std::make_pair((ds_ctx *)nullptr, 0);
    for (int s = 0; s < plan->nspecies; s++) {
      HostSpecies &H = c->host[tube][s];
      H.n = (int)plan->count[s];
      for (int f = 0; f < NF; f++) std::vector<double>().swap(H.f[f]);
      std::vector<int>().swap(H.ind);
      H.gen = plan;
    }
    return DS_OK;
  }
  // resident tube: overwrite its segments in caller order (the next step sorts)
  const TubeDesc &T = c->tdesc[tube];
  for (int s = 0; s < plan->nspecies; s++)
    if (plan->count[s] != T.seg_end[s] - T.seg_begin[s])
      return fail(c, DS_ERR_STATE, "particle count differs from the resident state");
  CK(cudaSetDevice(c->device));
  for (int s = 0; s < plan->nspecies; s++) {
    ds_launch_ic(*plan, s, c->buf[c->parity].view(), T.seg_begin[s], c->stream);
    CK(cudaGetLastError());
  }
  if (c->reuse) CK(cudaMemsetAsync(c->d_force, 1, sizeof(int), c->stream));  // the next step re-sorts
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_upload_gas(ds_ctx *c, int n, const double *x, const double *y, const double *z, const double *vx,
                        const double *vy, const double *vz, const double *ax, const double *ay, const double *az,
                        const double *rho, const double *p, const double *e, const double *mas, const double *h,
                        const int *ind) {
  return ds_set_gas(c, 0, n, x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, mas, h, ind);
}

ds_status ds_upload_dust(ds_ctx *c, int species, int n, const double *x, const double *y, const double *z,
                         const double *vx, const double *vy, const double *vz, const double *rho, const double *mas,
                         const double *t_stop, const double *h, const int *ind) {
  return ds_set_dust(c, 0, species, n, x, y, z, vx, vy, vz, rho, mas, t_stop, h, ind);
}

ds_status ds_step_async(ds_ctx *c, int nsteps) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c || nsteps < 0) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  CK(cudaSetDevice(c->device));
  for (int k = 0; k < nsteps; k++) {
    st = capture_graph(c, c->parity);
    if (st != DS_OK) return st;
    CK(cudaGraphLaunch(c->graph[c->parity], c->stream));
    c->parity ^= 1;  // the step's reorder swapped the buffers
  }
  return DS_OK;
}

ds_status ds_synchronize(ds_ctx *c) {
  if (!c) return DS_ERR_ARG;
  if (!c->finalized) return DS_OK;
  CK(cudaStreamSynchronize(c->stream));
  return check_flags(c);
}

ds_status ds_step(ds_ctx *c, int nsteps) {
  ds_status st = ds_step_async(c, nsteps);
  if (st != DS_OK) return st;
  return ds_synchronize(c);
}

ds_status ds_bind_host(ds_ctx *c, int tube, int species, int n, double *const *fields, int *ind) {
  if (!c) return DS_ERR_ARG;
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  if (species < 0 || species > c->params[tube].n_dust) return fail(c, DS_ERR_ARG, "bad species index");
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  if (fields && n != T.seg_end[species] - T.seg_begin[species])
    return fail(c, DS_ERR_ARG, "ds_bind_host: n differs from the tube's particle count");
  BoundSeg B;
  memset(&B, 0, sizeof(B));
  if (fields) {
    for (int f = 0; f < NF; f++)
      if (fields[f]) {
        B.f[f] = mapped_ptr(fields[f]);
        if (!B.f[f]) return fail(c, DS_ERR_ARG, "ds_bind_host: arrays must be pinned host memory (ds_host_alloc, "
                                                "cudaMallocHost or cudaHostRegister)");
      }
    if (ind) {
      B.ind = mapped_ptr(ind);
      if (!B.ind) return fail(c, DS_ERR_ARG, "ds_bind_host: ind must be pinned host memory");
    }
    B.bound = 1;
    // written back: what a step can change in the reference's layout (dust rho
    // only with the per-step dust density, t_stop only when not constant)
    const int mode = c->params[tube].mode;
    B.out_mask = species == 0 ? (1 << FX | 1 << FY | 1 << FZ | 1 << FVX | 1 << FVY | 1 << FVZ | 1 << FAX | 1 << FAY |
                                 1 << FAZ | 1 << FRHO | 1 << FP | 1 << FE)
                              : (1 << FX | 1 << FY | 1 << FZ | 1 << FVX | 1 << FVY | 1 << FVZ |
                                 ((mode & DS_MODE_DUST_RHO) ? 1 << FRHO : 0) |
                                 ((mode & DS_MODE_TSTOP_CONST) ? 0 : 1 << FTS));
  }
  if (c->hbound.empty()) {
    BoundSeg z;
    memset(&z, 0, sizeof(z));
    c->hbound.assign((size_t)c->ntubes * DS_MAXS, z);
  }
  if (!c->inv) DA(c->inv, c->N ? c->N : 1);
  if (!c->d_bound) DA(c->d_bound, c->hbound.size());
  if (!c->stream2) {
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
#ifndef DS_SIDE_BLOCKS_PER_SM
#define DS_SIDE_BLOCKS_PER_SM 1  // measured on the 1.44M tube: 1 beats 2 and 4
#endif
    c->side_blocks = (sms > 0 ? sms : 1) * DS_SIDE_BLOCKS_PER_SM;
    CK(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    cudaEvent_t *evs[] = {&c->e_fork, &c->e_up, &c->e_dens, &c->e_force, &c->e_join};
    for (cudaEvent_t *e : evs) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  c->hbound[(size_t)tube * DS_MAXS + species] = B;
  c->any_bound = false;
  for (const BoundSeg &x : c->hbound) c->any_bound |= x.bound != 0;
  CK(cudaStreamSynchronize(c->stream));  // no step reads the table while it changes
  CK(cudaMemcpy(c->d_bound, c->hbound.data(), sizeof(BoundSeg) * c->hbound.size(), cudaMemcpyHostToDevice));
  return DS_OK;
}

ds_status ds_step_host(ds_ctx *c, int nsteps) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c || nsteps < 0) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  if (!c->any_bound) return fail(c, DS_ERR_STATE, "ds_step_host: no host arrays bound (ds_bind_host)");
  CK(cudaSetDevice(c->device));
  for (int k = 0; k < nsteps; k++) {
    st = capture_bound_graph(c, c->parity);
    if (st != DS_OK) return st;
    CK(cudaGraphLaunch(c->hgraph[c->parity], c->stream));  // leaves the state in the same buffer set
  }
  return ds_synchronize(c);
}

ds_status ds_step_timed(ds_ctx *c, int nsteps, float *total_ms, float *phase_ms) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c || nsteps < 0) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  CK(cudaSetDevice(c->device));
  if (!phase_ms) {  // the steps as ds_step runs them: graph replays between two events
    if (c->tev.size() < 2) {
      for (int k = (int)c->tev.size(); k < 2; k++) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c->tev.push_back(e);
      }
    }
    CK(cudaEventRecord(c->tev[0], c->stream));
    for (int k = 0; k < nsteps; k++) {
      st = capture_graph(c, c->parity);
      if (st != DS_OK) return st;
      CK(cudaGraphLaunch(c->graph[c->parity], c->stream));
      c->parity ^= 1;
    }
    CK(cudaEventRecord(c->tev[1], c->stream));
    CK(cudaEventSynchronize(c->tev[1]));
    float tot = 0;
    CK(cudaEventElapsedTime(&tot, c->tev[0], c->tev[1]));
    if (total_ms) *total_ms = tot;
    return check_flags(c);
  }
  // one event set per step so that the steps run back to back with a single
  // synchronisation at the end
  const size_t need = (size_t)nsteps * (DS_NPHASE + 1);
  while (c->tev.size() < need) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->tev.push_back(e);
  }
  for (int k = 0; k < nsteps; k++) enqueue_step(c, &c->tev[(size_t)k * (DS_NPHASE + 1)]);
  CK(cudaGetLastError());
  float acc[DS_NPHASE] = {0, 0, 0, 0}, tot = 0;
  if (nsteps > 0) {
    CK(cudaEventSynchronize(c->tev[need - 1]));
    for (int k = 0; k < nsteps; k++) {
      cudaEvent_t *ev = &c->tev[(size_t)k * (DS_NPHASE + 1)];
      for (int p = 0; p < DS_NPHASE; p++) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev[p], ev[p + 1]));
        acc[p] += ms;
      }
    }
    CK(cudaEventElapsedTime(&tot, c->tev[0], c->tev[need - 1]));
  }
  if (total_ms) *total_ms = tot;
  if (phase_ms)
    for (int p = 0; p < DS_NPHASE; p++) phase_ms[p] = acc[p];
  return check_flags(c);
}

ds_status ds_dust_density(ds_ctx *c) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  CK(cudaSetDevice(c->device));
  if (c->ch_dust.empty()) return DS_OK;
  enqueue_sort(c);  // cells for the current positions (caller-index order on the FP64 path)
  SweepArgs ad = sweep_args(c, c->d_ch_dust, (int)c->ch_dust.size());
  ad.all_tubes = 1;
  if (c->any_fp32) ds_launch_density32(ad, c->any_hpp, 1, c->params[0].list_depth, c->stream);
  else ds_launch_density64(ad, c->any_hpp, c->any_proper, 1, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_kernels_per_step(ds_ctx *c, int *count) {
  if (!c || !count) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  // step_begin, keys, reorder, cell_start, density, t_stop, dt, force,
  // idic_reduce, idic_solve, relax_move, step_end, 3 per radix pass, dust density
  // list reuse: displacements, cell statistics, bound, decision, density stream
  *count = 13 + 3 * (ds_radix_passes(c->key_bits + c->xl) + ds_radix_passes(c->ikey_bits)) + (c->any_dust_rho ? 1 : 0) +
           (c->any_stencil2 ? 4 : 0) + (c->nbl ? 1 : 0) + (c->reuse ? 5 : 0);
  return DS_OK;
}

ds_status ds_list_stats(ds_ctx *c, int tube, long long *rebuilds, long long *steps) {
  if (!c || tube < 0 || tube >= c->ntubes) return DS_ERR_ARG;
  if (!c->finalized) {
    if (rebuilds) *rebuilds = 0;
    if (steps) *steps = 0;
    return DS_OK;
  }
  TubeState ts;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(&ts, c->d_tstate + tube, sizeof(ts), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (rebuilds) *rebuilds = c->reuse ? ts.nrebuild : ts.nstep;  // without reuse every step re-sorts
  if (steps) *steps = ts.nstep;
  return DS_OK;
}

// ---------------------------------------------------------------------------
// Split step (slab decomposition of one tube across processes)
// ---------------------------------------------------------------------------

ds_status ds_step_density(ds_ctx *c) {
  if (!c) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  if (c->split) return fail(c, DS_ERR_STATE, "ds_step_density: the previous step is not complete (ds_step_complete)");
  CK(cudaSetDevice(c->device));
  enqueue_step_begin(c);
  enqueue_density(c, nullptr);
  CK(cudaGetLastError());
  c->split = 1;
  CK(cudaStreamSynchronize(c->stream));
  return check_flags(c);
}

ds_status ds_get_cfl_min(ds_ctx *c, int tube, double *dtmin) {
  if (!c || tube < 0 || tube >= c->ntubes || !dtmin) return DS_ERR_ARG;
  if (!c->split) return fail(c, DS_ERR_STATE, "ds_get_cfl_min: between ds_step_density and ds_step_complete only");
  CK(cudaSetDevice(c->device));
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, &c->d_tstate[tube].dtmin_bits, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  memcpy(dtmin, &bits, sizeof(double));
  return DS_OK;
}

ds_status ds_set_cfl_min(ds_ctx *c, int tube, double dtmin) {
  if (!c || tube < 0 || tube >= c->ntubes) return DS_ERR_ARG;
  if (!c->split) return fail(c, DS_ERR_STATE, "ds_set_cfl_min: between ds_step_density and ds_step_complete only");
  if (!(dtmin > 0)) return fail(c, DS_ERR_ARG, "ds_set_cfl_min: dtmin must be positive (or +inf)");
  CK(cudaSetDevice(c->device));
  unsigned long long bits = 0;
  memcpy(&bits, &dtmin, sizeof(double));
  CK(cudaMemcpyAsync(&c->d_tstate[tube].dtmin_bits, &bits, sizeof(bits), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_set_gas_hydro(ds_ctx *c, int tube, int n, const int *idx, const double *rho, const double *p) {
  if (!c || tube < 0 || tube >= c->ntubes || n < 0 || (n > 0 && (!idx || !rho || !p))) return DS_ERR_ARG;
  if (!c->split) return fail(c, DS_ERR_STATE, "ds_set_gas_hydro: between ds_step_density and ds_step_complete only");
  const TubeDesc &T = c->tdesc[tube];
  const int ng = T.seg_end[0] - T.seg_begin[0];
  if (n > ng) return fail(c, DS_ERR_ARG, "ds_set_gas_hydro: more entries than gas particles");
  for (int k = 0; k < n; k++)
    if (idx[k] < 0 || idx[k] >= ng) return fail(c, DS_ERR_ARG, "ds_set_gas_hydro: index out of range");
  if (n == 0) return DS_OK;
  CK(cudaSetDevice(c->device));
  if (c->hy_cap < n) {  // once, for every gas particle of the largest tube
    int cap = 0;
    for (const auto &D : c->tdesc) cap = std::max(cap, D.seg_end[0] - D.seg_begin[0]);
    DA(c->hy_idx, (size_t)cap);
    DA(c->hy_val, 2 * (size_t)cap);
    c->hy_cap = cap;
  }
  if (!c->inv) DA(c->inv, c->N ? c->N : 1);
  CK(cudaMemcpyAsync(c->hy_idx, idx, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->hy_val, rho, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->hy_val + n, p, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  const int nch = (int)c->ch_all.size();
  DevState st = c->buf[c->parity].view();
  if (nch) k_inverse<<<nch, DS_CHUNK, 0, c->stream>>>(c->d_ch_all, c->d_tubes, st.pid, c->inv);
  ds_launch_set_hydro(c->d_tubes, tube, n, c->hy_idx, c->hy_val, c->inv, st, c->cs64, c->pt64, c->hyd32, c->pos32,
                      c->any_fp32, c->any_hpp, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_step_complete(ds_ctx *c) {
  if (!c) return DS_ERR_ARG;
  if (!c->split) return fail(c, DS_ERR_STATE, "ds_step_complete: no step begun (ds_step_density)");
  CK(cudaSetDevice(c->device));
  enqueue_rest(c, nullptr);
  CK(cudaGetLastError());
  c->split = 0;
  CK(cudaStreamSynchronize(c->stream));
  return check_flags(c);
}

ds_status ds_set_time(ds_ctx *c, int tube, double Tm, long long nsteps) {
  if (!c || tube < 0 || tube >= c->ntubes || nsteps < 0 || !std::isfinite(Tm)) return DS_ERR_ARG;
  if (c->split) return fail(c, DS_ERR_STATE, "ds_set_time: a split step is in progress");
  if (!c->finalized) {
    if (c->clock_set.empty()) c->clock_set.assign(c->ntubes, {false, {0.0, 0LL}});
    c->clock_set[tube] = {true, {Tm, nsteps}};
    return DS_OK;
  }
  TubeState ts;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&ts, c->d_tstate + tube, sizeof ts, cudaMemcpyDeviceToHost));
  ts.Tm = Tm;
  ts.nstep = nsteps;
  CK(cudaMemcpy(c->d_tstate + tube, &ts, sizeof ts, cudaMemcpyHostToDevice));
  return DS_OK;
}

ds_status ds_idic_columns(const ds_params *p, int n, const double *x, int *col) {
  if (!p || n < 0 || (n > 0 && (!x || !col))) return DS_ERR_ARG;
  TubeDesc T;
  build_desc(*p, T);
  if (!(T.aw > 0) || !std::isfinite(T.aw)) return DS_ERR_ARG;
  const bool fast = p->precision == DS_PRECISION_FP32;
  const bool proper = (p->mode & DS_MODE_IDIC_PROPER) != 0;
  for (int i = 0; i < n; i++) {
    double v;
    if (fast) v = std::floor(std::fma(x[i], T.iaa, T.iab[0]));  // fast_idic_cell
    else if (proper) v = std::floor((x[i] - T.ox) / T.aw);     // ds_idic_cell, proper grid
    else v = std::trunc((x[i] - T.ox) / T.aw);                  // ds_idic_cell, the reference's int()
    col[i] = v < -2147483647.0 ? -2147483647 : (v > 2147483647.0 ? 2147483647 : (int)v);
  }
  return DS_OK;
}

ds_status ds_debug_force_lists(ds_ctx *c, int tube, int cap, int *count, int *nbr) {
  if (!c || tube < 0 || tube >= c->ntubes || cap < 0 || !count || (cap > 0 && !nbr)) return DS_ERR_ARG;
  if (!c->finalized) return fail(c, DS_ERR_STATE, "no resident state yet (call ds_step first)");
  if (!c->nbl) return fail(c, DS_ERR_UNSUPPORTED, "no recorded force lists (FP32 path with force lists only)");
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  const int n = T.seg_end[0] - T.seg_begin[0];
  if (n == 0) return DS_OK;
  ScratchDev tmp;
  int *dc = nullptr, *dn = nullptr;
  CK(tmp.alloc(&dc, (size_t)n));
  if (cap > 0) CK(tmp.alloc(&dn, (size_t)n * (size_t)cap));
  CK(cudaMemsetAsync(dc, 0, sizeof(int) * (size_t)n, c->stream));
  SweepArgs ag = sweep_args(c, c->d_ch_gas, (int)c->ch_gas.size());
  ag.nbl = c->nbl;
  ag.nbl_cnt = c->nbl_cnt;
  ag.nbl_walk = c->nbl_walk;
  ag.nbl_cap = c->nbl_cap;
  ds_launch_debug_force_lists(ag, tube, cap, dc, dn, c->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(count, dc, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  if (cap > 0) CK(cudaMemcpyAsync(nbr, dn, sizeof(int) * (size_t)n * (size_t)cap, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_get_gas(ds_ctx *c, int tube, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                     double *ax, double *ay, double *az, double *rho, double *p, double *e, int *ind) {
  double *f[NF] = {x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, nullptr, nullptr, nullptr};
  return get_species(c, tube, 0, f, ind);
}

ds_status ds_get_dust(ds_ctx *c, int tube, int species, double *x, double *y, double *z, double *vx, double *vy,
                      double *vz, double *rho, double *t_stop, int *ind) {
  if (species < 1) return fail(c, DS_ERR_ARG, "dust species are numbered from 1");
  double *f[NF] = {x, y, z, vx, vy, vz, nullptr, nullptr, nullptr, rho, nullptr, nullptr, nullptr, nullptr, t_stop};
  return get_species(c, tube, species, f, ind);
}

ds_status ds_download_gas(ds_ctx *c, double *x, double *y, double *z, double *vx, double *vy, double *vz, double *ax,
                          double *ay, double *az, double *rho, double *p, double *e, int *ind) {
  return ds_get_gas(c, 0, x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, ind);
}

ds_status ds_download_dust(ds_ctx *c, int species, double *x, double *y, double *z, double *vx, double *vy,
                           double *vz, double *rho, double *t_stop, int *ind) {
  return ds_get_dust(c, 0, species, x, y, z, vx, vy, vz, rho, t_stop, ind);
}

// ---------------------------------------------------------------------------
// Binary checkpoints of one tube: "DSCKPT01", the tube's ds_params, its clock
// (Tm, dt of the last step, step count), then per species the particle count
// and every field in caller order (the fifteen FP64 fields, then Ind).
// ---------------------------------------------------------------------------
namespace {
const char kCkptMagic[8] = {'D', 'S', 'C', 'K', 'P', 'T', '0', '1'};

struct FileCloser {
  FILE *f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};
}  // namespace

ds_status ds_checkpoint_params(const char *path, ds_params *p) {
  if (!path || !p) return DS_ERR_ARG;
  FileCloser F{fopen(path, "rb")};
  if (!F.f) return DS_ERR_IO;
  char magic[8];
  if (fread(magic, 1, 8, F.f) != 8 || memcmp(magic, kCkptMagic, 8) != 0) return DS_ERR_IO;
  if (fread(p, sizeof(ds_params), 1, F.f) != 1) return DS_ERR_IO;
  return DS_OK;
}

ds_status ds_save_tube(ds_ctx *c, int tube, const char *path) {
  if (!c || !path) return DS_ERR_ARG;
  if (!c->finalized) return fail(c, DS_ERR_STATE, "no resident state yet (call ds_step first)");
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  double Tm = 0, dt = 0;
  long long ns = 0;
  ds_status st = ds_get_time(c, tube, &Tm, &dt, &ns);
  if (st != DS_OK) return st;
  const TubeDesc &T = c->tdesc[tube];
  const int nsp = 1 + c->params[tube].n_dust;
  FileCloser F{fopen(path, "wb")};
  if (!F.f) return fail(c, DS_ERR_IO, std::string("cannot write ") + path);
  bool ok = fwrite(kCkptMagic, 1, 8, F.f) == 8 && fwrite(&c->params[tube], sizeof(ds_params), 1, F.f) == 1 &&
            fwrite(&Tm, sizeof Tm, 1, F.f) == 1 && fwrite(&dt, sizeof dt, 1, F.f) == 1 &&
            fwrite(&ns, sizeof ns, 1, F.f) == 1 && fwrite(&nsp, sizeof nsp, 1, F.f) == 1;
  for (int s = 0; ok && s < nsp; s++) {
    const long long n = T.seg_end[s] - T.seg_begin[s];
    std::vector<double> buf((size_t)NF * (size_t)(n > 0 ? n : 1));
    std::vector<int> ind((size_t)(n > 0 ? n : 1));
    double *f[NF];
    for (int k = 0; k < NF; k++) f[k] = buf.data() + (size_t)k * (size_t)n;
    if (n > 0 && (st = get_species(c, tube, s, f, ind.data())) != DS_OK) return st;
    ok = fwrite(&n, sizeof n, 1, F.f) == 1 &&
         (n == 0 || (fwrite(buf.data(), sizeof(double), (size_t)NF * n, F.f) == (size_t)NF * n &&
                     fwrite(ind.data(), sizeof(int), (size_t)n, F.f) == (size_t)n));
  }
  if (!ok) return fail(c, DS_ERR_IO, std::string("short write to ") + path);
  return DS_OK;
}

}  // extern "C"

// The first run parameter that differs between a checkpoint's parameters and
// the tube's, by name, or nullptr.  Compared: everything that changes the
// physics, the grids or the step (box, equation of state, h, cell widths,
// fixed step, AV constants, gamma, sound speed, species and their constants,
// mode bits, precision, stencil, CFL number, empty-cell defaults, list skin).  Not
// compared: T_end and T_out (a resumed run may go further), Maximum_particle
// and Particle_on_length (initial conditions only), list_depth and force_list
// (tuning choices that leave the results unchanged).
static const char *checkpoint_param_mismatch(const ds_params &a, const ds_params &b) {
#define DS_CK_FIELD(f) \
  if (!(a.f == b.f)) return #f;
  DS_CK_FIELD(X_min) DS_CK_FIELD(X_max) DS_CK_FIELD(Y_min) DS_CK_FIELD(Y_max) DS_CK_FIELD(Z_min)
  DS_CK_FIELD(Z_max) DS_CK_FIELD(Type_of_state) DS_CK_FIELD(h) DS_CK_FIELD(Coeff_h_dust_cell) DS_CK_FIELD(tau)
  DS_CK_FIELD(alpha) DS_CK_FIELD(beta) DS_CK_FIELD(eps) DS_CK_FIELD(Gam_g) DS_CK_FIELD(Speed_of_sound_gas)
  DS_CK_FIELD(n_dust) DS_CK_FIELD(mode) DS_CK_FIELD(precision) DS_CK_FIELD(stencil) DS_CK_FIELD(cell_w)
  DS_CK_FIELD(idic_w) DS_CK_FIELD(cfl) DS_CK_FIELD(t_empty) DS_CK_FIELD(list_skin)
  for (int k = 0; k < DS_MAX_DUST && k < a.n_dust; k++) {
    DS_CK_FIELD(mass_ratio[k]) DS_CK_FIELD(R_dust[k]) DS_CK_FIELD(t_stop_const[k]) DS_CK_FIELD(eps_empty[k])
  }
#undef DS_CK_FIELD
  return nullptr;
}

extern "C" {

ds_status ds_load_tube(ds_ctx *c, int tube, const char *path) {
  if (!c || !path) return DS_ERR_ARG;
  if (tube < 0 || tube >= c->ntubes) return fail(c, DS_ERR_ARG, "bad tube index");
  FileCloser F{fopen(path, "rb")};
  if (!F.f) return fail(c, DS_ERR_IO, std::string("cannot read ") + path);
  char magic[8];
  ds_params P;
  double Tm = 0, dt = 0;
  long long ns = 0;
  int nsp = 0;
  if (fread(magic, 1, 8, F.f) != 8 || memcmp(magic, kCkptMagic, 8) != 0 || fread(&P, sizeof P, 1, F.f) != 1 ||
      fread(&Tm, sizeof Tm, 1, F.f) != 1 || fread(&dt, sizeof dt, 1, F.f) != 1 || fread(&ns, sizeof ns, 1, F.f) != 1 ||
      fread(&nsp, sizeof nsp, 1, F.f) != 1)
    return fail(c, DS_ERR_IO, std::string("not a checkpoint: ") + path);
  if (nsp != 1 + c->params[tube].n_dust) return fail(c, DS_ERR_ARG, "checkpoint species count differs from the tube's");
  const char *differs = checkpoint_param_mismatch(P, c->params[tube]);
  if (differs)
    return fail(c, DS_ERR_ARG, std::string("checkpoint was saved with a different ") + differs + " than the tube's");
  // Every species is read and checked before any is written, so a bad file
  // leaves the tube as it was.
  std::vector<long long> counts(nsp);
  std::vector<std::vector<double>> bufs(nsp);
  std::vector<std::vector<int>> inds(nsp);
  for (int s = 0; s < nsp; s++) {
    long long n = 0;
    if (fread(&n, sizeof n, 1, F.f) != 1 || n < 0 || n > INT32_MAX) return fail(c, DS_ERR_IO, "truncated checkpoint");
    counts[s] = n;
    bufs[s].resize((size_t)NF * (size_t)(n > 0 ? n : 1));
    inds[s].resize((size_t)(n > 0 ? n : 1));
    if (n > 0 && (fread(bufs[s].data(), sizeof(double), (size_t)NF * n, F.f) != (size_t)NF * n ||
                  fread(inds[s].data(), sizeof(int), (size_t)n, F.f) != (size_t)n))
      return fail(c, DS_ERR_IO, "truncated checkpoint");
  }
  for (int s = 0; s < nsp; s++) {
    const long long n = counts[s];
    const double *f[NF];
    for (int k = 0; k < NF; k++) f[k] = bufs[s].data() + (size_t)k * (size_t)n;
    ds_status st = set_species(c, tube, s, (int)n, f, inds[s].data());
    if (st != DS_OK) return st;
  }
  if (c->finalized) {  // resident context: set the clock now
    TubeState ts;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&ts, c->d_tstate + tube, sizeof ts, cudaMemcpyDeviceToHost));
    ts.Tm = Tm;
    ts.nstep = ns;
    CK(cudaMemcpy(c->d_tstate + tube, &ts, sizeof ts, cudaMemcpyHostToDevice));
  } else {
    if (c->clock_set.empty()) c->clock_set.assign(c->ntubes, {false, {0.0, 0LL}});
    c->clock_set[tube] = {true, {Tm, ns}};
  }
  return DS_OK;
}

ds_status ds_get_time(ds_ctx *c, int tube, double *Tm, double *dt_last, long long *nsteps) {
  if (!c || tube < 0 || tube >= c->ntubes) return DS_ERR_ARG;
  if (!c->finalized) {  // the clock a checkpoint set, else zero
    const bool set = !c->clock_set.empty() && c->clock_set[tube].first;
    if (Tm) *Tm = set ? c->clock_set[tube].second.first : 0.0;
    if (dt_last) *dt_last = 0;
    if (nsteps) *nsteps = set ? c->clock_set[tube].second.second : 0;
    return DS_OK;
  }
  TubeState ts;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(&ts, c->d_tstate + tube, sizeof(ts), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (Tm) *Tm = ts.Tm;
  if (dt_last) *dt_last = ts.dt;
  if (nsteps) *nsteps = ts.nstep;
  return DS_OK;
}

ds_status ds_debug_cells(ds_ctx *c, int tube, int species, int *cell_key, int *head, int *next, int *ncand,
                         int *nnb, int *ncells) {
  if (c && c->split) return fail(c, DS_ERR_STATE, "a split step is in progress (call ds_step_complete first)");
  if (!c) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  if (tube < 0 || tube >= c->ntubes || species < 0 || species > c->params[tube].n_dust)
    return fail(c, DS_ERR_ARG, "bad tube or species");
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  const int b = T.seg_begin[species], n = T.seg_end[species] - b;
  if (ncells) *ncells = T.ncells;
  enqueue_sort(c, true);  // lists for the current positions, caller-index order
  if (ncand || nnb) {
    std::vector<Chunk> ch;
    add_chunks(ch, tube, species, b, b + n);
    ScratchDev tmp;
    Chunk *d_ch = nullptr;
    if (!ch.empty()) {
      CK(tmp.alloc(&d_ch, ch.size()));
      CK(cudaMemcpyAsync(d_ch, ch.data(), sizeof(Chunk) * ch.size(), cudaMemcpyHostToDevice, c->stream));
      SweepArgs a = sweep_args(c, d_ch, (int)ch.size());
      ds_launch_counts64(a, (c->params[tube].mode & DS_MODE_H_PER_PARTICLE) != 0, c->any_proper, c->stream);
      CK(cudaGetLastError());
    }
    if (ncand && n) CK(cudaMemcpyAsync(ncand, c->ncand + b, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    if (nnb && n) CK(cudaMemcpyAsync(nnb, c->nnb + b, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (cell_key || head || next) {
    ScratchDev tmp;
    int *dh = nullptr, *dn = nullptr, *dk = nullptr;
    CK(tmp.alloc(&dh, (size_t)T.ncells + 1));
    CK(tmp.alloc(&dn, (size_t)n));
    CK(tmp.alloc(&dk, (size_t)n));
    ds_launch_debug_lists(c->d_tubes, tube, species, n, T.ncells, c->buf[c->parity].view(), c->cell_start, 0, dh,
                          dn, dk, c->stream);
    CK(cudaGetLastError());
    if (head) CK(cudaMemcpyAsync(head, dh, sizeof(int) * (T.ncells + 1), cudaMemcpyDeviceToHost, c->stream));
    if (next && n) CK(cudaMemcpyAsync(next, dn, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    if (cell_key && n) CK(cudaMemcpyAsync(cell_key, dk, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return DS_OK;
}

ds_status ds_step_lists(ds_ctx *c, int tube, int species, int *head, int *next, int *ncells) {
  if (!c) return DS_ERR_ARG;
  if (!c->finalized) return fail(c, DS_ERR_STATE, "no resident state yet (call ds_step first)");
  if (tube < 0 || tube >= c->ntubes || species < 0 || species > c->params[tube].n_dust)
    return fail(c, DS_ERR_ARG, "bad tube or species");
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  const int n = T.seg_end[species] - T.seg_begin[species];
  if (ncells) *ncells = T.ncells;
  if (!head && !next) return DS_OK;
  ScratchDev tmp;
  int *dh = nullptr, *dn = nullptr, *dk = nullptr;
  CK(tmp.alloc(&dh, (size_t)T.ncells + 1));
  CK(tmp.alloc(&dn, (size_t)n));
  CK(tmp.alloc(&dk, (size_t)n));
  // the slots still hold the last sort's order (the step moves particles in place)
  ds_launch_debug_lists(c->d_tubes, tube, species, n, T.ncells, c->buf[c->parity].view(), c->cell_start, c->last_xl,
                        dh, dn, dk, c->stream);
  CK(cudaGetLastError());
  if (head) CK(cudaMemcpyAsync(head, dh, sizeof(int) * (T.ncells + 1), cudaMemcpyDeviceToHost, c->stream));
  if (next && n) CK(cudaMemcpyAsync(next, dn, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_get_fields(ds_ctx *c, int tube, int species, double *const *fields, int *ind) {
  if (!c || !fields) return DS_ERR_ARG;
  return get_species(c, tube, species, fields, ind);
}

ds_status ds_debug_idic(ds_ctx *c, int tube, int species, int *count, double *cells, int *ncells) {
  if (!c) return DS_ERR_ARG;
  if (!c->finalized) return fail(c, DS_ERR_STATE, "no resident state yet (call ds_step first)");
  if (tube < 0 || tube >= c->ntubes || species < 0 || species > c->params[tube].n_dust)
    return fail(c, DS_ERR_ARG, "bad tube or species");
  CK(cudaSetDevice(c->device));
  const TubeDesc &T = c->tdesc[tube];
  const int n = T.n_idic + 1, k0 = T.idic_base[species];
  if (ncells) *ncells = n;
  CK(cudaStreamSynchronize(c->stream));
  if (count) CK(cudaMemcpy(count, c->ca.cnt + k0, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (cells) {
    const double *arr[12] = {c->ca.vx, c->ca.vy, c->ca.vz, c->ca.a0, c->ca.a1, c->ca.a2,
                             c->ca.nvx, c->ca.nvy, c->ca.nvz, c->ca.px, c->ca.py, c->ca.pz};
    for (int k = 0; k < 12; k++)
      CK(cudaMemcpy(cells + (size_t)k * n, arr[k] + k0, sizeof(double) * n, cudaMemcpyDeviceToHost));
  }
  return DS_OK;
}

ds_status ds_conservation(ds_ctx *c, int tube, double *out6) {
  if (!c || !out6 || tube < 0 || tube >= c->ntubes) return DS_ERR_ARG;
  ds_status st = finalize(c);
  if (st != DS_OK) return st;
  CK(cudaSetDevice(c->device));
  ds_launch_conservation(c->d_tubes, tube, c->buf[c->parity].view(), c->d_cons, c->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out6, c->d_cons, sizeof(double) * 6, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return DS_OK;
}

ds_status ds_memory_bytes(ds_ctx *c, long long *bytes) {
  if (!c || !bytes) return DS_ERR_ARG;
  *bytes = c->bytes;
  return DS_OK;
}

ds_status ds_last_error(ds_ctx *c, int *device_flags, char *msg, int msglen) {
  if (!c) return DS_ERR_ARG;
  if (device_flags) {
    *device_flags = 0;
    if (c->finalized) {
      CK(cudaSetDevice(c->device));
      CK(cudaMemcpy(device_flags, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
    }
  }
  if (msg && msglen > 0) {
    strncpy(msg, c->msg.c_str(), (size_t)msglen - 1);
    msg[msglen - 1] = 0;
  }
  return DS_OK;
}

ds_status ds_host_alloc(void **ptr, long long bytes) {
  if (!ptr || bytes < 0) return DS_ERR_ARG;
  return cudaMallocHost(ptr, (size_t)(bytes ? bytes : 1)) == cudaSuccess ? DS_OK : DS_ERR_NOMEM;
}

ds_status ds_host_free(void *ptr) { return cudaFreeHost(ptr) == cudaSuccess ? DS_OK : DS_ERR_CUDA; }

void ds_destroy(ds_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int p = 0; p < 2; p++) {
    if (c->graph[p]) cudaGraphExecDestroy(c->graph[p]);
    if (c->hgraph[p]) cudaGraphExecDestroy(c->hgraph[p]);
  }
  cudaEvent_t evs[] = {c->e_fork, c->e_up, c->e_dens, c->e_force, c->e_join};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->e_wfork) cudaEventDestroy(c->e_wfork);
  if (c->e_wjoin) cudaEventDestroy(c->e_wjoin);
  if (c->wstream) cudaStreamDestroy(c->wstream);
  for (int k = 0; k <= DS_NPHASE; k++)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  for (cudaEvent_t e : c->tev) cudaEventDestroy(e);
  for (void *p : c->allocs) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

}  // extern "C"

// ===========================================================================
// Allocation-free cell lists (ds_cell_lists_noalloc)
//
// For callers that cannot call cudaMalloc: a host whose device memory is all
// handed to its own pool allocator, or code that runs where an allocation
// would be an error or would stall the device (cudaMalloc can synchronise the
// whole device).  The sort's scratch (keys, values, their alternates and the
// radix histograms) lives in the file-scope array below instead of in
// context-owned memory.  It is sized for DS_NOALLOC_MAX_PARTICLES particles
// (about 4.7 MB), and every GPU that loads this library holds it until the
// process exits.  All calls share it: calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it.  Every scratch
// word a call reads has been written earlier in the same call, so nothing
// needs clearing between calls.
//
// The array belongs to this library's device code, which the CUDA runtime
// loads into a device's context only when first used there (lazy module
// loading is the default).  That load takes device memory through the driver,
// and the first call on each device is what triggers it, together with the
// address set-up below.  A host that hands the rest of the memory to its pool
// makes that first call before it does so, and before any stream capture.
// ===========================================================================
namespace {

constexpr int kNaTile = DS_RADIX_TILE;  // keys per radix tile (ds_sort.cu)
constexpr int kNaMax = DS_NOALLOC_MAX_PARTICLES;
constexpr size_t kNaHistWords = DS_RADIX_BINS * (size_t)((kNaMax + kNaTile - 1) / kNaTile) + DS_RADIX_BINS;
constexpr size_t kNaWords = 4 * (size_t)kNaMax + kNaHistWords;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

std::mutex g_noalloc_mu;

// The scratch array's device address, per device, with the ID of the context
// it was resolved in.  Context IDs are unique for the life of the process, so
// a context re-created after cudaDeviceReset does not match a stale entry.
struct NoallocSlot {
  unsigned long long ctx_id;
  uint32_t *ptr;
};
NoallocSlot g_noalloc_slot[256] = {};

typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

// ID of the context current on this thread, 0 if none is current or the driver
// does not offer the query.  The two driver functions are fetched through the
// runtime, so the library does not link libcuda itself.  Caller holds
// g_noalloc_mu.
unsigned long long current_ctx_id() {
  static bool looked_up = false;
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!looked_up) {
    looked_up = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)f;
  }
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// The device address of the scratch array for the current device.  The host
// symbol is only a stand-in: the set-up resolves it with cudaGetSymbolAddress
// on the first call made with the device current, and again whenever the
// device's context has changed since (a cudaDeviceReset in between).  Where the
// context cannot be identified, it is resolved on every call.
ds_status noalloc_scratch(uint32_t **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return DS_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocSlot &slot = g_noalloc_slot[dev];
  const unsigned long long id = current_ctx_id();
  if (slot.ptr && id != 0 && slot.ctx_id == id) {
    *out = slot.ptr;
    return DS_OK;
  }
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return DS_ERR_CUDA;
  slot.ptr = (uint32_t *)p;
  slot.ctx_id = current_ctx_id();  // the context is current now
  *out = slot.ptr;
  return DS_OK;
}

__global__ void k_na_keys(const TubeDesc T, const double *x, const double *y, const double *z, int n,
                          int *cell_key, uint32_t *kin, uint32_t *vin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int raw = ds_raw_key(T, x[i], y[i], z[i]);
  cell_key[i] = raw;
  int local;
  if (!(T.mode & M_GRID_PROPER))
    local = (raw >= 0 && raw <= T.ncells) ? raw : T.ncells + 1;  // kernel.cu:1950
  else
    local = raw >= 0 ? raw : T.ncells + 1;
  kin[i] = (uint32_t)local;
  vin[i] = (uint32_t)i;
}

__global__ void k_na_fill(int *a, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// head[c] = first particle of cell c, next[p] = following particle of p's cell
// in ascending index, -1 at the end and for unlisted particles.
__global__ void k_na_lists(const uint32_t *skey, const uint32_t *sidx, int n, int ncells, int *head, int *next) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint32_t k = skey[q];
  const int p = (int)sidx[q];
  if ((int)k > ncells) {
    next[p] = -1;
    return;
  }
  if (q == 0 || skey[q - 1] != k) head[k] = p;
  next[p] = (q + 1 < n && skey[q + 1] == k) ? (int)sidx[q + 1] : -1;
}

}  // namespace

extern "C" ds_status ds_cell_lists_noalloc(const ds_params *p, int n, const double *d_x, const double *d_y,
                                           const double *d_z, int *d_cell_key, int *d_head, int head_len,
                                           int *d_next, void *stream) {
  if (!p || n < 0 || !d_head) return DS_ERR_ARG;
  if (n > kNaMax) return DS_ERR_ARG;  // beyond the static scratch
  if (n > 0 && (!d_x || !d_y || !d_z || !d_cell_key || !d_next)) return DS_ERR_ARG;
  if (check_params(nullptr, *p) != DS_OK) return DS_ERR_ARG;
  TubeDesc T;
  build_desc(*p, T);
  if (head_len < T.ncells + 1) return DS_ERR_ARG;
  if (ds_radix_scratch_words(n > 0 ? n : 1) > kNaHistWords) return DS_ERR_ARG;
  uint32_t *s = nullptr;
  ds_status st = noalloc_scratch(&s);
  if (st != DS_OK) return st;
  uint32_t *kin = s, *vin = s + kNaMax, *kalt = s + 2 * (size_t)kNaMax, *valt = s + 3 * (size_t)kNaMax;
  uint32_t *hist = s + 4 * (size_t)kNaMax;
  cudaStream_t cs = (cudaStream_t)stream;
  const int nh = T.ncells + 1;
  // Each launch's own status is checked; the thread's last-error state is not
  // read, so an earlier failure of someone else's call is not reported here.
  cudaError_t e = ds_launch(k_na_fill, dim3((nh + 255) / 256), dim3(256), cs, d_head, nh, -1);
  if (n > 0) {
    bool alt = false;
    if (e == cudaSuccess)
      e = ds_launch(k_na_keys, dim3((n + 255) / 256), dim3(256), cs, T, d_x, d_y, d_z, n, d_cell_key, kin, vin);
    if (e == cudaSuccess) e = ds_radix_sort(kin, vin, kalt, valt, n, bits_for((long long)T.ncells + 2), hist, cs, &alt);
    if (e == cudaSuccess)
      e = ds_launch(k_na_lists, dim3((n + 255) / 256), dim3(256), cs, (const uint32_t *)(alt ? kalt : kin),
                    (const uint32_t *)(alt ? valt : vin), n, T.ncells, d_head, d_next);
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // the failed launch recorded e there; it is reported by the status
    return DS_ERR_CUDA;
  }
  return DS_OK;
}
