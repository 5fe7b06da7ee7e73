// ds_common.cuh -- device-side data layout and helpers shared by the kernels.
//
// Layout in HBM (one context = a batch of tubes; a single tube is a batch of 1):
//   particles of every (tube, species) segment packed tube-major, species-minor,
//   as SoA FP64 arrays in SORTED order (cell key, then caller index); a slot's
//   caller index is pid[slot].  Two copies of every persistent field (A/B) are
//   swapped by the per-step reorder.  Keys of all segments live in one key
//   space (key_base per segment), so a single stable radix sort orders all
//   tubes and species at once and cell_start[] gives every cell's slot range.
#pragma once
#include <cstdint>

#define DS_MAXD 4            // dust species per tube
#define DS_MAXS (1 + DS_MAXD)  // species per tube (gas + dust)

// mode bits (same values as the public header)
#define M_PER_Y 0x0001
#define M_PER_Z 0x0002
#define M_HPP 0x0004
#define M_TSTOP_CONST 0x0008
#define M_GAS_ACC_P 0x0010
#define M_REF_COUPLING 0x0020
#define M_REF_EPS_GUARD 0x0040
#define M_REF_SOLVE2 0x0080
#define M_CFL 0x0100
#define M_DUST_RHO 0x0200
#define M_GRID_PROPER 0x0400
#define M_IDIC_PROPER 0x0800

// One tube's constants, built on the host (ds_api.cu) and kept in device memory.
struct TubeDesc {
  // neighbour grid (kernel.cu:1767-1778; proper grid for the extensions)
  double ox, oy, oz;   // Clx, Cly, Clz
  double wx, wy, wz;   // cell widths (Clh in the reference)
  double Ly, Lz;       // periodic lengths
  double ymax, zmax;   // Y_max, Z_max (periodic wrap bounds)
  int Cnx, Cny, Cnz;   // int((max - min) / Clh)
  int nx, ny, nz;      // cells per axis (proper grid)
  int sy, sz;          // key strides
  int ncells;          // Number_of_fihd_cells (reference) / nx*ny*nz (proper)
  int mode;
  // IDIC grid (kernel.cu:1577-1582)
  double aw;
  int Nax, Nay, Naz, asy, asz, n_idic;  // cells 0..n_idic are valid (kernel.cu:2060)
  int anx, any_, anz, pad0;
  // physics
  double h, alpha, beta, eps, gam, cs, tau, cfl, t_end, t_empty;
  int type_of_state, n_dust, precision, pad1;
  double mass_ratio[DS_MAXD], R_dust[DS_MAXD], t_stop_const[DS_MAXD], eps_empty[DS_MAXD];
  // FP32 prefilter / FP32 path coordinates: absolute coordinates relative to
  // (fx, fy, fz) in the reference grid; offsets from the own cell origin in
  // the proper grid (cellrel = 1)
  double fx, fy, fz;
  float pre_abs;   // absolute slack of the FP32 distance prefilter
  int cellrel;
  // segments
  int seg_begin[DS_MAXS], seg_end[DS_MAXS];
  int key_base[DS_MAXS];   // neighbour keys of species s: key_base[s] + 0..ncells+1
  int idic_base[DS_MAXS];  // IDIC keys of species s:      idic_base[s] + 0..n_idic+1
};

struct TubeState {
  double Tm;           // simulation time
  double dt;           // step size of the current step
  unsigned long long dtmin_bits;  // CFL min-reduction (bits of a positive double)
  long long nstep;
  int active;          // Tm < T_end at the start of the step
  int pad;
};

// A block-sized chunk of one segment: blocks of the per-phase kernels walk a
// table of these (persistent, grid-stride), so one launch covers all tubes.
struct Chunk {
  int tube, species, begin, end;
};

struct DevState {  // pointers into one buffer set (A or B)
  double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *rho, *p, *e, *m, *h, *ts;
  int *ind, *pid;
};

// ---------------------------------------------------------------------------
// Kernel functions, written in the reference's operation order so that the
// FP64 path (compiled without FMA contraction) equals the reference's CPU
// build bit for bit.
// ---------------------------------------------------------------------------
#define DS_PI_REF 3.14159265  // the reference's truncated constant (kernel.cu:14)

// M4 cubic spline, kernel.cu:12-23
__device__ __forceinline__ double ds_W(double r, double h) {
  const double c = (double)1 / (DS_PI_REF);
  double k = fabs(r) / h, tmp1 = 0.0;
  if (k < 1.0) tmp1 = 1.0 - 1.5 * k * k + 0.75 * k * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = 0.25 * (2.0 - k) * (2.0 - k) * (2.0 - k);
  if (k > 2.0) tmp1 = 0.0;
  return c / (h * h * h) * tmp1;
}

// signed derivative, kernel.cu:25-39 (later matching branch wins)
__device__ __forceinline__ double ds_dW(double r, double h) {
  const double c = (double)1 / (DS_PI_REF);
  double k = r / h, tmp1 = 0.0;
  if ((k >= -2.0) && (k <= -1.0)) tmp1 = 0.75 * (2.0 + k) * (2.0 + k);
  if ((k > -1.0) && (k < 0)) tmp1 = -3.0 * k - 2.25 * k * k;
  if ((k >= 0) && (k <= 1.0)) tmp1 = -3.0 * k + 2.25 * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = -0.75 * (2.0 - k) * (2.0 - k);
  if ((k > 2.0) || (k < -2.0)) tmp1 = 0.0;
  return c / (h * h * h * h) * tmp1;
}

// kernel.cu:92-97
__device__ __forceinline__ double ds_eq_state(double rho, double e, int type, double gam, double cs) {
  if (type == 1) return cs * cs * rho;
  return rho * e * (gam - 1);
}

// Per-axis cell of a position in the proper grid: floor, periodic axes clamped.
__device__ __forceinline__ void ds_proper_cell(const TubeDesc &T, double x, double y, double z, int &ix,
                                               int &iy, int &iz) {
  ix = (int)floor((x - T.ox) / T.wx);
  iy = (int)floor((y - T.oy) / T.wy);
  iz = (int)floor((z - T.oz) / T.wz);
  if (T.mode & M_PER_Y) { iy = iy < 0 ? 0 : iy; iy = iy >= T.ny ? T.ny - 1 : iy; }
  if (T.mode & M_PER_Z) { iz = iz < 0 ? 0 : iz; iz = iz >= T.nz ? T.nz - 1 : iz; }
}

// Raw neighbour-cell key, kernel.cu:1949 / IDIC.h:28 (int() truncation).
// Proper grid: -1 when an axis is out of range.
__device__ __forceinline__ int ds_raw_key(const TubeDesc &T, double x, double y, double z) {
  if (!(T.mode & M_GRID_PROPER))
    return (int)((x - T.ox) / T.wx) + ((int)((y - T.oy) / T.wx)) * T.Cnx +
           ((int)((z - T.oz) / T.wx)) * T.Cnx * T.Cny;
  int ix, iy, iz;
  ds_proper_cell(T, x, y, z, ix, iy, iz);
  if (ix < 0 || ix >= T.nx || iy < 0 || iy >= T.ny || iz < 0 || iz >= T.nz) return -1;
  return ix + iy * T.sy + iz * T.sz;
}

// Raw IDIC cell, kernel.cu:2116; -1 when outside [0, n_idic] (the reference
// has no check there).
__device__ __forceinline__ int ds_idic_cell(const TubeDesc &T, double x, double y, double z) {
  int c;
  if (!(T.mode & M_IDIC_PROPER)) {
    c = (int)((x - T.ox) / T.aw) + ((int)((y - T.oy) / T.aw)) * T.Nax +
        ((int)((z - T.oz) / T.aw)) * T.Nax * T.Nay;
  } else {
    int ix = (int)floor((x - T.ox) / T.aw);
    int iy = (int)floor((y - T.oy) / T.aw);
    int iz = (int)floor((z - T.oz) / T.aw);
    if (ix < 0 || ix >= T.anx || iy < 0 || iy >= T.any_ || iz < 0 || iz >= T.anz) return -1;
    c = ix + iy * T.asy + iz * T.asz;
  }
  return (c < 0 || c > T.n_idic) ? -1 : c;
}

// The 27 neighbour cells of a particle, in the reference's launch order
// (k = x offset outer, l = y, g = z inner; kernel.cu:2014-2016) and with its
// validity test (IDIC.h:30-31).  Proper grid: per-axis range checks and
// periodic wrap; sy/sz are the image shifts of the neighbour cell and
// (cx, cy, cz) its offset in cells (for cell-relative FP32 coordinates).
struct Stencil {
  int ni;            // reference grid: raw key of the own cell
  int ix, iy, iz;    // proper grid: own cell
};

__device__ __forceinline__ void ds_stencil_init(const TubeDesc &T, double x, double y, double z, Stencil &s) {
  if (!(T.mode & M_GRID_PROPER)) {
    s.ni = ds_raw_key(T, x, y, z);
    s.ix = s.iy = s.iz = 0;
  } else {
    s.ni = 0;
    ds_proper_cell(T, x, y, z, s.ix, s.iy, s.iz);
  }
}

// offset o = 0..26 -> local cell (or -1) and image shifts
__device__ __forceinline__ int ds_stencil_cell(const TubeDesc &T, const Stencil &s, int o, double &shy,
                                               double &shz) {
  const int k = o / 9 - 1, l = (o / 3) % 3 - 1, g = o % 3 - 1;
  shy = 0.0;
  shz = 0.0;
  if (!(T.mode & M_GRID_PROPER)) {
    int Ci = s.ni + k + l * T.Cnx + g * T.Cnx * T.Cny;
    return ((Ci > -1) && (Ci < T.ncells)) ? Ci : -1;
  }
  int cx = s.ix + k, cy = s.iy + l, cz = s.iz + g;
  if (cx < 0 || cx >= T.nx) return -1;
  if (T.mode & M_PER_Y) {
    if (cy < 0) { cy += T.ny; shy = -T.Ly; }
    else if (cy >= T.ny) { cy -= T.ny; shy = T.Ly; }
  }
  if (T.mode & M_PER_Z) {
    if (cz < 0) { cz += T.nz; shz = -T.Lz; }
    else if (cz >= T.nz) { cz -= T.nz; shz = T.Lz; }
  }
  if (cy < 0 || cy >= T.ny || cz < 0 || cz >= T.nz) return -1;
  return cx + cy * T.sy + cz * T.sz;
}

// neighbour coordinate (with its image shift) minus ours, as the oracle does
__device__ __forceinline__ double ds_diff(double xj, double s, double xi) {
  return s != 0.0 ? (xj + s) - xi : xj - xi;
}

// Arguments shared by the sweep kernels.
struct SweepArgs {
  const TubeDesc *tubes;
  const TubeState *tstate;
  const Chunk *chunks;
  int nchunks;
  DevState st;
  const int *cell_start;    // [nkeys + 1]
  const float4 *pos32;      // prefilter / FP32 coordinates + h
  const float4 *vm32;       // FP32 vx, vy, vz, m
  float4 *hyd32;            // FP32 c, p/rho^2, rho, (unused) -- written by density
  double *cs64;             // sqrt(gam p / rho) per gas slot -- written by density
  double *pt64;             // p / (rho rho) per gas slot     -- written by density
  double *edot;             // energy rate per gas slot
  int *ncand, *nnb;         // optional counts (parity hook), indexed by slot
  const int *gas_slot_of_pid;  // slot of gas particle pid (index coupling)
  const int *gas_ind_pid;      // gas Ind by pid (index-coupled dust rho zeroing)
  TubeState *tstate_rw;
  int *flags;
};
