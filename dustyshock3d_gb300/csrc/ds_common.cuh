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

#include "ds_bits.cuh"

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
  int stencil;       // cells searched on each side at most (FP64 path: 1 or 2; FP32 path: 1..4)
  int xl;            // FP32 path: sub-cell x bits of the sort keys (key = cell << xl | x bin)
  double r1_hmax;    // particles and cells with h <= r1_hmax need only the 27 inner cells
  double reach_hmax; // proper grid: largest h whose cut-off 2h the stencil's cells cover
  double rw;         // 1 / (min cell width (1 - 1e-9)): a cut-off c needs ceil(c rw) cells per side
  double skin;       // FP32 path, list reuse: recorded cut-off 2 max(h_i, h_j) + skin (0: lists rebuilt every step)
  double inv_wx, inv_wy, inv_wz, inv_aw;  // reciprocal cell widths (FP32 path: no FP64 divisions)
  // FP32 path index maps, one FMA and one rounding conversion per axis (GB300's
  // FP64 pipe runs 2 lanes per SM per clock): fine x index floor(fma(x, kxa,
  // kxb)) = cell << xl | x bin; cells floor(fma(y, kya, kyb)), floor(fma(z, kza,
  // kzb)); IDIC cells floor(fma(coordinate, iaa, iab[axis]))
  double kxa, kxb, kya, kyb, kza, kzb, iaa, iab[3];
  const double *orig;  // FP32 path: FP64 origins of the nbx x-blocks, the ny y cells, the nz z cells
  int nbx;
  int64_t wrap_key[4];  // FP32 path: ds_order_key of oy, ymax, oz, zmax (periodic wrap on the integer pipe)
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
  int rebuild;         // list reuse: this step sorts, walks and records the lists (1 without reuse)
  unsigned disp_bits;  // list reuse: largest bound over nearby cell pairs (bits of a float >= 0)
  int built;           // list reuse: lists recorded since the context's state was last replaced
  unsigned gdev_bits;  // list reuse: largest distance of a displacement from its cell's mean (float bits)
  unsigned mlo[3], mhi[3];  // list reuse: box of the cells' mean displacements (order-preserving bits)
  long long nrebuild;  // list reuse: steps that sorted and recorded
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

// ds_dW with its normalisation c/(h*h*h*h) precomputed by the caller (the
// same double, so the same result)
__device__ __forceinline__ double ds_dW_n(double r, double h, double norm) {
  double k = r / h, tmp1 = 0.0;
  if ((k >= -2.0) && (k <= -1.0)) tmp1 = 0.75 * (2.0 + k) * (2.0 + k);
  if ((k > -1.0) && (k < 0)) tmp1 = -3.0 * k - 2.25 * k * k;
  if ((k >= 0) && (k <= 1.0)) tmp1 = -3.0 * k + 2.25 * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = -0.75 * (2.0 - k) * (2.0 - k);
  if ((k > 2.0) || (k < -2.0)) tmp1 = 0.0;
  return norm * tmp1;
}

// ds_W with its normalisation c/(h*h*h) precomputed
__device__ __forceinline__ double ds_W_n(double r, double h, double norm) {
  double k = fabs(r) / h, tmp1 = 0.0;
  if (k < 1.0) tmp1 = 1.0 - 1.5 * k * k + 0.75 * k * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = 0.25 * (2.0 - k) * (2.0 - k) * (2.0 - k);
  if (k > 2.0) tmp1 = 0.0;
  return norm * tmp1;
}

__device__ __forceinline__ double ds_W_norm(double h) { return ((double)1 / (DS_PI_REF)) / (h * h * h); }
__device__ __forceinline__ double ds_dW_norm(double h) { return ((double)1 / (DS_PI_REF)) / (h * h * h * h); }

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

// FP32 path: fine x index of the keys (the x cell << xl | the x bin within it)
// and the proper cell, from the index maps (no FP64 division; the FP32 path's
// keys, and so its sorted cells, come from these).
__device__ __forceinline__ int ds_fast_fine_x(const TubeDesc &T, double x) {
  return __double2int_rd(fma(x, T.kxa, T.kxb));
}
__device__ __forceinline__ void ds_fast_proper_cell(const TubeDesc &T, double x, double y, double z, int &ix,
                                                    int &iy, int &iz) {
  ix = ds_fast_fine_x(T, x) >> T.xl;  // arithmetic shift: floor division
  iy = __double2int_rd(fma(y, T.kya, T.kyb));
  iz = __double2int_rd(fma(z, T.kza, T.kzb));
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

// Own cell of a slot on the FP32 path: decoded from its sorted key -- the cell
// its FP32 coordinates are relative to -- or, for a particle outside the grid
// (orphan bucket), from its position as the FP32 keys compute it.
__device__ __forceinline__ void ds_stencil_from_key(const TubeDesc &T, int local, double x, double y, double z,
                                                    Stencil &s) {
  s.ni = 0;
  if (local < T.ncells) {
    s.ix = local % T.nx;
    s.iy = (local / T.nx) % T.ny;
    s.iz = local / (T.nx * T.ny);
  } else {
    ds_fast_proper_cell(T, x, y, z, s.ix, s.iy, s.iz);
  }
}

// Offset o of the (2r+1)^3 stencil, in the reference's launch order (k = x
// offset outer, l = y, g = z inner): local cell (or -1), image shifts and the
// cell offsets (k, l, g).  For r = 1 this is the reference's 27-offset loop;
// the 27 inner offsets of r = 2 come in the same relative order.
__device__ __forceinline__ int ds_stencil_cell(const TubeDesc &T, const Stencil &s, int r, int o, double &shy,
                                               double &shz, int &k, int &l, int &g) {
  const int w = 2 * r + 1;
  k = o / (w * w) - r;
  l = (o / w) % w - r;
  g = o % w - r;
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

// FP32 cell widths and periodic lengths of a tube, converted once per thread
// so that the per-candidate shifts below cost no FP64 work.
struct Shift32 {
  float wx, wy, wz, Ly, Lz;
};

__device__ __forceinline__ Shift32 ds_shift32_init(const TubeDesc &T) {
  return Shift32{(float)T.wx, (float)T.wy, (float)T.wz, (float)T.Ly, (float)T.Lz};
}

// FP32 shift that brings the FP32 coordinates of the neighbour cell at
// offsets (k, l, g) into ours: whole cell widths when coordinates are
// cell-relative (this also applies the periodic image), the periodic image
// shift when they are tube-relative on a proper grid, none on the reference
// grid.  The image shift is +-(float)L, which equals (float)(+-L), the FP64
// image shift rounded once.
__device__ __forceinline__ void ds_shift32(const TubeDesc &T, const Stencil &S, const Shift32 &f, int k, int l,
                                           int g, float &sx, float &sy, float &sz) {
  if (T.cellrel) {
    sx = (float)k * f.wx;
    sy = (float)l * f.wy;
    sz = (float)g * f.wz;
    return;
  }
  sx = sy = sz = 0.0f;
  if (!(T.mode & M_GRID_PROPER)) return;
  if (T.mode & M_PER_Y) {
    const int cy = S.iy + l;
    sy = cy < 0 ? -f.Ly : (cy >= T.ny ? f.Ly : 0.0f);
  }
  if (T.mode & M_PER_Z) {
    const int cz = S.iz + g;
    sz = cz < 0 ? -f.Lz : (cz >= T.nz ? f.Lz : 0.0f);
  }
}

// Image shifts of the neighbour cell at offsets (l, g) from the own cell.
__device__ __forceinline__ void ds_wrap_shift(const TubeDesc &T, const Stencil &S, int l, int g, double &shy,
                                              double &shz) {
  shy = 0.0;
  shz = 0.0;
  if (!(T.mode & M_GRID_PROPER)) return;
  if (T.mode & M_PER_Y) {
    const int cy = S.iy + l;
    shy = cy < 0 ? -T.Ly : (cy >= T.ny ? T.Ly : 0.0);
  }
  if (T.mode & M_PER_Z) {
    const int cz = S.iz + g;
    shz = cz < 0 ? -T.Lz : (cz >= T.nz ? T.Lz : 0.0);
  }
}

// Offset code of a list entry: (k, l, g) in [-2, 2]^3 as (k+2)*25+(l+2)*5+(g+2),
// increasing in the reference's visiting order for either stencil radius.
__device__ __forceinline__ void ds_decode_ofs(int o5, int &k, int &l, int &g) {
  k = o5 / 25 - 2;
  l = (o5 / 5) % 5 - 2;
  g = o5 % 5 - 2;
}

// Warp-synchronous neighbour walk with per-thread candidate lists.
//
// All 32 lanes run the same loops: over the stencil offsets (to the largest
// stencil in the warp), and over each offset's cell in pieces of DS_PIECE
// candidates (to the longest cell in the warp).  Each lane screens its own
// candidates with a cheap FP32 test (`screen(slot, ox, oy, oz)`, where
// (ox, oy, oz) = the cell's FP32 shift minus the particle's own FP32
// coordinates, so a candidate's offset is pos32 + o) and appends survivors to
// its column of the block's shared list (entry = offset code << 25 | slot -
// sb, sb = the segment's first slot, so a segment may hold up to 2^25
// particles).  When any lane's list could overflow, every lane runs `use(slot,
// offset code)` over its entries, in visiting order, and the lists restart.
// The expensive pair work thus runs on dense lists with the warp converged,
// instead of a warp idling while one lane meets a neighbour.  Lanes without a
// particle (act false) take part with empty stencils.
#define DS_SWEEP_THREADS 128
#define DS_LIST_CAP 32  // entries per thread in the shared list
#ifndef DS_PIECE
#define DS_PIECE 4      // candidates screened together (loads in flight); measured best of 1-16
#endif
#define DS_OFS_SHIFT 25
#define DS_SLOT_MASK ((1u << DS_OFS_SHIFT) - 1u)

template <int CAP = DS_LIST_CAP, class Screen, class Use>
__device__ __forceinline__ void ds_walk(const TubeDesc &T, const Stencil &S, bool act, int r, int kb, int sb,
                                        const int *cell_start, const float4 &pi, uint32_t *lst, Screen screen,
                                        Use use) {
  const unsigned FULL = 0xffffffffu;
  const int w = 2 * r + 1;
  const int nofs = act ? w * w * w : 0;
  const int nofs_w = __reduce_max_sync(FULL, nofs);
  const Shift32 f32 = ds_shift32_init(T);
  int n = 0;
  auto flush = [&]() {
    const int nw = __reduce_max_sync(FULL, n);
    for (int t = 0; t < nw; t++)
      if (t < n) {
        const uint32_t e = lst[t * DS_SWEEP_THREADS];
        use(sb + (int)(e & DS_SLOT_MASK), (int)(e >> DS_OFS_SHIFT));
      }
    n = 0;
  };
  for (int o = 0; o < nofs_w; o++) {
    int j0 = 0, j1 = 0;
    uint32_t code = 0;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    if (o < nofs) {
      double shy, shz;
      int k, l, g;
      const int cell = ds_stencil_cell(T, S, r, o, shy, shz, k, l, g);
      if (cell >= 0) {
        j0 = cell_start[kb + cell];
        j1 = cell_start[kb + cell + 1];
      }
      ds_shift32(T, S, f32, k, l, g, sx, sy, sz);
      sx -= pi.x;
      sy -= pi.y;
      sz -= pi.z;
      code = (uint32_t)((k + 2) * 25 + (l + 2) * 5 + (g + 2)) << DS_OFS_SHIFT;
    }
    const int len_w = __reduce_max_sync(FULL, j1 - j0);
    for (int p0 = 0; p0 < len_w; p0 += DS_PIECE) {
      if (__any_sync(FULL, n + DS_PIECE > CAP)) flush();
      // the piece's screens are independent: unrolled, their loads are in flight together
      bool pass[DS_PIECE];
#pragma unroll
      for (int t = 0; t < DS_PIECE; t++) {
        const int j = j0 + p0 + t;
        pass[t] = (j < j1) && screen(j, sx, sy, sz);  // j1 - j0 <= len_w
      }
#pragma unroll
      for (int t = 0; t < DS_PIECE; t++)
        if (pass[t]) {
          lst[n * DS_SWEEP_THREADS] = code | (uint32_t)(j0 + p0 + t - sb);
          n++;
        }
    }
  }
  flush();
}

// ---------------------------------------------------------------------------
// FP32 path: x offsets relative to x-blocks of DS_XB cells, row walks
// ---------------------------------------------------------------------------
// On the FP32 path a particle's x is stored relative to the origin of its
// x-block (DS_XB consecutive cells of its row; y and z stay relative to the
// own cell).  The cells ix - r .. ix + r of one (y, z) row are consecutive
// keys, so their particles are one slot range, and with block-relative x one
// shift serves the whole range -- two ranges where the row crosses a block
// edge.  Offset codes o = (db + 1) * 81 + (l + 4) * 9 + (g + 4) name the
// neighbour block (db in -1..1) and row (l, g in -4..4); a list entry is
// o << DS_OFS32_SHIFT | slot - segment start.
#define DS_XB_LOG 4
#define DS_XB (1 << DS_XB_LOG)
#define DS_NOFS32 243
#define DS_OFS32_SHIFT 24
#define DS_SLOT32_MASK ((1u << DS_OFS32_SHIFT) - 1u)
#ifndef DS_XWIN_MARGIN
#define DS_XWIN_MARGIN 0.01f  // fine x bins added on each side of a lane's row window
#endif
#ifndef DS_RPIECE
#define DS_RPIECE 8  // candidates of a row screened together (measured: 8 beats 4 and 6)
#endif

// cells each side a cut-off c needs (at least 1, at most the tube's stencil)
__device__ __forceinline__ int ds_radius(const TubeDesc &T, double c) {
  const int r = (int)ceil(c * T.rw);
  return r < 1 ? 1 : (r > T.stencil ? T.stencil : r);
}

// FP32 shifts of the offset codes: (db DS_XB wx, l wy, g wz); one table per
// block for the tube of its chunk
__device__ __forceinline__ void ds_fill_shift_table32(const TubeDesc &T, float4 *tab) {
  const float wx = (float)T.wx, wy = (float)T.wy, wz = (float)T.wz;
  for (int o = threadIdx.x; o < DS_NOFS32; o += blockDim.x) {
    const int db = o / 81 - 1, l = (o / 9) % 9 - 4, g = o % 9 - 4;
    tab[o] = make_float4((float)(db * DS_XB) * wx, (float)l * wy, (float)g * wz, 0.0f);
  }
}

// Warp-synchronous row walk with per-thread candidate lists (as ds_walk, over
// half-rows instead of cells): rows (l, g) in [-r, r]^2, l outer; within a row
// ascending slot.  The sort keys carry T.xl bits of x within the cell, so a
// row's slots are sorted by x and cell_start (indexed by cell << xl | bin)
// bounds the lane's x window instead of the whole row.  cutx bounds the
// distance of every partner the screen can accept.  On a proper grid the rows
// are true (y, z) rows, so of row (l, g) a lane needs only the x within
// sqrt(cutx^2 - d^2) of its own, d its distance to the row's y-z rectangle,
// and nothing of a row farther than cutx: the window shrinks toward the outer
// rows (a relative margin of 1e-4 on cutx^2 keeps FP32 rounding out of it).
// Dropped candidates lie outside the cut-off sphere, so the accepted pairs and
// their order are those of the full rows.  A row crossing an x-block edge is
// two ranges; the second pass runs only when some lane's window crosses one.
// screen(slot, ox, oy, oz) gets the range's shift minus the particle's own
// FP32 coordinates; use(slot, code) runs over the survivors.
template <int CAP, class Screen, class Use>
__device__ __forceinline__ void ds_walk_rows(const TubeDesc &T, const Stencil &S, bool act, int r, int kb, int sb,
                                             const int *cell_start, const float4 &pi, float cutx,
                                             const float4 *shtab, uint32_t *lst, Screen screen, Use use) {
  const unsigned FULL = 0xffffffffu;
  const int w = 2 * r + 1;
  const int nrow = act ? w * w : 0;
  const int nrow_w = __reduce_max_sync(FULL, nrow);
  const int xl = T.xl;
  const int bi = S.ix >> DS_XB_LOG;
  const int cx0 = S.ix - r < 0 ? 0 : S.ix - r;
  const int cx1 = S.ix + r > T.nx - 1 ? T.nx - 1 : S.ix + r;
  // windows in fine x indices (cell << xl | bin), clipped to the rows' cells;
  // the margin covers a partner whose FP64 key put it in the next bin (the
  // FP32 window and the FP64 keys disagree by ~1e-5 of a bin at most)
  const float sc = (float)(1 << xl) * (float)T.inv_wx;
  const int fb = (bi * DS_XB) << xl;  // fine index of the own block's origin
  const int fmin = cx0 << xl, fmax = ((cx1 + 1) << xl) - 1;
  const bool narrow = (T.mode & M_GRID_PROPER) != 0;
  const float c2 = cutx * cutx * 1.0001f;
  const float wy = (float)T.wy, wz = (float)T.wz;
  int n = 0;
  auto flush = [&]() {
    const int nw = __reduce_max_sync(FULL, n);
    for (int t = 0; t < nw; t++)
      if (t < n) {
        const uint32_t e = lst[t * DS_SWEEP_THREADS];
        use(sb + (int)(e & DS_SLOT32_MASK), (int)(e >> DS_OFS32_SHIFT));
      }
    n = 0;
  };
  int l = -r, g = -r;
  for (int q = 0; q < nrow_w; q++) {
    int f_lo = 1, f_hi = 0, cy = 0, cz = 0;
    bool ok = false;
    if (q < nrow) {
      cy = S.iy + l;
      cz = S.iz + g;
      ok = true;
      if (T.mode & M_PER_Y) cy += cy < 0 ? T.ny : (cy >= T.ny ? -T.ny : 0);
      else ok = ok && cy >= 0 && cy < T.ny;
      if (T.mode & M_PER_Z) cz += cz < 0 ? T.nz : (cz >= T.nz ? -T.nz : 0);
      else ok = ok && cz >= 0 && cz < T.nz;
      float reach = cutx;
      if (narrow) {  // y and z are relative to the own cell: the row spans [l wy, (l + 1) wy)
        const float dy = l > 0 ? (float)l * wy - pi.y : (l < 0 ? pi.y - (float)(l + 1) * wy : 0.0f);
        const float dz = g > 0 ? (float)g * wz - pi.z : (g < 0 ? pi.z - (float)(g + 1) * wz : 0.0f);
        const float d2 = (dy > 0.0f ? dy * dy : 0.0f) + (dz > 0.0f ? dz * dz : 0.0f);
        ok = ok && d2 < c2;
        reach = sqrtf(fmaxf(c2 - d2, 0.0f));
      }
      f_lo = fb + (int)floorf((pi.x - reach) * sc - DS_XWIN_MARGIN);
      f_hi = fb + (int)floorf((pi.x + reach) * sc + DS_XWIN_MARGIN);
      f_lo = f_lo < fmin ? fmin : f_lo;
      f_hi = f_hi > fmax ? fmax : f_hi;
      ok = ok && f_lo <= f_hi;
    }
    const int bsplit = (f_hi >> (xl + DS_XB_LOG)) << (xl + DS_XB_LOG);  // first fine index of f_hi's block
    const bool split = ok && bsplit > f_lo;
    const int nhalf = __any_sync(FULL, split) ? 2 : 1;
    for (int half = 0; half < nhalf; half++) {
      int j0 = 0, j1 = 0;
      uint32_t code = 0;
      float ox = 0.0f, oy = 0.0f, oz = 0.0f;
      const int a0 = half == 0 ? f_lo : bsplit;
      const int a1 = half == 0 ? (split ? bsplit - 1 : f_hi) : (split ? f_hi : bsplit - 1);
      if (ok && a0 <= a1) {
        const int base = (kb + cy * T.sy + cz * T.sz) << xl;
        j0 = cell_start[base + a0];
        j1 = cell_start[base + a1 + 1];
        const int o = ((a0 >> (xl + DS_XB_LOG)) - bi + 1) * 81 + (l + 4) * 9 + (g + 4);
        const float4 sh = shtab[o];
        ox = sh.x - pi.x;
        oy = sh.y - pi.y;
        oz = sh.z - pi.z;
        code = (uint32_t)o << DS_OFS32_SHIFT;
      }
      const int len_w = __reduce_max_sync(FULL, j1 - j0);
      for (int p0 = 0; p0 < len_w; p0 += DS_RPIECE) {
        if (__any_sync(FULL, n + DS_RPIECE > CAP)) flush();
        bool pass[DS_RPIECE];
#pragma unroll
        for (int t = 0; t < DS_RPIECE; t++) {
          const int j = j0 + p0 + t;
          pass[t] = (j < j1) && screen(j, ox, oy, oz);  // j1 - j0 <= len_w
        }
#pragma unroll
        for (int t = 0; t < DS_RPIECE; t++)
          if (pass[t]) {
            lst[n * DS_SWEEP_THREADS] = code | (uint32_t)(j0 + p0 + t - sb);
            n++;
          }
      }
    }
    if (q < nrow && ++g > r) {
      g = -r;
      ++l;
    }
  }
  flush();
}

// neighbour coordinate (with its image shift) minus ours, as the oracle does
__device__ __forceinline__ double ds_diff(double xj, double s, double xi) {
  return s != 0.0 ? (xj + s) - xi : xj - xi;
}

// Arguments shared by the sweep kernels.
// FP32 sweeps with a work counter each (SweepArgs::work + the index)
#define DS_SW_DENSITY 0
#define DS_SW_DENSITY_LST 1
#define DS_SW_DUST_DENSITY 2
#define DS_SW_FORCE_LIST 3
#define DS_SW_FORCE_WALK 4
#define DS_NSWEEP 5

struct SweepArgs {
  const TubeDesc *tubes;
  const TubeState *tstate;
  const Chunk *chunks;
  int nchunks;
  DevState st;
  const int *cell_start;    // [nkeys + 1]
  const float4 *pos32;      // prefilter / FP32 coordinates + h
  const float4 *vm32;       // FP32 vx, vy, vz, m
  const float4 *pm32;       // with list reuse: FP32 coordinates + m (the streamed density's partners), else nullptr
  float4 *hyd32;            // FP32 c, p/rho^2, rho, (unused) -- written by density
  double *cs64;             // sqrt(gam p / rho) per gas slot -- written by density
  double *pt64;             // p / (rho rho) per gas slot     -- written by density
  double *dwn64;            // dW normalisation c/h^4 per gas slot -- written by density
  double *edot;             // energy rate per gas slot
  int *ncand, *nnb;         // optional counts (parity hook), indexed by slot
  const uint32_t *skey;        // sorted neighbour key of each slot
  const unsigned char *krad;   // stencil radius each cell's force sweep needs
  const int *gas_slot_of_pid;  // slot of gas particle pid (index coupling)
  const int *gas_ind_pid;      // gas Ind by pid (index-coupled dust rho zeroing)
  TubeState *tstate_rw;
  int *flags;
  int all_tubes;               // density on demand: tubes past their end time too
  // FP32 force neighbour lists (recorded by the gas density sweep): entry e of
  // the particle in lane t of gas chunk c at nbl[(c * nbl_cap + e) * 128 + t]
  uint32_t *nbl;               // nullptr: the force sweep walks the cells
  int *nbl_cnt;                // entries per slot
  unsigned char *nbl_walk;     // per warp of each gas chunk: 1 when a particle overflowed (that warp walks)
  int nbl_cap;
  // list reuse: a tube whose TubeState::rebuild is 0 this step keeps the lists
  // (and slot order) of its last re-sort; 0: every step re-sorts and records
  int reuse;
  // persistent sweeps: nullptr -> one block per chunk; else the FP32 sweeps
  // run on a grid of about as many blocks as fit on the GPU at once, each
  // claiming its next chunk from work[k] (k: the sweep's counter, zeroed by
  // k_step_begin)
  int *work;
  int nsm;
  int bps[DS_NSWEEP];  // blocks per SM that fit, per sweep (the persistent grid: nsm x bps)
};
