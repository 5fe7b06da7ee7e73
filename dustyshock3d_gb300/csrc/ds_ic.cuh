// Initial conditions generated on the device, straight into a tube's state:
// the reference's lattice generators (kernel.cu:938-1042, 1391-1582) and the
// dusty Sod tube of the benchmark configurations.
#pragma once

#include <string>

#include "ds_common.cuh"
#include "../../include/dustyshock3d_gb300.h"

// One lattice of the reference's generators: points (i, j, k) with
// 0 <= i <= Im, 0 <= j <= Jm, 0 <= k <= Km visited with k innermost, at
// x = 0.0 - i dl (left, sgn < 0) or dl + i dl (right), y = Y_min + j dl,
// z = Z_min + k dl.  Each coordinate is monotone in its index (rounding is
// monotone), so the accept test |x| <= cube_x && |y| <= cube_y && |z| <= cube_z
// holds exactly on a box of indices [ia, ib] x [ja, jb] x [ka, kb].
struct IcLattice {
  double dl;
  int sgn;
  int Im, Jm, Km;
  int ia, ib, ja, jb, ka, kb;  // accepted index ranges
  long long base;              // linear index of point (0, 0, 0) over both lattices
  long long p0, count;         // first particle index, accepted points
  double e, p, rho;
};

// One side of the dusty Sod tube: an nx x ny x nz lattice, k innermost.
struct IcTubeSide {
  double xa, dx, dy, dz, mass, h, rho, p, e;
  int nx, ny, nz;
  long long p0, count;
};

struct IcPlan {
  int kind = 0;
  int nspecies = 0;
  long long count[DS_MAXS] = {};
  ds_params params{};
  // reference lattices
  IcLattice lat[2]{};
  double Y_min = 0, Z_min = 0;
  double inner[3] = {};  // interior (Ind = 0) thresholds on |x|, |y|, |z|
  double mas = 0, h = 0, gam = 0;
  long long M = 0;       // lattice points of both lattices
  double mass_ratio[DS_MAXD] = {}, R_dust[DS_MAXD] = {};
  // dusty Sod tube
  IcTubeSide side[2]{};
  double off = 0, Ly = 0, Lz = 0, eps = 0, t_s = 0, x0 = 0, x1 = 0, wall = 0;
};

// Host-side plan: run parameters, counts and lattice ranges.  init: the
// Init.txt parameters the reference generators read (may be null for the
// dusty tube).  err receives the reason of a failure.
ds_status ds_ic_make_plan(const ds_ic &ic, const ds_params *init, IcPlan &plan, std::string &err);

// Writes species `species` of the plan into dst at slots b .. b + count - 1,
// caller order (pid = particle index).
void ds_launch_ic(const IcPlan &plan, int species, DevState dst, int b, cudaStream_t s);
