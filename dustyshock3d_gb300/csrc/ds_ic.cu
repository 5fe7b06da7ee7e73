// Initial conditions generated on the device.
//
// The reference fills its host arrays with one of its generators before the
// upload (init_Sod_X_Dust, kernel.cu:1391-1582, is the one main calls;
// init_Sod_X_mas, kernel.cu:938-1042, is the equal-mass lattice model).  Here
// the host only plans (parameters, counts, the accepted index box of each
// lattice) and one thread per particle writes the particle's fields into the
// tube's segment.  The arithmetic is the generators' own, operation by
// operation (explicit round-to-nearest intrinsics on the device; this file's
// host code is compiled without FP contraction), so the particles equal the
// host generators' bit for bit.
//
// The reference visits lattice points (i, j, k) with k innermost and appends
// each accepted one; its Ind assignment sits outside the accept test
// (kernel.cu:1441-1448, 1481-1488), so every lattice point writes the flag of
// the last accepted particle.  Particle p's Ind is therefore the interior flag
// of the last lattice point before particle p + 1's point (or of the very last
// point, for the last particle) -- computed here per particle, in parallel.

#include "ds_ic.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int kIcThreads = 256;

// lattice coordinates (kernel.cu:1422-1424, 1462-1464)
__host__ __device__ __forceinline__ double lat_x(int sgn, double dl, int i) {
#ifdef __CUDA_ARCH__
  const double t = __dmul_rn((double)i, dl);
  return sgn < 0 ? __dsub_rn(0.0, t) : __dadd_rn(dl, t);
#else
  const double t = (double)i * dl;
  return sgn < 0 ? 0.0 - t : dl + t;
#endif
}

__host__ __device__ __forceinline__ double lat_yz(double org, double dl, int j) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(org, __dmul_rn((double)j, dl));
#else
  return org + (double)j * dl;
#endif
}

// Eq_State and Eq_State1 (kernel.cu:92-103) with the literal gamma 1.4 and
// sound speed 1.0 the generators pass; a Type_of_state other than 1 takes the
// ideal-gas branch.
double eq_state(double rho, double e, int type) { return type == 1 ? 1.0 * 1.0 * rho : rho * e * (1.4 - 1); }
double eq_state1(double p, double e, int type) { return type == 1 ? p / (1.0 * 1.0) : p / (e * (1.4 - 1)); }

// The accepted indices 0..nmax of one axis, [a, b] (empty: a > b).  False if
// they are not one contiguous range (cannot happen for monotone coordinates).
template <class F> bool accepted_range(int nmax, double cube, F coord, int &a, int &b) {
  int first = -1, last = -2;
  for (int i = 0; i <= nmax; i++)
    if (std::fabs(coord(i)) <= cube) {
      if (first < 0) first = i;
      last = i;
    }
  a = 0;
  b = -1;
  if (first < 0) return true;
  for (int i = first; i <= last; i++)
    if (!(std::fabs(coord(i)) <= cube)) return false;
  a = first;
  b = last;
  return true;
}

bool to_int(double v, int &out) {  // int(v), truncation, within +-2^30
  if (!std::isfinite(v) || std::fabs(v) >= 1073741824.0) return false;
  out = (int)v;
  return true;
}

bool round_half_even(double v, int &out) {  // Python's int(round(v))
  if (!std::isfinite(v) || std::fabs(v) >= 1073741824.0) return false;
  out = (int)std::nearbyint(v);
  return true;
}

// The two lattices of kernel.cu:938-1042 (mas) or 1391-1582 (dust).
ds_status plan_reference(const ds_ic &ic, const ds_params &init, IcPlan &P, std::string &err) {
  const bool dust_gen = ic.kind == DS_IC_SOD_X_DUST;
  const double h = init.h;
  const double border_length = 2.5 * h;
  double cube[3], e_lr[2], p_lr[2], rho_lr[2];
  if (dust_gen) {  // kernel.cu:1394-1404
    cube[0] = 1.0; cube[1] = 0.8; cube[2] = 0.8;
    e_lr[0] = 2.5; e_lr[1] = 2.0;
    rho_lr[0] = 1.0; rho_lr[1] = 1.0;
    p_lr[0] = eq_state(rho_lr[0], e_lr[0], init.Type_of_state);
    p_lr[1] = eq_state(rho_lr[1], e_lr[1], init.Type_of_state);
    // the interior test compares y with X_cube (kernel.cu:1441, 1481)
    P.inner[0] = cube[0] - border_length;
    P.inner[1] = cube[0] - border_length;
    P.inner[2] = cube[2] - border_length;
  } else {  // kernel.cu:945-951
    cube[0] = cube[1] = cube[2] = 1.0;
    p_lr[0] = 1.0; p_lr[1] = 0.1;
    e_lr[0] = 2.5; e_lr[1] = 2.0;
    rho_lr[0] = eq_state1(p_lr[0], e_lr[0], init.Type_of_state);
    rho_lr[1] = eq_state1(p_lr[1], e_lr[1], init.Type_of_state);
    P.inner[0] = P.inner[1] = P.inner[2] = 1.0 - border_length;
  }
  const double mas = 1.0 / (init.Particle_on_length * init.Particle_on_length * init.Particle_on_length);
  P.mas = mas;
  P.h = h;
  P.gam = init.Gam_g;
  P.Y_min = init.Y_min;
  P.Z_min = init.Z_min;
  long long base = 0, p0 = 0;
  for (int s = 0; s < 2; s++) {
    IcLattice &L = P.lat[s];
    L.dl = std::pow(mas / rho_lr[s], 1 / 3.0);
    L.sgn = s == 0 ? -1 : 1;
    L.e = e_lr[s];
    L.p = p_lr[s];
    L.rho = rho_lr[s];
    const double span_x = s == 0 ? (0.0 - init.X_min) : (init.X_max - 0.0);
    if (!to_int(span_x / L.dl, L.Im) || !to_int((init.Y_max - init.Y_min) / L.dl, L.Jm) ||
        !to_int((init.Z_max - init.Z_min) / L.dl, L.Km)) {
      err = "lattice too large or spacing not finite (Particle_on_length, box)";
      return DS_ERR_ARG;
    }
    L.Im += 1;  // kernel.cu:1414-1416, 1455-1457
    L.Jm += 1;
    L.Km += 1;
    const long long pts = (long long)std::max(0, L.Im + 1) * std::max(0, L.Jm + 1) * std::max(0, L.Km + 1);
    L.base = base;
    base += pts;
    bool ok = accepted_range(L.Im, cube[0], [&](int i) { return lat_x(L.sgn, L.dl, i); }, L.ia, L.ib);
    ok = ok && accepted_range(L.Jm, cube[1], [&](int j) { return lat_yz(init.Y_min, L.dl, j); }, L.ja, L.jb);
    ok = ok && accepted_range(L.Km, cube[2], [&](int k) { return lat_yz(init.Z_min, L.dl, k); }, L.ka, L.kb);
    if (!ok) {
      err = "accepted lattice points are not a box of indices";
      return DS_ERR_UNSUPPORTED;
    }
    L.count = (L.ib >= L.ia && L.jb >= L.ja && L.kb >= L.ka)
                  ? (long long)(L.ib - L.ia + 1) * (L.jb - L.ja + 1) * (L.kb - L.ka + 1) : 0;
    L.p0 = p0;
    p0 += L.count;
  }
  P.M = base;
  // the first lattice point must be accepted: otherwise the reference writes
  // Ind_gas[-1] (undefined behaviour)
  if (P.M > 0) {
    const IcLattice &F = P.lat[P.lat[0].base < P.lat[1].base ? 0 : 1];
    if (!(F.count > 0 && F.ia == 0 && F.ja == 0 && F.ka == 0)) {
      err = "first lattice point rejected: the reference writes Ind_gas[-1] there (undefined behaviour); "
            "choose Y_min, Z_min inside the accept cube";
      return DS_ERR_ARG;
    }
  }
  const long long N = p0;
  if (N > init.Maximum_particle || N > 0x7fffffffLL) {
    err = std::to_string(N) + " gas particles exceed Maximum_particle (the reference would overrun its "
                              "arrays, kernel.cu:1751)";
    return DS_ERR_ARG;
  }
  P.params = init;
  if (dust_gen) {  // kernel.cu:1497-1502
    P.params.Coeff_h_dust_cell = 0.5;
    P.params.n_dust = 2;
    for (int k = 0; k < DS_MAX_DUST; k++) P.params.mass_ratio[k] = P.params.R_dust[k] = 0.0;
    P.params.mass_ratio[0] = 0.75;
    P.params.mass_ratio[1] = 0.5;
    P.params.R_dust[0] = 0.01;
    P.params.R_dust[1] = 1.0;
    P.params.mode = DS_MODE_REFERENCE;
  }
  if (P.params.n_dust < 1 || P.params.n_dust > DS_MAXD) {
    err = "n_dust out of range";
    return DS_ERR_ARG;
  }
  for (int k = 0; k < P.params.n_dust; k++) {
    P.mass_ratio[k] = P.params.mass_ratio[k];
    P.R_dust[k] = P.params.R_dust[k];
  }
  P.nspecies = 1 + P.params.n_dust;
  for (int s = 0; s < P.nspecies; s++) P.count[s] = N;
  return DS_OK;
}

// One side of the dusty Sod tube (two lattices of equal particle mass).
bool tube_side(const ds_ic &ic, double rho, double p, double xa, double xb, double dxy_target, double Ly,
               double Lz, IcTubeSide &S) {
  if (!round_half_even(Ly / dxy_target, S.ny) || !round_half_even(Lz / dxy_target, S.nz)) return false;
  S.ny = std::max(1, S.ny);
  S.nz = std::max(1, S.nz);
  S.dy = Ly / S.ny;
  S.dz = Lz / S.nz;
  const double m = ic.rho_L * std::pow(ic.dx_left, 3.0);
  const double dx = m / (rho * S.dy * S.dz);
  if (!round_half_even((xb - xa) / dx, S.nx)) return false;
  S.nx = std::max(1, S.nx);
  S.dx = (xb - xa) / S.nx;
  S.mass = rho * S.dx * S.dy * S.dz;
  S.h = ic.h_factor * std::pow(S.dx * S.dy * S.dz, 1.0 / 3.0);
  S.xa = xa;
  S.rho = rho;
  S.p = p;
  S.e = p / ((ic.gamma - 1.0) * rho);
  S.count = (long long)S.nx * S.ny * S.nz;
  return true;
}

ds_status plan_tube(const ds_ic &ic, IcPlan &P, std::string &err) {
  const double Lz = ic.Lz > 0 ? ic.Lz : ic.Ly;
  const double vals[] = {ic.dx_left, ic.Ly, Lz, ic.rho_L, ic.rho_R, ic.p_L, ic.p_R, ic.h_factor};
  for (double v : vals)
    if (!(v > 0) || !std::isfinite(v)) {
      err = "dx_left, Ly, Lz, densities, pressures and h_factor must be positive";
      return DS_ERR_ARG;
    }
  if (!(ic.x1 > ic.x0) || !(ic.gamma > 1.0) || !(ic.eps > 0) || !(ic.t_s > 0) || ic.fixed_tau < 0) {
    err = "need x1 > x0, gamma > 1, eps > 0, t_s > 0, fixed_tau >= 0";
    return DS_ERR_ARG;
  }
  const double xm = 0.5 * (ic.x0 + ic.x1);
  const double target_R = ic.dx_left * std::pow(ic.rho_L / ic.rho_R, 1.0 / 3.0);
  if (!tube_side(ic, ic.rho_L, ic.p_L, ic.x0, xm, ic.dx_left, ic.Ly, Lz, P.side[0]) ||
      !tube_side(ic, ic.rho_R, ic.p_R, xm, ic.x1, target_R, ic.Ly, Lz, P.side[1])) {
    err = "lattice counts out of range";
    return DS_ERR_ARG;
  }
  P.side[0].p0 = 0;
  P.side[1].p0 = P.side[0].count;
  const long long N = P.side[0].count + P.side[1].count;
  if (N > 0x7fffffffLL) {
    err = "more than 2^31 - 1 particles";
    return DS_ERR_ARG;
  }
  P.off = ic.lattice_offset;
  P.Ly = ic.Ly;
  P.Lz = Lz;
  P.eps = ic.eps;
  P.t_s = ic.t_s;
  P.x0 = ic.x0;
  P.x1 = ic.x1;
  P.wall = ic.wall;
  const double h_max = std::max(P.side[0].h, P.side[1].h);
  ds_params &Q = P.params;
  ds_params_init(&Q);
  Q.X_min = ic.x0;
  Q.X_max = ic.x1;
  Q.Y_min = 0.0;
  Q.Y_max = ic.Ly;
  Q.Z_min = 0.0;
  Q.Z_max = Lz;
  Q.Type_of_state = 0;
  Q.Maximum_particle = (int)N;
  Q.Particle_on_length = 1.0 / ic.dx_left;
  Q.h = h_max;
  Q.Coeff_h_dust_cell = 0.5;
  Q.tau = ic.fixed_tau > 0 ? ic.fixed_tau : 1e-4;
  Q.T_end = ic.t_end;
  Q.T_out = ic.t_end;
  Q.alpha = ic.alpha;
  Q.beta = ic.beta;
  Q.eps = ic.av_eps;
  Q.Gam_g = ic.gamma;
  Q.Speed_of_sound_gas = 1.0;
  Q.n_dust = 1;
  for (int k = 0; k < DS_MAX_DUST; k++) Q.mass_ratio[k] = Q.R_dust[k] = Q.t_stop_const[k] = Q.eps_empty[k] = 0.0;
  Q.mass_ratio[0] = ic.eps;
  Q.t_stop_const[0] = ic.t_s;
  Q.eps_empty[0] = ic.eps;
  Q.t_empty = ic.t_s;
  Q.cell_w = 1.001 * h_max;
  Q.stencil = 2;
  Q.idic_w = ic.idic_cells * P.side[1].dx;
  Q.cfl = ic.cfl;
  Q.mode = DS_MODE_PERIODIC_Y | DS_MODE_PERIODIC_Z | DS_MODE_H_PER_PARTICLE | DS_MODE_TSTOP_CONST |
           DS_MODE_GAS_ACCEL_PARTICLE | DS_MODE_CFL | DS_MODE_GRID_PROPER | DS_MODE_IDIC_PROPER;
  if (ic.fixed_tau > 0) Q.mode &= ~DS_MODE_CFL;
  Q.precision = DS_PRECISION_FP64;
  Q.list_depth = 0;
  Q.force_list = 0;
  P.nspecies = 2;
  P.count[0] = P.count[1] = N;
  return DS_OK;
}

// ---------------------------------------------------------------------------
// Device
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long lattice_point(const IcPlan &P, long long p, int &s, int &i, int &j, int &k) {
  s = p < P.lat[0].count ? 0 : 1;
  const IcLattice &L = P.lat[s];
  const long long q = p - L.p0;
  const long long nj = L.jb - L.ja + 1, nk = L.kb - L.ka + 1;
  i = L.ia + (int)(q / (nj * nk));
  j = L.ja + (int)((q / nk) % nj);
  k = L.ka + (int)(q % nk);
  return L.base + ((long long)i * (L.Jm + 1) + j) * (L.Km + 1) + k;
}

__global__ void __launch_bounds__(kIcThreads) k_ic_lattice(IcPlan P, int species, DevState d, int b) {
  const long long n = P.count[0];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    int s, i, j, k;
    lattice_point(P, p, s, i, j, k);
    const IcLattice &L = P.lat[s];
    const double x = lat_x(L.sgn, L.dl, i), y = lat_yz(P.Y_min, L.dl, j), z = lat_yz(P.Z_min, L.dl, k);
    // Ind: interior flag of the lattice point just before the next particle's
    long long last = P.M - 1;
    if (p + 1 < n) {
      int s2, i2, j2, k2;
      last = lattice_point(P, p + 1, s2, i2, j2, k2) - 1;
    }
    const IcLattice &T = P.lat[last >= P.lat[1].base ? 1 : 0];
    const long long r = last - T.base, nk = T.Km + 1, nj = T.Jm + 1;
    const int it = (int)(r / (nk * nj)), jt = (int)((r / nk) % nj), kt = (int)(r % nk);
    const double xt = lat_x(T.sgn, T.dl, it), yt = lat_yz(P.Y_min, T.dl, jt), zt = lat_yz(P.Z_min, T.dl, kt);
    const int ind = (fabs(xt) <= P.inner[0] && fabs(yt) <= P.inner[1] && fabs(zt) <= P.inner[2]) ? 0 : 1;
    const int q = b + (int)p;
    d.x[q] = x;
    d.y[q] = y;
    d.z[q] = z;
    d.vx[q] = 0.0; d.vy[q] = 0.0; d.vz[q] = 0.0;
    d.ax[q] = 0.0; d.ay[q] = 0.0; d.az[q] = 0.0;
    d.h[q] = P.h;
    if (species == 0) {  // kernel.cu:1428-1437
      d.rho[q] = L.rho;
      d.p[q] = L.p;
      d.e[q] = L.e;
      d.m[q] = P.mas;
      d.ts[q] = 0.0;
    } else {  // dust on the gas site (kernel.cu:1505-1548); t_stop = Eq_t_stop (kernel.cu:43-46)
      const double mr = P.mass_ratio[species - 1], R = P.R_dust[species - 1];
      d.rho[q] = __dmul_rn(L.rho, mr);
      d.p[q] = 0.0;
      d.e[q] = 0.0;
      d.m[q] = __dmul_rn(P.mas, mr);
      d.ts[q] = __ddiv_rn(R, __dmul_rn(__dsqrt_rn(__ddiv_rn(__dmul_rn(P.gam, L.p), L.rho)), L.rho));
    }
    d.ind[q] = ind;
    d.pid[q] = (int)p;
  }
}

__global__ void __launch_bounds__(kIcThreads) k_ic_tube(IcPlan P, int species, DevState d, int b) {
  const long long n = P.count[species];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    const IcTubeSide &S = P.side[p < P.side[0].count ? 0 : 1];
    const long long q = p - S.p0, nyz = (long long)S.ny * S.nz;
    const int i = (int)(q / nyz), j = (int)((q / S.nz) % S.ny), k = (int)(q % S.nz);
    double x = __dadd_rn(S.xa, __dmul_rn(__dadd_rn((double)i, P.off), S.dx));
    double y = __dmul_rn(__dadd_rn((double)j, P.off), S.dy);
    double z = __dmul_rn(__dadd_rn((double)k, P.off), S.dz);
    if (species) {  // half a spacing further; y, z wrap onto the periodic lattice
      x = __dadd_rn(x, __dmul_rn(0.5, S.dx));
      y = fmod(__dadd_rn(y, __dmul_rn(0.5, S.dy)), P.Ly);
      z = fmod(__dadd_rn(z, __dmul_rn(0.5, S.dz)), P.Lz);
    }
    const double wh = __dmul_rn(P.wall, S.h);
    const int ind = (x < __dadd_rn(P.x0, wh) || x > __dsub_rn(P.x1, wh)) ? 1 : 0;
    const int o = b + (int)p;
    d.x[o] = x;
    d.y[o] = y;
    d.z[o] = z;
    d.vx[o] = 0.0; d.vy[o] = 0.0; d.vz[o] = 0.0;
    d.ax[o] = 0.0; d.ay[o] = 0.0; d.az[o] = 0.0;
    d.h[o] = S.h;
    if (species == 0) {
      d.rho[o] = S.rho;
      d.p[o] = S.p;
      d.e[o] = S.e;
      d.m[o] = S.mass;
      d.ts[o] = 0.0;
    } else {
      d.rho[o] = __dmul_rn(S.rho, P.eps);
      d.p[o] = 0.0;
      d.e[o] = 0.0;
      d.m[o] = __dmul_rn(S.mass, P.eps);
      d.ts[o] = P.t_s;
    }
    d.ind[o] = ind;
    d.pid[o] = (int)p;
  }
}

}  // namespace

ds_status ds_ic_make_plan(const ds_ic &ic, const ds_params *init, IcPlan &plan, std::string &err) {
  plan = IcPlan{};
  plan.kind = ic.kind;
  switch (ic.kind) {
    case DS_IC_SOD_X_DUST:
    case DS_IC_SOD_X_MAS:
      if (!init) {
        err = "the reference generators read the Init.txt parameters (init is NULL)";
        return DS_ERR_ARG;
      }
      if (!(init->Particle_on_length > 0) || !(init->h >= 0)) {
        err = "Particle_on_length must be positive";
        return DS_ERR_ARG;
      }
      return plan_reference(ic, *init, plan, err);
    case DS_IC_DUSTY_SOD:
      return plan_tube(ic, plan, err);
    default:
      err = "unknown initial-condition kind";
      return DS_ERR_ARG;
  }
}

void ds_launch_ic(const IcPlan &plan, int species, DevState dst, int b, cudaStream_t s) {
  const long long n = plan.count[species];
  if (n <= 0) return;
  const long long want = (n + kIcThreads - 1) / kIcThreads;
  const int blocks = (int)std::min<long long>(want, 152LL * 16);
  if (plan.kind == DS_IC_DUSTY_SOD) k_ic_tube<<<blocks, kIcThreads, 0, s>>>(plan, species, dst, b);
  else k_ic_lattice<<<blocks, kIcThreads, 0, s>>>(plan, species, dst, b);
}
