/*
 * ref_gpu.c -- the reference's own CUDA kernels on this GPU, under a host loop
 * that restates the reference's main loop (kernel.cu:1929-2523).
 *
 * BASELINE AND TEST INFRASTRUCTURE.  Only bench.py (the reference-GPU
 * baseline) and tests/ load this library; the product never does.
 *
 * The kernels are the reference's: kernel.cu (which includes IDIC.h) compiled
 * unmodified, with nvcc's default floating-point options, into a cubin by
 * oracle/build_ref_gpu.sh.  This file loads that cubin through the CUDA driver
 * API (libcuda, opened at run time) and launches its kernels exactly where the
 * reference's loop launches them:
 *   - linked cell lists of the three species built on the host
 *     (kernel.cu:1937-1995) and copied up;
 *   - one launch per stencil offset (k, l, g) for every neighbour sum, each
 *     followed by a device synchronize (kernel.cu:2011-2046, 2233-2266);
 *   - the stopping-time, relaxation, move and energy kernels (kernel.cu:
 *     2049-2056, 2468-2523);
 *   - the IDIC cell averages and the two-species implicit solve on the host
 *     (kernel.cu:2060-2437), with the reference's blocking copies around them.
 * Grid and block shapes are the reference's: Pm / 256 + 1 blocks of 16 x 16
 * threads (kernel.cu:1867-1868).  Snapshot output (kernel.cu:2528-2564) is
 * left out: the timing excludes I/O.
 *
 * One guard is added that the reference does not have: before the relaxation
 * kernels, every IDIC cell index the host computed (the same positions the
 * kernels index with) is checked against the cell arrays, and the run stops
 * with an error instead of launching kernels that would read outside them.
 */
#define _POSIX_C_SOURCE 200809L
#include <dlfcn.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "oracle.h"

/* ---- the few driver-API types and entry points used (CUDA 12/13 ABI) ---- */
typedef int CUresult;
typedef int CUdevice;
typedef struct CUctx_st *CUcontext;
typedef struct CUmod_st *CUmodule;
typedef struct CUfunc_st *CUfunction;
typedef struct CUstream_st *CUstream;
typedef unsigned long long CUdeviceptr;

static struct {
  void *so;
  CUresult (*Init)(unsigned);
  CUresult (*DeviceGet)(CUdevice *, int);
  CUresult (*PrimaryCtxRetain)(CUcontext *, CUdevice);
  CUresult (*PrimaryCtxRelease)(CUdevice);
  CUresult (*CtxSetCurrent)(CUcontext);
  CUresult (*ModuleLoad)(CUmodule *, const char *);
  CUresult (*ModuleUnload)(CUmodule);
  CUresult (*ModuleGetFunction)(CUfunction *, CUmodule, const char *);
  CUresult (*MemAlloc)(CUdeviceptr *, size_t);
  CUresult (*MemFree)(CUdeviceptr);
  CUresult (*MemcpyHtoD)(CUdeviceptr, const void *, size_t);
  CUresult (*MemcpyDtoH)(void *, CUdeviceptr, size_t);
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           CUstream, void **, void **);
  CUresult (*CtxSynchronize)(void);
  CUresult (*GetErrorString)(CUresult, const char **);
} D;

static char g_err[512];

static int fail(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return -1;
}

static int cu_check(CUresult r, const char *what) {
  if (r == 0) return 0;
  const char *s = "unknown";
  if (D.GetErrorString) D.GetErrorString(r, &s);
  return fail("%s: CUDA driver error %d (%s)", what, r, s ? s : "?");
}
#define CU(call, what) \
  do {                 \
    if (cu_check((call), (what))) goto out; \
  } while (0)

static int load_driver(void) {
  if (D.so) return 0;
  void *so = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!so) return fail("libcuda.so.1 not found: %s", dlerror());
#define SYM(field, name)                                        \
  do {                                                          \
    *(void **)(&D.field) = dlsym(so, name);                     \
    if (!D.field) return fail("libcuda.so.1 lacks %s", name);   \
  } while (0)
  SYM(Init, "cuInit");
  SYM(DeviceGet, "cuDeviceGet");
  SYM(PrimaryCtxRetain, "cuDevicePrimaryCtxRetain");
  SYM(PrimaryCtxRelease, "cuDevicePrimaryCtxRelease_v2");
  SYM(CtxSetCurrent, "cuCtxSetCurrent");
  SYM(ModuleLoad, "cuModuleLoad");
  SYM(ModuleUnload, "cuModuleUnload");
  SYM(ModuleGetFunction, "cuModuleGetFunction");
  SYM(MemAlloc, "cuMemAlloc_v2");
  SYM(MemFree, "cuMemFree_v2");
  SYM(MemcpyHtoD, "cuMemcpyHtoD_v2");
  SYM(MemcpyDtoH, "cuMemcpyDtoH_v2");
  SYM(LaunchKernel, "cuLaunchKernel");
  SYM(CtxSynchronize, "cuCtxSynchronize");
  SYM(GetErrorString, "cuGetErrorString");
#undef SYM
  D.so = so;
  return 0;
}

/* The reference's kernels by their (C++) symbol names in the cubin. */
enum { K_RHO_INIT, K_RHO, K_P, K_TSTOP, K_E_INIT, K_F_INIT, K_FORCE, K_V_DUST, K_V_GAS, K_MOVE, K_ENERGY, K_N };
static const char *const kname[K_N] = {
    "_Z19Rho_InitKernel_IDICPdS_S_Pii",                                  /* IDIC.h:2   */
    "_Z15Rho_Kernel_IDICPdS_S_S_S_PiS0_S0_iddddiiidiii",                 /* IDIC.h:17  */
    "_Z7PKernelPdS_S_Piiidd",                                            /* kernel.cu:107 */
    "_Z18t_stop_Kernel_IDICPdS_S_Piidd",                                 /* IDIC.h:78  */
    "_Z21EnergyInitKernel_IDICPdPii",                                    /* IDIC.h:93  */
    "_Z21Force_InitKernel_IDICPdS_S_Pii",                                /* IDIC.h:183 */
    "_Z16ForceKernel_IDICPdS_S_S_S_S_S_S_S_S_S_S_S_PiS0_S0_iddddiiiddddddiii", /* IDIC.h:198 */
    "_Z17V_dustKernel_IDICPdS_S_S_S_S_S_S_S_S_Piddddiiidi",              /* IDIC.h:264 */
    "_Z16V_gasKernel_IDICPdS_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_Piddddiiidi", /* IDIC.h:287 */
    "_Z15MoveKernel_IDICPdS_S_S_S_S_Pidi",                               /* IDIC.h:319 */
    "_Z17EnergyKernel_IDICPdS_Pidi",                                     /* IDIC.h:335 */
};

static CUdevice g_dev;
static CUcontext g_ctx;
static CUmodule g_mod;
static CUfunction g_fn[K_N];

const char *rg_last_error(void) { return g_err; }

/* Load libcuda, make device 0's primary context current and load the cubin.
 * Returns 0, or -1 with rg_last_error() set. */
int rg_open(const char *cubin) {
  if (g_mod) return 0;
  if (load_driver()) return -1;
  CU(D.Init(0), "cuInit");
  CU(D.DeviceGet(&g_dev, 0), "cuDeviceGet");
  CU(D.PrimaryCtxRetain(&g_ctx, g_dev), "cuDevicePrimaryCtxRetain");
  CU(D.CtxSetCurrent(g_ctx), "cuCtxSetCurrent");
  CU(D.ModuleLoad(&g_mod, cubin), "cuModuleLoad");
  for (int k = 0; k < K_N; k++) CU(D.ModuleGetFunction(&g_fn[k], g_mod, kname[k]), kname[k]);
  return 0;
out:
  g_mod = NULL;
  return -1;
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* Wall time of the last rg_run by kind of work: host cell lists, kernels
 * (launch + synchronize), blocking copies, host IDIC averages and solve. */
enum { PH_LISTS, PH_KERNELS, PH_COPIES, PH_IDIC, PH_N };
static double g_phase[PH_N];

/* ---- launches: the reference's gridSize / blockSize, then a synchronize ---- */
static unsigned g_blocks;
static int launch(int k, void **args, int sync) {
  const double t = now_s();
  int r = cu_check(D.LaunchKernel(g_fn[k], g_blocks, 1, 1, 16, 16, 1, 0, NULL, args, NULL), kname[k]);
  if (!r && sync) r = cu_check(D.CtxSynchronize(), "cudaDeviceSynchronize");
  g_phase[PH_KERNELS] += now_s() - t;
  return r;
}
static int h2d(CUdeviceptr d, const void *h, size_t n) {
  const double t = now_s();
  const int r = cu_check(D.MemcpyHtoD(d, h, n), "cudaMemcpy H2D");
  g_phase[PH_COPIES] += now_s() - t;
  return r;
}
static int d2h(void *h, CUdeviceptr d, size_t n) {
  const double t = now_s();
  const int r = cu_check(D.MemcpyDtoH(h, d, n), "cudaMemcpy D2H");
  g_phase[PH_COPIES] += now_s() - t;
  return r;
}

void rg_phase_seconds(double *out) {
  for (int k = 0; k < PH_N; k++) out[k] = g_phase[k];
}

/* device copies of one species' fields (kernel.cu:1800-1865) */
typedef struct {
  CUdeviceptr x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, m, ts, ind, cell, nn;
} dspecies;

/* host-side per-cell arrays of the IDIC phase (kernel.cu:1586-1660) */
typedef struct {
  double *vxg, *vyg, *vzg, *rhog, *eg, *psix, *psiy, *psiz;
  double *yx, *yy, *yz, *ynx, *yny, *ynz, *beta;
  int *gcount;
  double *vxd[2], *vyd[2], *vzd[2], *rhod[2], *epsc[2], *tsav[2], *bcell[2];
  double *xx[2], *xy[2], *xz[2], *xnx[2], *xny[2], *xnz[2];
  int *dcount[2];
} idic_cells;

/* Host linked list of one species (kernel.cu:1937-1955). */
static void build_list(const orc_species *s, int Pm, double Clx, double Cly, double Clz, double Clh, int Cnx,
                       int Cny, int ncells, int *Cell, int *Ne, int *Nn) {
  for (int i = 0; i <= ncells; i++) Cell[i] = -1;
  for (int p = 0; p <= Pm; p++) Nn[p] = -1;
  for (int p = 0; p <= Pm; p++) {
    const int i = (int)((s->x[p] - Clx) / Clh) + ((int)((s->y[p] - Cly) / Clh)) * Cnx +
                  ((int)((s->z[p] - Clz) / Clh)) * Cnx * Cny;
    if (i >= 0 && i <= ncells) {
      if (Cell[i] == -1) {
        Cell[i] = p;
        Ne[i] = p;
        Nn[p] = -1;
      } else {
        Nn[Ne[i]] = p;
        Ne[i] = p;
        Nn[p] = -1;
      }
    }
  }
}

static inline int idic_index(const orc_species *s, int p, double X_min, double Y_min, double Z_min, double w,
                             int Nax, int Nay) {
  return (int)((s->x[p] - X_min) / w) + ((int)((s->y[p] - Y_min) / w)) * Nax +
         ((int)((s->z[p] - Z_min) / w)) * Nax * Nay;
}

/*
 * Run nsteps of the reference's loop on sp[0] (gas), sp[1], sp[2] (dust 1, 2):
 * equal counts, the reference's two-species layout.  The caller's arrays are
 * the reference's host arrays: they are copied to the device first
 * (kernel.cu:1800-1865) and hold the state the loop's copies leave there at
 * the end.  *Tm advances by tau per step (kernel.cu:1931).  step_s[n] gets the
 * wall time of each step (the whole loop body: host lists, copies, launches,
 * synchronizes and host IDIC).  Returns 0, or -1 with rg_last_error() set.
 */
int rg_run(const orc_params *P, orc_species *sp, int nsteps, double *Tm, double *step_s) {
  if (!g_mod) return fail("rg_open has not succeeded");
  if (P->n_dust != 2) return fail("the reference's loop has two dust species (n_dust %d)", P->n_dust);
  if (sp[0].n != sp[1].n || sp[0].n != sp[2].n || sp[0].n < 1)
    return fail("the reference's species share one count Pm + 1 (%d, %d, %d)", sp[0].n, sp[1].n, sp[2].n);
  const int Pm = sp[0].n - 1;
  const double h = P->h, tau = P->tau, Gam_g = P->Gam_g, alpha = P->alpha, beta = P->beta, eps = P->eps;
  const double Speed_of_sound_gas = P->Speed_of_sound_gas;
  const int Type_of_state = P->Type_of_state;
  /* neighbour grid, kernel.cu:1767-1778 */
  const double Clx = P->X_min, Cly = P->Y_min, Clz = P->Z_min, Clh = P->cell_w;
  const int Cnx = (int)((P->X_max - Clx) / Clh), Cny = (int)((P->Y_max - Cly) / Clh),
            Cnz = (int)((P->Z_max - Clz) / Clh);
  const int Number_of_fihd_cells = (Cnx + 1) * (Cny + 1) * (Cnz + 1);
  /* IDIC grid, kernel.cu:1577-1582 */
  const double X_min = P->X_min, Y_min = P->Y_min, Z_min = P->Z_min, average_cell_width = P->idic_w;
  const int Nax = (int)((P->X_max - P->X_min) / average_cell_width);
  const int Nay = (int)((P->Y_max - P->Y_min) / average_cell_width);
  const int Naz = (int)((P->Z_max - P->Z_min) / average_cell_width);
  const int Number_of_average_cell = (Nax + 1) * (Nay + 1) * (Naz + 1);
  const double mas_gas_dust[2] = {P->mass_ratio[0], P->mass_ratio[1]};
  const double R_dust[2] = {P->R_dust[0], P->R_dust[1]};
  const double eps_empty[2] = {P->eps_empty[0], P->eps_empty[1]};
  const double t_empty = P->t_empty;
  g_blocks = (unsigned)(Pm / 256 + 1);

  const size_t nd = (size_t)(Pm + 1) * sizeof(double), ni = (size_t)(Pm + 1) * sizeof(int);
  const size_t cd = (size_t)(Number_of_average_cell + 1) * sizeof(double);
  const size_t fc = (size_t)(Number_of_fihd_cells + 1) * sizeof(int);
  int rc = -1;
  dspecies ds[3];
  memset(ds, 0, sizeof ds);
  CUdeviceptr e_temp = 0, dvxg = 0, dvyg = 0, dvzg = 0, dpx = 0, dpy = 0, dpz = 0;
  CUdeviceptr dvxd[2] = {0, 0}, dvyd[2] = {0, 0}, dvzd[2] = {0, 0}, dtsav[2] = {0, 0}, depsc[2] = {0, 0};
  int *Cell[3] = {0, 0, 0}, *Ne[3] = {0, 0, 0}, *Nn[3] = {0, 0, 0};
  idic_cells C;
  memset(&C, 0, sizeof C);
  void *hbufs[64];
  int nh = 0;
#define HALLOC(ptr, bytes)                              \
  do {                                                  \
    *(void **)&(ptr) = calloc(1, (bytes));              \
    if (!(ptr)) { fail("host allocation failed"); goto out; } \
    hbufs[nh++] = (void *)(ptr);                        \
  } while (0)
  for (int s = 0; s < 3; s++) {
    HALLOC(Cell[s], fc);
    HALLOC(Ne[s], fc);
    HALLOC(Nn[s], ni);
  }
  HALLOC(C.vxg, cd); HALLOC(C.vyg, cd); HALLOC(C.vzg, cd); HALLOC(C.rhog, cd); HALLOC(C.eg, cd);
  HALLOC(C.psix, cd); HALLOC(C.psiy, cd); HALLOC(C.psiz, cd);
  HALLOC(C.yx, cd); HALLOC(C.yy, cd); HALLOC(C.yz, cd); HALLOC(C.ynx, cd); HALLOC(C.yny, cd); HALLOC(C.ynz, cd);
  HALLOC(C.beta, cd);
  HALLOC(C.gcount, (size_t)(Number_of_average_cell + 1) * sizeof(int));
  for (int k = 0; k < 2; k++) {
    HALLOC(C.vxd[k], cd); HALLOC(C.vyd[k], cd); HALLOC(C.vzd[k], cd); HALLOC(C.rhod[k], cd);
    HALLOC(C.epsc[k], cd); HALLOC(C.tsav[k], cd); HALLOC(C.bcell[k], cd);
    HALLOC(C.xx[k], cd); HALLOC(C.xy[k], cd); HALLOC(C.xz[k], cd);
    HALLOC(C.xnx[k], cd); HALLOC(C.xny[k], cd); HALLOC(C.xnz[k], cd);
    HALLOC(C.dcount[k], (size_t)(Number_of_average_cell + 1) * sizeof(int));
  }
#undef HALLOC

  /* device arrays and the initial copies (kernel.cu:1800-1865) */
  for (int s = 0; s < 3; s++) {
    dspecies *d = &ds[s];
    CUdeviceptr *dbl[] = {&d->x, &d->y, &d->z, &d->vx, &d->vy, &d->vz, &d->ax, &d->ay, &d->az, &d->rho, &d->p,
                          &d->e, &d->m, &d->ts};
    for (size_t q = 0; q < sizeof dbl / sizeof dbl[0]; q++) CU(D.MemAlloc(dbl[q], nd), "cudaMalloc");
    CU(D.MemAlloc(&d->ind, ni), "cudaMalloc");
    CU(D.MemAlloc(&d->nn, ni), "cudaMalloc");
    CU(D.MemAlloc(&d->cell, fc), "cudaMalloc");
    const orc_species *o = &sp[s];
    const double *src[] = {o->x, o->y, o->z, o->vx, o->vy, o->vz, o->ax, o->ay, o->az, o->rho, o->p, o->e, o->m,
                           o->ts};
    for (size_t q = 0; q < sizeof dbl / sizeof dbl[0]; q++)
      if (src[q] && h2d(*dbl[q], src[q], nd)) goto out;
    if (h2d(d->ind, o->ind, ni)) goto out;
  }
  CU(D.MemAlloc(&e_temp, nd), "cudaMalloc");
  CU(D.MemAlloc(&dvxg, cd), "cudaMalloc"); CU(D.MemAlloc(&dvyg, cd), "cudaMalloc"); CU(D.MemAlloc(&dvzg, cd), "cudaMalloc");
  CU(D.MemAlloc(&dpx, cd), "cudaMalloc"); CU(D.MemAlloc(&dpy, cd), "cudaMalloc"); CU(D.MemAlloc(&dpz, cd), "cudaMalloc");
  for (int k = 0; k < 2; k++) {
    CU(D.MemAlloc(&dvxd[k], cd), "cudaMalloc"); CU(D.MemAlloc(&dvyd[k], cd), "cudaMalloc");
    CU(D.MemAlloc(&dvzd[k], cd), "cudaMalloc"); CU(D.MemAlloc(&dtsav[k], cd), "cudaMalloc");
    CU(D.MemAlloc(&depsc[k], cd), "cudaMalloc");
  }

  orc_species *gas = &sp[0];
  for (int k = 0; k < PH_N; k++) g_phase[k] = 0.0;  /* the steps only, not the set-up above */
  for (int step = 0; step < nsteps; step++) {
    const double t0 = now_s();
    *Tm = *Tm + tau; /* kernel.cu:1931 */

    /* cell lists of the three species, then up (kernel.cu:1937-2005) */
    double th = now_s();
    for (int s = 0; s < 3; s++)
      build_list(&sp[s], Pm, Clx, Cly, Clz, Clh, Cnx, Cny, Number_of_fihd_cells, Cell[s], Ne[s], Nn[s]);
    g_phase[PH_LISTS] += now_s() - th;
    for (int s = 0; s < 3; s++) {
      if (h2d(ds[s].cell, Cell[s], fc) || h2d(ds[s].nn, Nn[s], ni)) goto out;
    }

    /* densities (kernel.cu:2011-2046) */
    {
      void *a[] = {&ds[0].rho, &ds[1].rho, &ds[2].rho, &ds[0].ind, (void *)&Pm};
      if (launch(K_RHO_INIT, a, 1)) goto out;
    }
    double Clx_ = Clx, Cly_ = Cly, Clz_ = Clz, Clh_ = Clh, h_ = h;
    int Cnx_ = Cnx, Cny_ = Cny, Cl_ = Number_of_fihd_cells, Pm_ = Pm;
    for (int s = 0; s < 3; s++) {
      for (int k = -1; k <= 1; k++)
        for (int l = -1; l <= 1; l++)
          for (int g = -1; g <= 1; g++) {
            int k_ = k, l_ = l, g_ = g;
            void *a[] = {&ds[s].x, &ds[s].y, &ds[s].z, &ds[s].rho, &ds[s].m, &ds[s].ind, &ds[s].cell, &ds[s].nn,
                         &Pm_, &Clx_, &Cly_, &Clz_, &Clh_, &Cnx_, &Cny_, &Cl_, &h_, &k_, &l_, &g_};
            if (launch(K_RHO, a, 1)) goto out;
          }
      if (s == 0) {
        int tos = Type_of_state;
        double gam = Gam_g, cs = Speed_of_sound_gas;
        void *a[] = {&ds[0].rho, &ds[0].p, &ds[0].e, &ds[0].ind, &Pm_, &tos, &gam, &cs};
        if (launch(K_P, a, 1)) goto out;
        if (d2h(gas->rho, ds[0].rho, nd) || d2h(gas->p, ds[0].p, nd)) goto out;
      }
    }
    if (d2h(sp[1].rho, ds[1].rho, nd) || d2h(sp[2].rho, ds[2].rho, nd)) goto out;

    /* stopping times from the gas at the same index (kernel.cu:2049-2056) */
    for (int k = 0; k < 2; k++) {
      double R = R_dust[k], gam = Gam_g;
      void *a[] = {&ds[1 + k].ts, &ds[0].p, &ds[0].rho, &ds[1 + k].ind, &Pm_, &R, &gam};
      if (launch(K_TSTOP, a, 1)) goto out;
    }
    if (d2h(sp[1].ts, ds[1].ts, nd) || d2h(sp[2].ts, ds[2].ts, nd)) goto out;

    /* IDIC cell averages on the host (kernel.cu:2060-2211) */
    th = now_s();
    for (int i = 0; i <= Number_of_average_cell; i++) {
      C.vxg[i] = C.vyg[i] = C.vzg[i] = C.rhog[i] = C.eg[i] = 0.0;
      C.gcount[i] = 0;
      C.psix[i] = C.psiy[i] = C.psiz[i] = 0.0;
      C.ynx[i] = C.yny[i] = C.ynz[i] = C.yx[i] = C.yy[i] = C.yz[i] = 0.0;
      for (int k = 0; k < 2; k++) {
        C.vxd[k][i] = C.vyd[k][i] = C.vzd[k][i] = C.rhod[k][i] = C.epsc[k][i] = C.tsav[k][i] = 0.0;
        C.dcount[k][i] = 0;
        C.xnx[k][i] = C.xny[k][i] = C.xnz[k][i] = C.xx[k][i] = C.xy[k][i] = C.xz[k][i] = 0.0;
        C.bcell[k][i] = 0.0;
      }
    }
    /* every index below is checked once, here: the kernels index the cell
     * arrays with the same positions (no particle moves before they run) */
    for (int s = 0; s < 3; s++)
      for (int p = 0; p <= Pm; p++) {
        const int c = idic_index(&sp[s], p, X_min, Y_min, Z_min, average_cell_width, Nax, Nay);
        if (c < 0 || c > Number_of_average_cell)
          { fail("species %d particle %d: IDIC cell %d outside [0, %d] (step %d)", s, p, c,
                 Number_of_average_cell, step); goto out; }
      }
    for (int p = 0; p <= Pm; p++) {
      const int c = idic_index(gas, p, X_min, Y_min, Z_min, average_cell_width, Nax, Nay);
      C.gcount[c] = C.gcount[c] + 1;
      C.vxg[c] = C.vxg[c] + gas->vx[p];
      C.vyg[c] = C.vyg[c] + gas->vy[p];
      C.vzg[c] = C.vzg[c] + gas->vz[p];
      C.rhog[c] = C.rhog[c] + gas->rho[p];
      C.eg[c] = C.eg[c] + gas->e[p];
    }
    for (int i = 0; i <= Number_of_average_cell; i++)
      if (C.gcount[i] > 0) {
        C.vxg[i] = C.vxg[i] / C.gcount[i];
        C.vyg[i] = C.vyg[i] / C.gcount[i];
        C.vzg[i] = C.vzg[i] / C.gcount[i];
        C.eg[i] = C.eg[i] / C.gcount[i];
      }
    for (int k = 0; k < 2; k++) {
      const orc_species *d = &sp[1 + k];
      for (int p = 0; p <= Pm; p++) {
        const int c = idic_index(d, p, X_min, Y_min, Z_min, average_cell_width, Nax, Nay);
        C.dcount[k][c] = C.dcount[k][c] + 1;
        C.tsav[k][c] = C.tsav[k][c] + d->ts[p];
        C.vxd[k][c] = C.vxd[k][c] + d->vx[p];
        C.vyd[k][c] = C.vyd[k][c] + d->vy[p];
        C.vzd[k][c] = C.vzd[k][c] + d->vz[p];
        C.rhod[k][c] = C.rhod[k][c] + d->rho[p];
      }
      for (int i = 0; i <= Number_of_average_cell; i++) {
        if (C.dcount[k][i] > 0) {
          C.vxd[k][i] = C.vxd[k][i] / C.dcount[k][i];
          C.vyd[k][i] = C.vyd[k][i] / C.dcount[k][i];
          C.vzd[k][i] = C.vzd[k][i] / C.dcount[k][i];
          C.rhod[k][i] = C.rhod[k][i] / C.dcount[k][i];
          C.tsav[k][i] = C.tsav[k][i] / C.dcount[k][i];
        } else {
          C.tsav[k][i] = t_empty;
        }
      }
    }
    /* both species' guards test the count of species 1 (kernel.cu:2195-2210) */
    for (int i = 0; i <= Number_of_average_cell; i++)
      for (int k = 0; k < 2; k++)
        C.epsc[k][i] = (C.gcount[i] > 0 && C.dcount[0][i] > 0) ? C.dcount[k][i] * mas_gas_dust[k] / C.gcount[i]
                                                                : eps_empty[k];
    g_phase[PH_IDIC] += now_s() - th;

    /* force and energy rate (kernel.cu:2229-2268) */
    {
      void *a[] = {&e_temp, &ds[0].ind, &Pm_};
      if (launch(K_E_INIT, a, 1)) goto out;
    }
    {
      void *a[] = {&ds[0].ax, &ds[0].ay, &ds[0].az, &ds[0].ind, &Pm_};
      if (launch(K_F_INIT, a, 1)) goto out;
    }
    {
      double tau_ = tau, gam = Gam_g, al = alpha, be = beta, ep = eps;
      for (int k = -1; k <= 1; k++)
        for (int l = -1; l <= 1; l++)
          for (int g = -1; g <= 1; g++) {
            int k_ = k, l_ = l, g_ = g;
            void *a[] = {&ds[0].x, &ds[0].y, &ds[0].z, &ds[0].rho, &ds[0].p, &ds[0].m, &e_temp, &ds[0].vx, &ds[0].vy,
                         &ds[0].vz, &ds[0].ax, &ds[0].ay, &ds[0].az, &ds[0].ind, &ds[0].cell, &ds[0].nn, &Pm_,
                         &Clx_, &Cly_, &Clz_, &Clh_, &Cnx_, &Cny_, &Cl_, &h_, &tau_, &gam, &al, &be, &ep,
                         &k_, &l_, &g_};
            if (launch(K_FORCE, a, 1)) goto out;
          }
    }
    if (d2h(gas->ax, ds[0].ax, nd) || d2h(gas->ay, ds[0].ay, nd) || d2h(gas->az, ds[0].az, nd)) goto out;

    /* cell means of the gas acceleration and the two-species implicit solve
     * (kernel.cu:2294-2437) */
    th = now_s();
    for (int p = 0; p <= Pm; p++) {
      const int c = idic_index(gas, p, X_min, Y_min, Z_min, average_cell_width, Nax, Nay);
      C.psix[c] = C.psix[c] + gas->ax[p];
      C.psiy[c] = C.psiy[c] + gas->ay[p];
      C.psiz[c] = C.psiz[c] + gas->az[p];
    }
    for (int i = 0; i <= Number_of_average_cell; i++) {
      if (C.gcount[i] > 0) {
        C.psix[i] = C.psix[i] / C.gcount[i];
        C.psiy[i] = C.psiy[i] / C.gcount[i];
        C.psiz[i] = C.psiz[i] / C.gcount[i];
      }
      C.yx[i] = C.vxg[i];
      C.yy[i] = C.vyg[i];
      C.yz[i] = C.vzg[i];
      for (int k = 0; k < 2; k++) {
        C.xx[k][i] = C.vxg[i] - C.vxd[k][i];
        C.xy[k][i] = C.vyg[i] - C.vyd[k][i];
        C.xz[k][i] = C.vzg[i] - C.vzd[k][i];
      }
      C.yx[i] = C.yx[i] + C.epsc[0][i] * C.vxd[0][i] + C.epsc[1][i] * C.vxd[1][i];
      C.yy[i] = C.yy[i] + C.epsc[0][i] * C.vyd[0][i] + C.epsc[1][i] * C.vyd[1][i];
      C.yz[i] = C.yz[i] + C.epsc[0][i] * C.vzd[0][i] + C.epsc[1][i] * C.vzd[1][i];
      for (int k = 0; k < 2; k++) C.bcell[k][i] = (C.tsav[k][i] + tau) / (C.epsc[k][i] * tau);
    }
    for (int i = 0; i <= Number_of_average_cell; i++) {
      C.beta[i] = 1.0;
      C.beta[i] = C.beta[i] + 1.0 / C.bcell[0][i] + 1.0 / C.bcell[1][i];
    }
    for (int i = 0; i <= Number_of_average_cell; i++) {
      const double b1 = C.bcell[0][i], b2 = C.bcell[1][i], be = C.beta[i];
      const double psi[3] = {C.psix[i], C.psiy[i], C.psiz[i]};
      double *yv[3] = {&C.yx[i], &C.yy[i], &C.yz[i]};
      double *yn[3] = {&C.ynx[i], &C.yny[i], &C.ynz[i]};
      for (int a = 0; a < 3; a++) *yn[a] = *yv[a] + tau * psi[a];
      double *x1[3] = {&C.xx[0][i], &C.xy[0][i], &C.xz[0][i]}, *x2[3] = {&C.xx[1][i], &C.xy[1][i], &C.xz[1][i]};
      double *n1[3] = {&C.xnx[0][i], &C.xny[0][i], &C.xnz[0][i]}, *n2[3] = {&C.xnx[1][i], &C.xny[1][i], &C.xnz[1][i]};
      for (int a = 0; a < 3; a++) {
        *n1[a] = -1.0 * b1 * be * (*x1[a] + tau * psi[a]) / (b1 * b1);
        *n1[a] = *n1[a] + (*x1[a] + tau * psi[a]) / (b1 * b1) + (*x2[a] + tau * psi[a]) / (b1 * b2);
        *n1[a] = *n1[a] * (-1.0 * C.tsav[0][i]) / (tau * C.epsc[0][i] * be);
      }
      for (int a = 0; a < 3; a++) {
        *n2[a] = -1.0 * b2 * be * (*x2[a] + tau * psi[a]) / (b2 * b2);
        *n2[a] = *n2[a] + (*x1[a] + tau * psi[a]) / (b2 * b1) + (*x2[a] + tau * psi[a]) / (b2 * b2);
        *n2[a] = *n2[a] * (-1.0 * C.tsav[1][i]) / (tau * C.epsc[1][i] * be);
      }
    }
    for (int i = 0; i <= Number_of_average_cell; i++) {
      const double e1 = C.epsc[0][i], e2 = C.epsc[1][i];
      double tmp1 = 1.0;
      tmp1 = tmp1 + e1 + e2;
      double *vg[3] = {&C.vxg[i], &C.vyg[i], &C.vzg[i]};
      double *v1[3] = {&C.vxd[0][i], &C.vyd[0][i], &C.vzd[0][i]}, *v2[3] = {&C.vxd[1][i], &C.vyd[1][i], &C.vzd[1][i]};
      const double yn[3] = {C.ynx[i], C.yny[i], C.ynz[i]};
      const double n1[3] = {C.xnx[0][i], C.xny[0][i], C.xnz[0][i]}, n2[3] = {C.xnx[1][i], C.xny[1][i], C.xnz[1][i]};
      for (int a = 0; a < 3; a++) *vg[a] = yn[a];
      for (int a = 0; a < 3; a++) *vg[a] = *vg[a] + e1 * n1[a];
      for (int a = 0; a < 3; a++) *v1[a] = yn[a];
      for (int a = 0; a < 3; a++) *v1[a] = *v1[a] + e2 * n2[a];
      for (int a = 0; a < 3; a++) *v1[a] = *v1[a] - (tmp1 - e1) * n1[a];
      for (int a = 0; a < 3; a++) *v1[a] = *v1[a] / tmp1;
      for (int a = 0; a < 3; a++) *vg[a] = *vg[a] + e2 * n2[a];
      for (int a = 0; a < 3; a++) *v2[a] = yn[a];
      for (int a = 0; a < 3; a++) *v2[a] = *v2[a] + e1 * n1[a];
      for (int a = 0; a < 3; a++) *v2[a] = *v2[a] - (tmp1 - e2) * n2[a];
      for (int a = 0; a < 3; a++) *v2[a] = *v2[a] / tmp1;
      for (int a = 0; a < 3; a++) *vg[a] = *vg[a] / tmp1;
    }

    g_phase[PH_IDIC] += now_s() - th;

    /* relaxation on the device (kernel.cu:2453-2495) */
    if (h2d(dvxg, C.vxg, cd) || h2d(dvyg, C.vyg, cd) || h2d(dvzg, C.vzg, cd)) goto out;
    for (int k = 0; k < 2; k++)
      if (h2d(dvxd[k], C.vxd[k], cd) || h2d(dvyd[k], C.vyd[k], cd) || h2d(dvzd[k], C.vzd[k], cd) ||
          h2d(dtsav[k], C.tsav[k], cd) || h2d(depsc[k], C.epsc[k], cd))
        goto out;
    {
      double xm = X_min, ym = Y_min, zm = Z_min, aw = average_cell_width, tau_ = tau;
      int nax = Nax, nay = Nay, nac = Number_of_average_cell;
      for (int k = 0; k < 2; k++) {
        dspecies *d = &ds[1 + k];
        void *a[] = {&d->x, &d->y, &d->z, &d->vx, &d->vy, &d->vz, &dvxg, &dvyg, &dvzg, &dtsav[k], &d->ind,
                     &xm, &ym, &zm, &aw, &nax, &nay, &nac, &tau_, &Pm_};
        /* the reference synchronizes after the first only; the copies below block */
        if (launch(K_V_DUST, a, k == 0)) goto out;
      }
      for (int k = 0; k < 2; k++)
        if (d2h(sp[1 + k].vx, ds[1 + k].vx, nd) || d2h(sp[1 + k].vy, ds[1 + k].vy, nd) ||
            d2h(sp[1 + k].vz, ds[1 + k].vz, nd))
          goto out;
      if (h2d(dpx, C.psix, cd) || h2d(dpy, C.psiy, cd) || h2d(dpz, C.psiz, cd)) goto out;
      void *a[] = {&ds[0].x, &ds[0].y, &ds[0].z, &ds[0].vx, &ds[0].vy, &ds[0].vz, &dvxd[0], &dvyd[0], &dvzd[0],
                   &dvxd[1], &dvyd[1], &dvzd[1], &dpx, &dpy, &dpz, &dtsav[0], &dtsav[1], &depsc[0], &depsc[1],
                   &ds[0].ind, &xm, &ym, &zm, &aw, &nax, &nay, &nac, &tau_, &Pm_};
      if (launch(K_V_GAS, a, 1)) goto out;
      if (d2h(gas->vx, ds[0].vx, nd) || d2h(gas->vy, ds[0].vy, nd) || d2h(gas->vz, ds[0].vz, nd)) goto out;

      /* move every species, then the energy (kernel.cu:2497-2523) */
      for (int s = 0; s < 3; s++) {
        void *m[] = {&ds[s].x, &ds[s].y, &ds[s].z, &ds[s].vx, &ds[s].vy, &ds[s].vz, &ds[s].ind, &tau_, &Pm_};
        if (launch(K_MOVE, m, 1)) goto out;
      }
      for (int s = 0; s < 3; s++)
        if (d2h(sp[s].x, ds[s].x, nd) || d2h(sp[s].y, ds[s].y, nd) || d2h(sp[s].z, ds[s].z, nd)) goto out;
      void *en[] = {&ds[0].e, &e_temp, &ds[0].ind, &tau_, &Pm_};
      if (launch(K_ENERGY, en, 1)) goto out;
      if (d2h(gas->e, ds[0].e, nd)) goto out;
    }
    if (step_s) step_s[step] = now_s() - t0;
  }
  rc = 0;
out:
  for (int s = 0; s < 3; s++) {
    dspecies *d = &ds[s];
    CUdeviceptr all[] = {d->x, d->y, d->z, d->vx, d->vy, d->vz, d->ax, d->ay, d->az, d->rho, d->p, d->e, d->m,
                         d->ts, d->ind, d->cell, d->nn};
    for (size_t q = 0; q < sizeof all / sizeof all[0]; q++)
      if (all[q]) D.MemFree(all[q]);
  }
  CUdeviceptr rest[] = {e_temp, dvxg, dvyg, dvzg, dpx, dpy, dpz, dvxd[0], dvyd[0], dvzd[0], dtsav[0], depsc[0],
                        dvxd[1], dvyd[1], dvzd[1], dtsav[1], depsc[1]};
  for (size_t q = 0; q < sizeof rest / sizeof rest[0]; q++)
    if (rest[q]) D.MemFree(rest[q]);
  for (int q = 0; q < nh; q++) free(hbufs[q]);
  return rc;
}
