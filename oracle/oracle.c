/*
 * oracle.c -- FP64 CPU restatement of DustyShock3D's per-step hot path.
 *
 * TEST INFRASTRUCTURE (see oracle.h): the checker for the CUDA path and the
 * timed CPU baseline.  Never linked into or called by the product.
 *
 * Every function cites the reference lines it restates.  In reference mode the
 * arithmetic is written in the reference's own operation order and summation
 * order (27 offsets k,l,g; linked lists in ascending particle index; per-offset
 * partial density sums; direct force accumulation; host cell loops in particle
 * order), and the build uses -ffp-contract=off, so a reference-mode step equals
 * the reference's own CPU build bit for bit, except that the neighbour distance
 * uses the correctly rounded sqrt(r^2) where the reference writes pow(r^2, 0.5)
 * (IDIC.h:37, 219).  The two agree except in rare last-bit cases.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Truncated constant used by the reference's kernels (kernel.cu:14, 27). */
static const double ORC_PI = 3.14159265;

/* M4 cubic spline, kernel.cu:12-23. */
static double orc_W(double r, double h) {
  const double c = (double)1 / (ORC_PI);
  double k = (double)fabs(r) / h, tmp1 = 0.0;
  if (k < 1.0) tmp1 = (double)1.0 - 1.5 * k * k + 0.75 * k * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = (double)0.25 * (2.0 - k) * (2.0 - k) * (2.0 - k);
  if (k > 2.0) tmp1 = 0.0;
  return c / (h * h * h) * tmp1;
}

/* Signed kernel derivative, kernel.cu:25-39 (sequential ifs: the later
 * matching branch wins at k = -1, 0, 1, 2). */
static double orc_dW(double r, double h) {
  const double c = (double)1 / (ORC_PI);
  double k = (double)r / h, tmp1 = 0.0;
  if (k < -2.0) tmp1 = 0.0;
  if ((k >= -2.0) && (k <= -1.0)) tmp1 = (double)0.75 * (2.0 + k) * (2.0 + k);
  if ((k > -1.0) && (k < 0)) tmp1 = (double)-3.0 * k - 2.25 * k * k;
  if ((k >= 0) && (k <= 1.0)) tmp1 = (double)-3.0 * k + 2.25 * k * k;
  if ((k >= 1.0) && (k <= 2.0)) tmp1 = (double)-0.75 * (2.0 - k) * (2.0 - k);
  if (k > 2.0) tmp1 = 0.0;
  return c / (h * h * h * h) * tmp1;
}

/* Equation of state, kernel.cu:92-97. */
static double orc_eq_state(double rho, double e, int type, double gam, double cs) {
  if (type == 1) return cs * cs * rho;
  return rho * e * (gam - 1);
}

/* ------------------------------------------------------------------------ */
/* Grids                                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
  /* neighbour grid (kernel.cu:1767-1778) */
  double ox, oy, oz, wx, wy, wz, Ly, Lz;
  int Cnx, Cny, Cnz;  /* int((max - min) / Clh) */
  int nx, ny, nz;     /* cells per axis of the proper grid */
  int sy, sz;         /* key strides */
  int ncells;         /* Number_of_fihd_cells */
  int proper, per_y, per_z;
  /* IDIC grid (kernel.cu:1577-1582) */
  double aw;
  int Nax, Nay, Naz, asy, asz, n_idic; /* n_idic = Number_of_average_cell */
  int aproper, anx, any, anz;
} orc_grid;

static void orc_grid_setup(const orc_params *P, orc_grid *G) {
  memset(G, 0, sizeof(*G));
  G->ox = P->X_min; G->oy = P->Y_min; G->oz = P->Z_min;
  double w = P->cell_w;
  G->Cnx = (int)((P->X_max - P->X_min) / w);
  G->Cny = (int)((P->Y_max - P->Y_min) / w);
  G->Cnz = (int)((P->Z_max - P->Z_min) / w);
  G->proper = (P->flags & ORC_GRID_PROPER) != 0;
  G->per_y = (P->flags & ORC_PERIODIC_Y) != 0;
  G->per_z = (P->flags & ORC_PERIODIC_Z) != 0;
  G->Ly = P->Y_max - P->Y_min;
  G->Lz = P->Z_max - P->Z_min;
  G->wx = G->wy = G->wz = w;
  if (!G->proper) {
    G->sy = G->Cnx;
    G->sz = G->Cnx * G->Cny;
    G->ncells = (G->Cnx + 1) * (G->Cny + 1) * (G->Cnz + 1);
    G->nx = G->Cnx + 1; G->ny = G->Cny + 1; G->nz = G->Cnz + 1;
  } else {
    G->nx = G->Cnx + 1;
    G->ny = G->per_y ? (int)(G->Ly / w) : G->Cny + 1;
    G->nz = G->per_z ? (int)(G->Lz / w) : G->Cnz + 1;
    if (G->ny < 1) G->ny = 1;
    if (G->nz < 1) G->nz = 1;
    if (G->per_y) G->wy = G->Ly / G->ny;
    if (G->per_z) G->wz = G->Lz / G->nz;
    G->sy = G->nx;
    G->sz = G->nx * G->ny;
    G->ncells = G->nx * G->ny * G->nz;
  }
  G->aw = P->idic_w;
  G->Nax = (int)((P->X_max - P->X_min) / G->aw);
  G->Nay = (int)((P->Y_max - P->Y_min) / G->aw);
  G->Naz = (int)((P->Z_max - P->Z_min) / G->aw);
  G->n_idic = (G->Nax + 1) * (G->Nay + 1) * (G->Naz + 1);
  G->aproper = (P->flags & ORC_IDIC_PROPER) != 0;
  G->anx = G->Nax + 1; G->any = G->Nay + 1; G->anz = G->Naz + 1;
  if (!G->aproper) {
    G->asy = G->Nax;
    G->asz = G->Nax * G->Nay;
  } else {
    G->asy = G->anx;
    G->asz = G->anx * G->any;
  }
}

/* Per-axis cell coordinates of a position in the proper grid (extension):
 * floor division, periodic axes clamped into range after the wrap. */
static void orc_proper_cell(const orc_grid *G, double x, double y, double z, int *ix, int *iy, int *iz) {
  *ix = (int)floor((x - G->ox) / G->wx);
  *iy = (int)floor((y - G->oy) / G->wy);
  *iz = (int)floor((z - G->oz) / G->wz);
  if (G->per_y) { if (*iy < 0) *iy = 0; if (*iy >= G->ny) *iy = G->ny - 1; }
  if (G->per_z) { if (*iz < 0) *iz = 0; if (*iz >= G->nz) *iz = G->nz - 1; }
}

/* Raw neighbour-cell key, kernel.cu:1949 / IDIC.h:28.  In the proper grid an
 * out-of-range axis gives -1 (not listed). */
static int orc_key(const orc_grid *G, double x, double y, double z) {
  if (!G->proper)
    return (int)((x - G->ox) / G->wx) + ((int)((y - G->oy) / G->wx)) * G->Cnx +
           ((int)((z - G->oz) / G->wx)) * G->Cnx * G->Cny;
  int ix, iy, iz;
  orc_proper_cell(G, x, y, z, &ix, &iy, &iz);
  if (ix < 0 || ix >= G->nx || iy < 0 || iy >= G->ny || iz < 0 || iz >= G->nz) return -1;
  return ix + iy * G->sy + iz * G->sz;
}

/* Raw IDIC cell index, kernel.cu:2116 (no bounds check in the reference). */
static int orc_idic_key(const orc_grid *G, double x, double y, double z) {
  if (!G->aproper)
    return (int)((x - G->ox) / G->aw) + ((int)((y - G->oy) / G->aw)) * G->Nax +
           ((int)((z - G->oz) / G->aw)) * G->Nax * G->Nay;
  int ix = (int)floor((x - G->ox) / G->aw);
  int iy = (int)floor((y - G->oy) / G->aw);
  int iz = (int)floor((z - G->oz) / G->aw);
  if (ix < 0 || ix >= G->anx || iy < 0 || iy >= G->any || iz < 0 || iz >= G->anz) return -1;
  return ix + iy * G->asy + iz * G->asz;
}

/* ------------------------------------------------------------------------ */
/* Neighbour lists, kernel.cu:1937-1955                                      */
/* ------------------------------------------------------------------------ */

static void orc_list(const orc_grid *G, const orc_species *s, int *head, int *next, int *tail) {
  for (int i = 0; i <= G->ncells; i++) head[i] = -1;
  for (int p = 0; p < s->n; p++) next[p] = -1;
  for (int p = 0; p < s->n; p++) {
    int i = orc_key(G, s->x[p], s->y[p], s->z[p]);
    if ((i >= 0) && (i <= G->ncells)) {
      if (head[i] == -1) { head[i] = p; tail[i] = p; next[p] = -1; }
      else { next[tail[i]] = p; tail[i] = p; next[p] = -1; }
    }
  }
}

/* The neighbour cells of a particle in the reference's launch order (k = x
 * offset outer, l = y, g = z inner; kernel.cu:2014-2016) with the validity
 * test of IDIC.h:30-31: 27 cells for stencil 1 (the reference), 125 for
 * stencil 2 (extension: cells of half the width).  Proper grid: same order,
 * per-axis range checks, periodic wrap with image shifts.  Invalid offsets
 * get cell -1. */
#define ORC_MAX_OFS 125
typedef struct { int n; int cell[ORC_MAX_OFS]; double sx[ORC_MAX_OFS], sy[ORC_MAX_OFS], sz[ORC_MAX_OFS]; } orc_stencil;

static void orc_make_stencil(const orc_grid *G, int R, double x, double y, double z, orc_stencil *st) {
  int o = 0;
  if (!G->proper) {
    int Ni = orc_key(G, x, y, z);
    for (int k = -R; k <= R; k++)
      for (int l = -R; l <= R; l++)
        for (int g = -R; g <= R; g++, o++) {
          int Ci = Ni + k + l * G->Cnx + g * G->Cnx * G->Cny;
          st->cell[o] = ((Ci > -1) && (Ci < G->ncells)) ? Ci : -1;
          st->sx[o] = st->sy[o] = st->sz[o] = 0.0;
        }
    st->n = o;
    return;
  }
  int ix, iy, iz;
  orc_proper_cell(G, x, y, z, &ix, &iy, &iz);
  for (int k = -R; k <= R; k++)
    for (int l = -R; l <= R; l++)
      for (int g = -R; g <= R; g++, o++) {
        int cx = ix + k, cy = iy + l, cz = iz + g;
        double sy = 0.0, sz = 0.0;
        int ok = (cx >= 0 && cx < G->nx);
        if (G->per_y) {
          if (cy < 0) { cy += G->ny; sy = -G->Ly; }
          else if (cy >= G->ny) { cy -= G->ny; sy = G->Ly; }
        }
        if (G->per_z) {
          if (cz < 0) { cz += G->nz; sz = -G->Lz; }
          else if (cz >= G->nz) { cz -= G->nz; sz = G->Lz; }
        }
        ok = ok && cy >= 0 && cy < G->ny && cz >= 0 && cz < G->nz;
        st->cell[o] = ok ? cx + cy * G->sy + cz * G->sz : -1;
        st->sx[o] = 0.0; st->sy[o] = sy; st->sz[o] = sz;
      }
  st->n = o;
}

/* Difference of a neighbour coordinate (with its image shift) and ours. */
static inline double orc_diff(double xj, double s, double xi) { return s != 0.0 ? (xj + s) - xi : xj - xi; }

/* ------------------------------------------------------------------------ */
/* Sweeps                                                                     */
/* ------------------------------------------------------------------------ */

/* Density, IDIC.h:17-45 launched 27x (kernel.cu:2014-2021); the caller has
 * zeroed rho where the particle updates (IDIC.h:2-14). */
static void orc_density(const orc_params *P, const orc_grid *G, orc_species *s, const int *head,
                        const int *next, const int *upd) {
  const int hpp = (P->flags & ORC_H_PER_PARTICLE) != 0;
  const int R = P->stencil == 2 ? 2 : 1;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s->n; i++) {
    if (!upd[i]) continue;
    orc_stencil st;
    orc_make_stencil(G, R, s->x[i], s->y[i], s->z[i], &st);
    const double hi = hpp ? s->h[i] : P->h;
    for (int o = 0; o < st.n; o++) {
      double rho_tmp = 0.0;
      if (st.cell[o] >= 0) {
        int j = head[st.cell[o]];
        while (j > -1) {
          double dx = orc_diff(s->x[j], st.sx[o], s->x[i]);
          double dy = orc_diff(s->y[j], st.sy[o], s->y[i]);
          double dz = orc_diff(s->z[j], st.sz[o], s->z[i]);
          double d = sqrt(dx * dx + dy * dy + dz * dz);
          rho_tmp = rho_tmp + s->m[j] * orc_W(d, hi);
          j = next[j];
        }
      }
      s->rho[i] = s->rho[i] + rho_tmp;
    }
  }
}

/* Force and energy rate, IDIC.h:198-260 launched 27x (kernel.cu:2259-2266);
 * A and e_temp were zeroed where Ind == 0 (IDIC.h:93-103, 183-195). */
static void orc_force(const orc_params *P, const orc_grid *G, orc_species *s, const int *head,
                      const int *next, double *e_temp) {
  const int hpp = (P->flags & ORC_H_PER_PARTICLE) != 0;
  const int R = P->stencil == 2 ? 2 : 1;
  const double Gam_g = P->Gam_g, alpha = P->alpha, beta = P->beta, eps = P->eps;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s->n; i++) {
    if (s->ind[i] != 0) continue;
    orc_stencil st;
    orc_make_stencil(G, R, s->x[i], s->y[i], s->z[i], &st);
    const double hi = hpp ? s->h[i] : P->h;
    for (int o = 0; o < st.n; o++) {
      if (st.cell[o] < 0) continue;
      int j = head[st.cell[o]];
      while (j > -1) {
        double dxj = orc_diff(s->x[j], st.sx[o], s->x[i]);
        double dyj = orc_diff(s->y[j], st.sy[o], s->y[i]);
        double dzj = orc_diff(s->z[j], st.sz[o], s->z[i]);
        double dist = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
        double hj = hpp ? s->h[j] : hi;
        double hcut = hpp ? (hi > hj ? hi : hj) : hi;
        if ((dist < 2 * hcut) && (dist > 0)) {
          /* x_i - x_j, with the neighbour's image shift */
          double xij = st.sx[o] != 0.0 ? s->x[i] - (s->x[j] + st.sx[o]) : s->x[i] - s->x[j];
          double yij = st.sy[o] != 0.0 ? s->y[i] - (s->y[j] + st.sy[o]) : s->y[i] - s->y[j];
          double zij = st.sz[o] != 0.0 ? s->z[i] - (s->z[j] + st.sz[o]) : s->z[i] - s->z[j];
          double hh = hpp ? 0.5 * (hi + hj) : hi;
          double F_nu = 0;
          double nu1x = (s->vx[i] - s->vx[j]) * xij;
          double nu1y = (s->vy[i] - s->vy[j]) * yij;
          double nu1z = (s->vz[i] - s->vz[j]) * zij;
          double nu_temp = nu1x + nu1y + nu1z;
          if (nu_temp < 0.0) {
            double Cnu = 0.5 * (sqrt(Gam_g * s->p[i] / s->rho[i]) + sqrt(Gam_g * s->p[j] / s->rho[j]));
            nu_temp = hh * nu_temp / (dist * dist + eps * hh * hh);
            F_nu = (-alpha * Cnu * nu_temp + beta * nu_temp * nu_temp) / (0.5 * (s->rho[i] + s->rho[j]));
          }
          double dWr = hpp ? 0.5 * (orc_dW(dist, hi) + orc_dW(dist, hj)) : orc_dW(dist, hi);
          e_temp[i] = e_temp[i] + (s->m[i] * s->p[i] / (s->rho[i] * s->rho[i]) + s->m[i] * F_nu / 2.0) *
                                      (nu1x + nu1y + nu1z) * dWr / dist;
          double A = s->m[j] * (s->p[i] / (s->rho[i] * s->rho[i]) + s->p[j] / (s->rho[j] * s->rho[j]) + F_nu) * dWr;
          double d;
          d = dxj; s->ax[i] = s->ax[i] + d * A / dist;
          d = dyj; s->ay[i] = s->ay[i] + d * A / dist;
          d = dzj; s->az[i] = s->az[i] + d * A / dist;
        }
        j = next[j];
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* IDIC per-cell solve, kernel.cu:2310-2437                                  */
/* ------------------------------------------------------------------------ */

void orc_idic_solve_cell(int n, const double *eps, const double *t, double vg, const double *vd, double psi,
                         double tau, int ref2, double *vg_new, double *vd_new) {
  if (ref2 && n == 2) {
    /* The reference's two-species operation order, one velocity component. */
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
    *vg_new = g; vd_new[0] = d1; vd_new[1] = d2;
    return;
  }
  /* General species count: (diag(b) + 1 1^T) u = r by Sherman-Morrison,
   * u_k = eps_k tau x_k^new / t_k; reduces to kernel.cu:2310-2437 for n = 2. */
  double b[ORC_MAX_DUST], r[ORC_MAX_DUST], xn[ORC_MAX_DUST];
  double y = vg, beta = 1.0, S = 0.0, E = 1.0;
  for (int k = 0; k < n; k++) {
    y = y + eps[k] * vd[k];
    b[k] = (t[k] + tau) / (eps[k] * tau);
    beta = beta + 1.0 / b[k];
    r[k] = (vg - vd[k]) + tau * psi;
    S = S + r[k] / b[k];
    E = E + eps[k];
  }
  double yn = y + tau * psi;
  double g = yn;
  for (int k = 0; k < n; k++) {
    double u = r[k] / b[k] - S / (b[k] * beta);
    xn[k] = u * t[k] / (eps[k] * tau);
    g = g + eps[k] * xn[k];
  }
  g = g / E;
  *vg_new = g;
  for (int k = 0; k < n; k++) vd_new[k] = g - xn[k];
}

/* ------------------------------------------------------------------------ */
/* One step, kernel.cu:1929-2523                                              */
/* ------------------------------------------------------------------------ */

/* The step in two parts, as the reference runs it (kernel.cu:1937-2566): the
 * lists, the gas density and the EOS (and the dust density), ending with the
 * CFL candidate min h/(c_s + |v|) over the updated gas (+inf without CFL);
 * then t_stop, the step size, the IDIC averages, the force, the implicit
 * solve and the update.  The split lets a slab decomposition set the ghosts'
 * density and pressure and the global CFL minimum between the parts; orc_step
 * runs both. */
int orc_step_density(const orc_params *P, orc_species *sp, double *dtmin_out) {
  orc_grid G;
  orc_grid_setup(P, &G);
  {
    const int need = 2 * (P->stencil == 2 ? 2 : 1) + 1; /* a periodic axis must not alias its own stencil */
    if ((G.per_y && G.ny < need) || (G.per_z && G.nz < need)) return -1;
  }
  const int nd = P->n_dust, ns = 1 + nd;
  orc_species *gas = &sp[0];
  const int Ng = gas->n;
  const double Gam_g = P->Gam_g;
  const int hpp = (P->flags & ORC_H_PER_PARTICLE) != 0;
  const int coupled = (P->flags & ORC_REF_INDEX_COUPLING) != 0;
  int status = 0;
  if (G.proper) { /* a cut-off 2h past the stencil's cells would miss partners: flag 8 */
    const double reach = 0.5 * (P->stencil == 2 ? 2 : 1) * fmin(G.wx, fmin(G.wy, G.wz)) * (1.0 + 1e-9);
    for (int s = 0; s < ns; s++)
      for (int i = 0; i < sp[s].n; i++)
        if (!((hpp ? sp[s].h[i] : P->h) <= reach)) status |= 8;
  }

  /* lists for every species (kernel.cu:1937-1995) */
  int *head[1 + ORC_MAX_DUST], *next[1 + ORC_MAX_DUST];
  int *tail = (int *)malloc(sizeof(int) * (G.ncells + 1));
  for (int s = 0; s < ns; s++) {
    head[s] = (int *)malloc(sizeof(int) * (G.ncells + 1));
    next[s] = (int *)malloc(sizeof(int) * (sp[s].n > 0 ? sp[s].n : 1));
    orc_list(&G, &sp[s], head[s], next[s], tail);
  }
  free(tail);

  /* Rho_InitKernel_IDIC (IDIC.h:2-14): gas rho where Ind_gas == 0; dust rho
   * by the GAS Ind at the same index in reference mode (quirk), else by the
   * dust's own Ind. */
  for (int i = 0; i < Ng; i++)
    if (gas->ind[i] == 0) gas->rho[i] = 0.0;
  if (P->flags & ORC_DUST_RHO) /* dust rho is output only; untouched when not computed */
    for (int s = 1; s < ns; s++)
      for (int i = 0; i < sp[s].n; i++) {
        int z = coupled ? (i < Ng && gas->ind[i] == 0) : (sp[s].ind[i] == 0);
        if (z) sp[s].rho[i] = 0.0;
      }

  /* gas density + EOS (kernel.cu:2011-2024) */
  {
    int *upd = (int *)malloc(sizeof(int) * (Ng > 0 ? Ng : 1));
    for (int i = 0; i < Ng; i++) upd[i] = gas->ind[i] == 0;
    orc_density(P, &G, gas, head[0], next[0], upd);
    free(upd);
  }
  for (int i = 0; i < Ng; i++)
    if (gas->ind[i] == 0)
      gas->p[i] = orc_eq_state(gas->rho[i], gas->e[i], P->Type_of_state, Gam_g, P->Speed_of_sound_gas);

  /* dust self-density, output only (kernel.cu:2029-2043) */
  if (P->flags & ORC_DUST_RHO)
    for (int s = 1; s < ns; s++) {
      int *upd = (int *)malloc(sizeof(int) * (sp[s].n > 0 ? sp[s].n : 1));
      for (int i = 0; i < sp[s].n; i++) upd[i] = sp[s].ind[i] == 0;
      orc_density(P, &G, &sp[s], head[s], next[s], upd);
      free(upd);
    }

  /* CFL candidate (extension): the smallest h / (c_s + |v|) over the updated gas */
  double dtmin = INFINITY;
  if (P->flags & ORC_CFL)
    for (int i = 0; i < Ng; i++) {
      if (gas->ind[i] != 0) continue;
      double c = sqrt(Gam_g * gas->p[i] / gas->rho[i]);
      double v = sqrt(gas->vx[i] * gas->vx[i] + gas->vy[i] * gas->vy[i] + gas->vz[i] * gas->vz[i]);
      double hi = hpp ? gas->h[i] : P->h;
      double dt = hi / (c + v);
      if (dt < dtmin) dtmin = dt;
    }
  if (dtmin_out) *dtmin_out = dtmin;
  for (int s = 0; s < ns; s++) { free(head[s]); free(next[s]); }
  return status;
}

int orc_step_complete(const orc_params *P, orc_species *sp, double *Tm, double dtmin, double *dt_taken) {
  orc_grid G;
  orc_grid_setup(P, &G);
  const int nd = P->n_dust, ns = 1 + nd;
  orc_species *gas = &sp[0];
  const int Ng = gas->n;
  const double Gam_g = P->Gam_g;
  int status = 0;
  /* the lists again: the positions have not changed since the density part */
  int *head[1 + ORC_MAX_DUST], *next[1 + ORC_MAX_DUST];
  {
    int *tail = (int *)malloc(sizeof(int) * (G.ncells + 1));
    for (int s = 0; s < ns; s++) {
      head[s] = (int *)malloc(sizeof(int) * (G.ncells + 1));
      next[s] = (int *)malloc(sizeof(int) * (sp[s].n > 0 ? sp[s].n : 1));
      orc_list(&G, &sp[s], head[s], next[s], tail);
    }
    free(tail);
  }

  /* stopping time (IDIC.h:78-91, kernel.cu:2049-2053): gas p, rho at the
   * dust particle's index (reference quirk) */
  if (!(P->flags & ORC_TSTOP_CONST)) {
    for (int s = 1; s < ns; s++)
      for (int i = 0; i < sp[s].n; i++)
        if (sp[s].ind[i] == 0 && i < Ng)
          sp[s].ts[i] = P->R_dust[s - 1] / (sqrt(Gam_g * gas->p[i] / gas->rho[i]) * gas->rho[i]);
  } else {
    for (int s = 1; s < ns; s++)
      for (int i = 0; i < sp[s].n; i++)
        if (sp[s].ind[i] == 0) sp[s].ts[i] = P->t_stop_const[s - 1];
  }

  /* step size: fixed tau (kernel.cu:1931) or CFL (extension) */
  double tau = P->tau;
  if (P->flags & ORC_CFL) {
    tau = P->cfl * dtmin;
    if (*Tm + tau > P->T_end) tau = P->T_end - *Tm;
  }

  /* IDIC cell averages (kernel.cu:2060-2211) */
  const int NA = G.n_idic;
  int *cnt = (int *)calloc((size_t)(NA + 1) * ns, sizeof(int));
  double *vx_av = (double *)calloc((size_t)(NA + 1) * ns, sizeof(double));
  double *vy_av = (double *)calloc((size_t)(NA + 1) * ns, sizeof(double));
  double *vz_av = (double *)calloc((size_t)(NA + 1) * ns, sizeof(double));
  double *t_av = (double *)calloc((size_t)(NA + 1) * ns, sizeof(double));
  double *eps_c = (double *)calloc((size_t)(NA + 1) * ns, sizeof(double));
  double *psx = (double *)calloc((size_t)(NA + 1), sizeof(double));
  double *psy = (double *)calloc((size_t)(NA + 1), sizeof(double));
  double *psz = (double *)calloc((size_t)(NA + 1), sizeof(double));
  int *ckey[1 + ORC_MAX_DUST];
  for (int s = 0; s < ns; s++) {
    orc_species *q = &sp[s];
    ckey[s] = (int *)malloc(sizeof(int) * (q->n > 0 ? q->n : 1));
    for (int p = 0; p < q->n; p++) {
      int c = orc_idic_key(&G, q->x[p], q->y[p], q->z[p]);
      if (c < 0 || c > NA) { c = -1; status |= 1; } /* reference: out-of-bounds write */
      ckey[s][p] = c;
      if (c < 0) continue;
      size_t o = (size_t)s * (NA + 1) + c;
      cnt[o] = cnt[o] + 1;
      if (s > 0) t_av[o] = t_av[o] + q->ts[p];
      vx_av[o] = vx_av[o] + q->vx[p];
      vy_av[o] = vy_av[o] + q->vy[p];
      vz_av[o] = vz_av[o] + q->vz[p];
    }
    for (int c = 0; c <= NA; c++) {
      size_t o = (size_t)s * (NA + 1) + c;
      if (cnt[o] > 0) {
        vx_av[o] = vx_av[o] / cnt[o];
        vy_av[o] = vy_av[o] / cnt[o];
        vz_av[o] = vz_av[o] / cnt[o];
        if (s > 0) t_av[o] = t_av[o] / cnt[o];
      } else if (s > 0) {
        t_av[o] = P->t_empty;
      }
    }
  }
  for (int c = 0; c <= NA; c++)
    for (int s = 1; s < ns; s++) {
      int guard = (P->flags & ORC_REF_EPS_GUARD) ? cnt[(size_t)1 * (NA + 1) + c] : cnt[(size_t)s * (NA + 1) + c];
      if ((cnt[c] > 0) && (guard > 0))
        eps_c[(size_t)s * (NA + 1) + c] = cnt[(size_t)s * (NA + 1) + c] * P->mass_ratio[s - 1] / cnt[c];
      else
        eps_c[(size_t)s * (NA + 1) + c] = P->eps_empty[s - 1];
    }

  /* force + energy rate (kernel.cu:2233-2266) */
  double *e_temp = (double *)calloc((size_t)(Ng > 0 ? Ng : 1), sizeof(double));
  for (int i = 0; i < Ng; i++)
    if (gas->ind[i] == 0) { gas->ax[i] = 0.0; gas->ay[i] = 0.0; gas->az[i] = 0.0; }
  orc_force(P, &G, gas, head[0], next[0], e_temp);

  /* Psi = cell mean of A over every gas particle (kernel.cu:2294-2309) */
  for (int p = 0; p < Ng; p++) {
    int c = ckey[0][p];
    if (c < 0) continue;
    psx[c] = psx[c] + gas->ax[p];
    psy[c] = psy[c] + gas->ay[p];
    psz[c] = psz[c] + gas->az[p];
  }
  for (int c = 0; c <= NA; c++)
    if (cnt[c] > 0) { psx[c] = psx[c] / cnt[c]; psy[c] = psy[c] / cnt[c]; psz[c] = psz[c] / cnt[c]; }

  /* per-cell implicit solve (kernel.cu:2310-2437) */
  const int ref2 = (P->flags & ORC_REF_SOLVE2) != 0;
  double *gx = (double *)malloc(sizeof(double) * (NA + 1));
  double *gy = (double *)malloc(sizeof(double) * (NA + 1));
  double *gz = (double *)malloc(sizeof(double) * (NA + 1));
  double *dx_ = (double *)malloc(sizeof(double) * (size_t)(NA + 1) * ns);
  double *dy_ = (double *)malloc(sizeof(double) * (size_t)(NA + 1) * ns);
  double *dz_ = (double *)malloc(sizeof(double) * (size_t)(NA + 1) * ns);
#pragma omp parallel for schedule(static)
  for (int c = 0; c <= NA; c++) {
    double e[ORC_MAX_DUST], t[ORC_MAX_DUST], v[ORC_MAX_DUST], o[ORC_MAX_DUST];
    for (int k = 0; k < nd; k++) {
      size_t q = (size_t)(k + 1) * (NA + 1) + c;
      e[k] = eps_c[q]; t[k] = t_av[q];
    }
    for (int k = 0; k < nd; k++) v[k] = vx_av[(size_t)(k + 1) * (NA + 1) + c];
    orc_idic_solve_cell(nd, e, t, vx_av[c], v, psx[c], tau, ref2, &gx[c], o);
    for (int k = 0; k < nd; k++) dx_[(size_t)(k + 1) * (NA + 1) + c] = o[k];
    for (int k = 0; k < nd; k++) v[k] = vy_av[(size_t)(k + 1) * (NA + 1) + c];
    orc_idic_solve_cell(nd, e, t, vy_av[c], v, psy[c], tau, ref2, &gy[c], o);
    for (int k = 0; k < nd; k++) dy_[(size_t)(k + 1) * (NA + 1) + c] = o[k];
    for (int k = 0; k < nd; k++) v[k] = vz_av[(size_t)(k + 1) * (NA + 1) + c];
    orc_idic_solve_cell(nd, e, t, vz_av[c], v, psz[c], tau, ref2, &gz[c], o);
    for (int k = 0; k < nd; k++) dz_[(size_t)(k + 1) * (NA + 1) + c] = o[k];
  }

  /* V_dustKernel_IDIC (IDIC.h:264-284) */
  for (int s = 1; s < ns; s++) {
    orc_species *q = &sp[s];
    for (int i = 0; i < q->n; i++) {
      if (q->ind[i] != 0) continue;
      int c = ckey[s][i];
      if (c < 0) continue;
      double ts = t_av[(size_t)s * (NA + 1) + c];
      q->vx[i] = (q->vx[i] / tau + gx[c] / ts) / (1.0 / tau + 1.0 / ts);
      q->vy[i] = (q->vy[i] / tau + gy[c] / ts) / (1.0 / tau + 1.0 / ts);
      q->vz[i] = (q->vz[i] / tau + gz[c] / ts) / (1.0 / tau + 1.0 / ts);
    }
  }
  /* V_gasKernel_IDIC (IDIC.h:287-315) */
  const int own_acc = (P->flags & ORC_GAS_ACCEL_PARTICLE) != 0;
  for (int i = 0; i < Ng; i++) {
    if (gas->ind[i] != 0) continue;
    int c = ckey[0][i];
    if (c < 0) continue;
    double tmp1 = 0.0, tmp_x = 0.0, tmp_y = 0.0, tmp_z = 0.0;
    for (int k = 1; k <= nd; k++) {
      size_t q = (size_t)k * (NA + 1) + c;
      tmp1 = tmp1 + eps_c[q] / t_av[q];
    }
    for (int k = 1; k <= nd; k++) {
      size_t q = (size_t)k * (NA + 1) + c;
      tmp_x = tmp_x + eps_c[q] * dx_[q] / t_av[q];
    }
    for (int k = 1; k <= nd; k++) {
      size_t q = (size_t)k * (NA + 1) + c;
      tmp_y = tmp_y + eps_c[q] * dy_[q] / t_av[q];
    }
    for (int k = 1; k <= nd; k++) {
      size_t q = (size_t)k * (NA + 1) + c;
      tmp_z = tmp_z + eps_c[q] * dz_[q] / t_av[q];
    }
    double ax = own_acc ? gas->ax[i] : psx[c];
    double ay = own_acc ? gas->ay[i] : psy[c];
    double az = own_acc ? gas->az[i] : psz[c];
    gas->vx[i] = (gas->vx[i] / tau + tmp_x + ax) / (1.0 / tau + tmp1);
    gas->vy[i] = (gas->vy[i] / tau + tmp_y + ay) / (1.0 / tau + tmp1);
    gas->vz[i] = (gas->vz[i] / tau + tmp_z + az) / (1.0 / tau + tmp1);
  }

  /* MoveKernel_IDIC x3 (IDIC.h:319-333), periodic wrap as an extension */
  for (int s = 0; s < ns; s++) {
    orc_species *q = &sp[s];
    for (int i = 0; i < q->n; i++) {
      if (q->ind[i] != 0) continue;
      q->x[i] = q->x[i] + q->vx[i] * tau;
      q->y[i] = q->y[i] + q->vy[i] * tau;
      q->z[i] = q->z[i] + q->vz[i] * tau;
      if (G.per_y) {
        if (q->y[i] < P->Y_min) q->y[i] = q->y[i] + G.Ly;
        else if (q->y[i] >= P->Y_max) q->y[i] = q->y[i] - G.Ly;
      }
      if (G.per_z) {
        if (q->z[i] < P->Z_min) q->z[i] = q->z[i] + G.Lz;
        else if (q->z[i] >= P->Z_max) q->z[i] = q->z[i] - G.Lz;
      }
    }
  }
  /* EnergyKernel_IDIC (IDIC.h:335-346) */
  for (int i = 0; i < Ng; i++)
    if (gas->ind[i] == 0) gas->e[i] = gas->e[i] + e_temp[i] * tau;

  *Tm = *Tm + tau;
  if (dt_taken) *dt_taken = tau;

  free(e_temp); free(gx); free(gy); free(gz); free(dx_); free(dy_); free(dz_);
  free(cnt); free(vx_av); free(vy_av); free(vz_av); free(t_av); free(eps_c);
  free(psx); free(psy); free(psz);
  for (int s = 0; s < ns; s++) { free(head[s]); free(next[s]); free(ckey[s]); }
  return status;
}

int orc_step(const orc_params *P, orc_species *sp, double *Tm, double *dt_taken) {
  double dtmin = INFINITY;
  int status = orc_step_density(P, sp, &dtmin);
  if (status < 0) return status;
  return status | orc_step_complete(P, sp, Tm, dtmin, dt_taken);
}

/* ------------------------------------------------------------------------ */
/* Parity hooks                                                               */
/* ------------------------------------------------------------------------ */

int orc_build_list(const orc_params *P, const orc_species *s, int *head, int *next) {
  orc_grid G;
  orc_grid_setup(P, &G);
  int *tail = (int *)malloc(sizeof(int) * (G.ncells + 1));
  orc_list(&G, s, head, next, tail);
  free(tail);
  return G.ncells;
}

void orc_cell_keys(const orc_params *P, const orc_species *s, int *key) {
  orc_grid G;
  orc_grid_setup(P, &G);
  for (int p = 0; p < s->n; p++) key[p] = orc_key(&G, s->x[p], s->y[p], s->z[p]);
}

void orc_idic_keys(const orc_params *P, const orc_species *s, int *key) {
  orc_grid G;
  orc_grid_setup(P, &G);
  for (int p = 0; p < s->n; p++) key[p] = orc_idic_key(&G, s->x[p], s->y[p], s->z[p]);
}

void orc_neighbour_counts(const orc_params *P, const orc_species *s, int *ncand, int *nnb) {
  orc_grid G;
  orc_grid_setup(P, &G);
  const int hpp = (P->flags & ORC_H_PER_PARTICLE) != 0;
  const int R = P->stencil == 2 ? 2 : 1;
  int *head = (int *)malloc(sizeof(int) * (G.ncells + 1));
  int *next = (int *)malloc(sizeof(int) * (s->n > 0 ? s->n : 1));
  int *tail = (int *)malloc(sizeof(int) * (G.ncells + 1));
  orc_list(&G, s, head, next, tail);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s->n; i++) {
    orc_stencil st;
    orc_make_stencil(&G, R, s->x[i], s->y[i], s->z[i], &st);
    const double hi = hpp ? s->h[i] : P->h;
    int nc = 0, nn = 0;
    for (int o = 0; o < st.n; o++) {
      if (st.cell[o] < 0) continue;
      for (int j = head[st.cell[o]]; j > -1; j = next[j]) {
        nc++;
        double dx = orc_diff(s->x[j], st.sx[o], s->x[i]);
        double dy = orc_diff(s->y[j], st.sy[o], s->y[i]);
        double dz = orc_diff(s->z[j], st.sz[o], s->z[i]);
        double dist = sqrt(dx * dx + dy * dy + dz * dz);
        double hj = hpp ? s->h[j] : hi;
        double hcut = hpp ? (hi > hj ? hi : hj) : hi;
        if ((dist < 2 * hcut) && (dist > 0)) nn++;
      }
    }
    ncand[i] = nc;
    nnb[i] = nn;
  }
  free(head); free(next); free(tail);
}

double orc_kernel_W(double r, double h) { return orc_W(r, h); }
double orc_kernel_dW(double r, double h) { return orc_dW(r, h); }

void orc_grid_info(const orc_params *P, int *out) {
  orc_grid G;
  orc_grid_setup(P, &G);
  out[0] = G.Cnx; out[1] = G.Cny; out[2] = G.Cnz; out[3] = G.ncells;
  out[4] = G.Nax; out[5] = G.Nay; out[6] = G.Naz; out[7] = G.n_idic;
}
