/*
 * oracle.h -- CPU restatement (FP64, OpenMP) of DustyShock3D's per-step
 * dusty-gas SPH + IDIC hot path, kernel.cu:1929-2523 with the IDIC.h kernels.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference-arm legs may load this library, and only as the
 * checker or as the timed CPU baseline; the product never calls it.
 *
 * Two families of behaviour live behind flags:
 *   - reference mode (flags 0 plus ORC_REF_*): the reference's own step, in
 *     its own loop and summation order, with its quirks (aliasing cell stride,
 *     index-coupled stopping time, empty-cell defaults, two-species solve);
 *   - extensions the reference cannot express (periodic y/z, per-particle h,
 *     constant stopping time, per-particle gas acceleration, CFL step,
 *     general species count).  With every extension flag off the step is the
 *     reference's step.
 */
#ifndef DS_ORACLE_H
#define DS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_DUST 4

/* flag bits */
#define ORC_PERIODIC_Y 0x0001         /* periodic y with image shift            */
#define ORC_PERIODIC_Z 0x0002         /* periodic z with image shift            */
#define ORC_H_PER_PARTICLE 0x0004     /* h_i per particle, symmetrised gradient */
#define ORC_TSTOP_CONST 0x0008        /* t_stop = t_stop_const[k] (no kernel)   */
#define ORC_GAS_ACCEL_PARTICLE 0x0010 /* gas relax uses A_i, not the cell Psi   */
#define ORC_REF_INDEX_COUPLING 0x0020 /* dust rho zeroed by gas Ind; t_stop from gas at same index */
#define ORC_REF_EPS_GUARD 0x0040      /* every species' eps guard tests count of species 1 */
#define ORC_REF_SOLVE2 0x0080         /* two-species solve in the reference's operation order */
#define ORC_CFL 0x0100                /* dt from CFL instead of fixed tau       */
#define ORC_DUST_RHO 0x0200           /* dust self-density every step           */
#define ORC_GRID_PROPER 0x0400        /* neighbour grid stride nx (not the aliasing Cnx) */
#define ORC_IDIC_PROPER 0x0800        /* IDIC grid stride nx (not the aliasing Nax)      */

typedef struct orc_params {
  double X_min, X_max, Y_min, Y_max, Z_min, Z_max; /* Init.txt lines 2-7 */
  int Type_of_state;                               /* Init.txt line 8 */
  int flags;
  double h;                  /* Init.txt line 11, global smoothing length   */
  double tau;                /* Init.txt line 13, fixed step                */
  double T_end;              /* Init.txt line 14                            */
  double alpha, beta, eps;   /* Init.txt lines 16-18                        */
  double Gam_g;              /* data.h:7 (1.4)                              */
  double Speed_of_sound_gas; /* kernel.cu:1744 (1.0)                        */
  double cell_w;             /* neighbour cell width; reference: 2h (kernel.cu:1773) */
  double idic_w;             /* IDIC cell width; reference: 0.5h (kernel.cu:1577)    */
  double cfl;
  double t_empty;            /* empty-cell mean stopping time (kernel.cu:2160)       */
  int n_dust;
  int stencil;               /* cells searched on each side: 1 (27 cells), 2 (125) */
  double mass_ratio[ORC_MAX_DUST];   /* mas_gas_dust_k (kernel.cu:1499-1502) */
  double R_dust[ORC_MAX_DUST];       /* R_dust_k                              */
  double t_stop_const[ORC_MAX_DUST]; /* extension: constant stopping time     */
  double eps_empty[ORC_MAX_DUST];    /* empty-cell eps (kernel.cu:2200, 2209) */
} orc_params;

typedef struct orc_species {
  int n;
  int pad_;
  double *x, *y, *z, *vx, *vy, *vz;
  double *ax, *ay, *az; /* gas only (may be NULL for dust) */
  double *rho, *p, *e;  /* p, e gas only                   */
  double *m, *h, *ts;   /* h: per particle (flag), ts: dust only */
  int *ind;
} orc_species;

/* One time step of every species (sp[0] gas, sp[1..n_dust] dust).
 * *Tm is advanced by the step actually taken (returned in *dt_taken).
 * Returns -1 for a periodic axis too short for the stencil, else the flags
 * of the library's DS_FLAG_* bits that the step raised: 1 IDIC index out of
 * range, 8 a cut-off 2h past the stencil's cells on the proper grid. */
int orc_step(const orc_params *P, orc_species *sp, double *Tm, double *dt_taken);
/* orc_step in two parts (what orc_step runs): the lists, densities and EOS,
 * with the CFL candidate min h / (c_s + |v|) over the updated gas (+inf
 * without CFL); then the rest of the step with the step size taken from
 * dtmin (CFL) or tau.  Between them a caller may overwrite the density and
 * pressure of frozen particles (slab ghosts) and dtmin (a global minimum). */
int orc_step_density(const orc_params *P, orc_species *sp, double *dtmin);
int orc_step_complete(const orc_params *P, orc_species *sp, double *Tm, double dtmin, double *dt_taken);

/* Linked lists of one species exactly as the reference builds them
 * (kernel.cu:1937-1955): head[ncells+1], next[n].  Returns ncells. */
int orc_build_list(const orc_params *P, const orc_species *s, int *head, int *next);

/* Raw (unchecked) neighbour-cell key per particle (kernel.cu:1949). */
void orc_cell_keys(const orc_params *P, const orc_species *s, int *key);

/* Raw IDIC cell index per particle (kernel.cu:2116). */
void orc_idic_keys(const orc_params *P, const orc_species *s, int *key);

/* Per particle: candidates visited over the 27 offsets and how many of them
 * satisfy 0 < r < 2h (the force-sweep test, IDIC.h:219-220). */
void orc_neighbour_counts(const orc_params *P, const orc_species *s, int *ncand, int *nnb);

/* Grid sizes derived from the parameters: out[0..3] = Cnx, Cny, Cnz, ncells;
 * out[4..7] = Nax, Nay, Naz, n_idic_cells. */
void orc_grid_info(const orc_params *P, int *out);

/* The reference's M4 kernel and its derivative (kernel.cu:12-39). */
double orc_kernel_W(double r, double h);
double orc_kernel_dW(double r, double h);

/* IDIC per-cell closed-form solve, exposed for known-answer tests.
 * Inputs per species k: eps[k], t[k], x[k] = v_g - v_k; Psi (one component).
 * Outputs v_g_new and v_k_new.  ref2 selects the reference's two-species
 * operation order (kernel.cu:2310-2437). */
void orc_idic_solve_cell(int n, const double *eps, const double *t, double vg,
                         const double *vd, double psi, double tau, int ref2,
                         double *vg_new, double *vd_new);

#ifdef __cplusplus
}
#endif
#endif
