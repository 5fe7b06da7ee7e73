/*
 * dustyshock3d_gb300.h -- C ABI of the GB300 (sm_103a) per-step dusty-gas
 * SPH + IDIC solver.
 *
 * Drop-in for the inline step loop of the reference program
 * (kernel.cu:1929-2523 with the IDIC.h kernels).  The reference's host driver
 * keeps its config parser (kernel.cu:1705-1742), initial conditions
 * (kernel.cu:1391) and snapshot output (kernel.cu:2528-2564); in between it
 * uploads its SoA FP64 arrays once (data.h:19-20, 49-55), calls ds_step for
 * the time loop and downloads at output times.  Nothing here includes data.h
 * (it defines globals).
 *
 * Conventions
 *  - every call returns a ds_status; nothing aborts, traps or exits;
 *  - host arrays are caller-owned and are read or written only during the
 *    call; device memory is owned by the context;
 *  - particle arrays are in the caller's index order (index p = 0..n-1, the
 *    reference's 0..Pm); the library sorts internally and restores the order
 *    on download;
 *  - one context per host thread; a context uses the current CUDA device at
 *    ds_create time and its own stream.
 */
#ifndef DUSTYSHOCK3D_GB300_H
#define DUSTYSHOCK3D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define DS_MAX_DUST 4
#define DS_NPHASE 4 /* timed phases per step, see ds_phase_times */

typedef enum ds_status {
  DS_OK = 0,
  DS_ERR_ARG = 1,      /* invalid argument (null pointer, bad size, bad species) */
  DS_ERR_CUDA = 2,     /* a CUDA runtime call failed; see ds_last_error          */
  DS_ERR_STATE = 3,    /* call out of order (e.g. step before particles are set) */
  DS_ERR_NOMEM = 4,    /* device allocation failed                                */
  DS_ERR_DEVICE = 5,   /* a kernel raised a sticky device-side flag               */
  DS_ERR_UNSUPPORTED = 6,
  DS_ERR_IO = 7        /* checkpoint file missing, unreadable or malformed         */
} ds_status;

/* Device-side flags (sticky per context, read with ds_last_error). */
#define DS_FLAG_IDIC_RANGE 0x1 /* a particle's IDIC cell index was outside the grid
                                  (the reference writes out of bounds there,
                                  kernel.cu:2116-2117); it was left unrelaxed   */
#define DS_FLAG_PID_RANGE 0x2  /* dust index beyond the gas count in the index-
                                  coupled stopping time (IDIC.h:86)             */
#define DS_FLAG_NONFINITE 0x4  /* a particle's velocity, position or energy became
                                  NaN or infinite in a step.  Reported only: the
                                  step succeeds and goes on, as the reference's
                                  does (its cell key of a NaN position, int(NaN),
                                  is undefined there; here the particle drops out
                                  of the cell lists).  The other flags make
                                  ds_step return DS_ERR_DEVICE.                 */
#define DS_FLAG_REACH 0x8      /* proper cell grid only: a particle's cut-off 2h
                                  reached past the cells the tube's stencil
                                  covers (2h > stencil x the narrowest cell
                                  width), so partners beyond them were missed.
                                  Raise the stencil or the cell width.  (On
                                  the reference grid the fixed 27 cells,
                                  kernel.cu:2014-2016, drop such partners
                                  silently, as the reference does.)            */

/* Mode bits (ds_params.mode).  0 = the reference's own step. */
#define DS_MODE_PERIODIC_Y 0x0001
#define DS_MODE_PERIODIC_Z 0x0002
#define DS_MODE_H_PER_PARTICLE 0x0004  /* h_i per particle; symmetrised gradient  */
#define DS_MODE_TSTOP_CONST 0x0008     /* constant stopping time per species      */
#define DS_MODE_GAS_ACCEL_PARTICLE 0x0010 /* gas relaxes with its own A_i, not Psi */
#define DS_MODE_REF_INDEX_COUPLING 0x0020 /* dust rho zeroed by gas Ind[p] (IDIC.h:8) */
#define DS_MODE_REF_EPS_GUARD 0x0040   /* all eps guards test species-1 count (kernel.cu:2203) */
#define DS_MODE_REF_SOLVE2 0x0080      /* 2-species solve in the reference's order */
#define DS_MODE_CFL 0x0100             /* CFL step instead of fixed tau           */
#define DS_MODE_DUST_RHO 0x0200        /* dust self-density every step            */
#define DS_MODE_GRID_PROPER 0x0400     /* cell key stride nx (reference: Cnx)     */
#define DS_MODE_IDIC_PROPER 0x0800     /* IDIC key stride nx (reference: Nax)     */
#define DS_MODE_REFERENCE (DS_MODE_REF_INDEX_COUPLING | DS_MODE_REF_EPS_GUARD | \
                           DS_MODE_REF_SOLVE2 | DS_MODE_DUST_RHO)

#define DS_PRECISION_FP64 0 /* FP64 everywhere, reference operation order */
#define DS_PRECISION_FP32 1 /* FP32 neighbour sums (Kahan), cell-relative FP32
                               positions; FP64 state, IDIC exchange, sums.
                               Needs DS_MODE_GRID_PROPER (else
                               DS_ERR_UNSUPPORTED at ds_create)              */

/* Run parameters: Init.txt lines 2-18 (kernel.cu:1707-1723), the constants the
 * reference hard-codes, and the extensions.  Fill with ds_params_init. */
typedef struct ds_params {
  double X_min, X_max, Y_min, Y_max, Z_min, Z_max; /* Init.txt 2-7              */
  int Type_of_state;                               /* Init.txt 8 (0: p=rho e(g-1), 1: c^2 rho) */
  int Maximum_particle;                            /* Init.txt 9                */
  double Particle_on_length;                       /* Init.txt 10 (IC only)     */
  double h;                                        /* Init.txt 11               */
  double Coeff_h_dust_cell;                        /* Init.txt 12               */
  double tau, T_end, T_out;                        /* Init.txt 13-15            */
  double alpha, beta, eps;                         /* Init.txt 16-18            */
  double Gam_g;              /* data.h:7, 1.4                                    */
  double Speed_of_sound_gas; /* kernel.cu:1744, 1.0                              */
  int n_dust;                /* dust species, 1..DS_MAX_DUST (reference: 2)      */
  int mode;                  /* DS_MODE_* bits                                   */
  int precision;             /* DS_PRECISION_*                                   */
  int stencil;               /* cells searched on each side at most: 0 or 1 -> 27 cells of
                                width >= 2h (the reference); 2 -> up to 125 cells of width
                                >= h_max (DS_MODE_GRID_PROPER), each particle walking only
                                the cells its cut-off reaches; 3 or 4 (fp32 path only) ->
                                smaller cells, up to 9 x 9 rows of 9 cells             */
  double cell_w;             /* neighbour cell width; 0 -> 2h (kernel.cu:1773)   */
  double idic_w;             /* IDIC cell width; 0 -> Coeff_h_dust_cell*h (kernel.cu:1577) */
  double cfl;                /* CFL number (DS_MODE_CFL)                          */
  double t_empty;            /* mean t_stop of a cell without dust (kernel.cu:2160) */
  int list_depth;             /* FP32 sweeps: candidate-list entries per thread, 32 or 64
                                (0 -> 32); an autotuner choice                         */
  int force_list;            /* FP32 path: neighbour entries per gas particle that the
                                density sweep records for the force sweep, which then
                                reads them instead of walking the cells again (0 -> 256,
                                or 512 with a list_skin; -1 -> off); a warp holding a
                                particle with more neighbours walks.  Results are the same
                                either way. */
  double mass_ratio[DS_MAX_DUST];   /* mas_gas_dust_k (kernel.cu:1499-1502)       */
  double R_dust[DS_MAX_DUST];       /* R_dust_k for t_stop = R/(c_s rho) (IDIC.h:86) */
  double t_stop_const[DS_MAX_DUST]; /* DS_MODE_TSTOP_CONST                        */
  double eps_empty[DS_MAX_DUST];    /* eps of a cell failing its guard (kernel.cu:2200, 2209) */
  double list_skin;          /* FP32 path with force lists: reuse of the recorded neighbour
                                lists across steps (0 -> off: every step sorts, walks and
                                records).  The density sweep records the pairs within
                                2 max(h_i, h_j) + list_skin x h; later steps stream those
                                lists (density and force, each pair tested against its exact
                                cut-off) and skip the sort and the cell walk, until the
                                tube's particles have moved far enough, relative to each
                                other, that a pair outside the lists could be within its
                                cut-off.  That test runs on the device at the start of every
                                step, per tube, from the displacements since the lists were
                                recorded: per neighbour cell their mean and largest deviation
                                from it; a tube re-sorts when, for two cells within one cell
                                beyond the recording walk's reach, the two deviations plus
                                the difference of the means reach the skin, or when twice
                                the largest deviation plus the spread of all cell means
                                reaches the skin plus a cell width.  Neighbour cells are
                                widened so that the recorded cut-off stays within the
                                stencil.  Ignored (off) on the FP64 path, without force
                                lists, and with DS_MODE_DUST_RHO. */
  int persistent;            /* FP32 path: 1 -> the neighbour sweeps run on a persistent grid
                                (as many 128-thread blocks as fit on the GPU at once), each
                                block claiming its next chunk of particles from a counter;
                                0 -> one block per chunk.  An autotuner choice (batch-wide:
                                tube 0's); results are the same either way. */
  int idic_lanes;            /* FP32 path: threads per IDIC cell in its cell sums, 2, 4 or 8
                                (0 -> 4); an autotuner choice (batch-wide: tube 0's); each
                                lane sums a contiguous part in order, so a tube's result
                                depends on it but not on its batch. */
} ds_params;

typedef struct ds_ctx ds_ctx;

/* Fills p with the reference's Init.txt values and constants (DS_MODE_REFERENCE). */
ds_status ds_params_init(ds_params *p);

/* Parses an Init.txt the way the reference's main does (kernel.cu:1705-1723):
 * title line, then 17 positional values, trailing comments ignored.  Lines
 * after those (the reference never reads them) may set the extensions as
 * "name = value", "//" starting a comment: any ds_params field by name
 * (mass_ratio, R_dust, t_stop_const, eps_empty take up to DS_MAX_DUST values
 * separated by spaces or commas; precision = fp32 | fp64), and "mode.<name> =
 * 0 | 1" for each DS_MODE_* bit (mode.periodic_y, mode.h_per_particle, ...,
 * mode.idic_proper).  "ic" lines belong to ds_ic_read_init_txt.  An unknown
 * name or a malformed value is DS_ERR_ARG.  p keeps its values for fields the
 * file does not set (start from ds_params_init). */
ds_status ds_params_read_init_txt(const char *path, ds_params *p);

/* Initial conditions generated on the device.  The reference's host driver
 * fills its arrays with a generator before the upload (kernel.cu:1391); here
 * the particles are generated straight into a tube's device state, so a run,
 * or a served request, needs no host particle arrays.  Particles come out in
 * the generators' own order and equal the host generators bit for bit.
 *
 *  DS_IC_SOD_X_DUST  init_Sod_X_Dust (kernel.cu:1391-1582), the generator the
 *                    reference's main calls, from the Init.txt parameters:
 *                    gas on two lattices of spacing (m / rho)^(1/3) (rho 1 | 1,
 *                    e 2.5 | 2.0; m = 1 / Particle_on_length^3) accepted in
 *                    |x| <= 1, |y|, |z| <= 0.8; two dust species on the gas
 *                    sites (mass ratios 0.75, 0.5; R_dust 0.01, 1.0; t_stop
 *                    from the gas p and rho, kernel.cu:43-46); sets n_dust 2,
 *                    Coeff_h_dust_cell 0.5 and DS_MODE_REFERENCE.  Kept quirks:
 *                    the interior (Ind = 0) test compares |y| with the x cube
 *                    (kernel.cu:1441, 1481), and every lattice point, accepted
 *                    or not, writes the Ind of the last accepted particle
 *                    (kernel.cu:1441-1448).
 *  DS_IC_SOD_X_MAS   the equal-mass lattices of init_Sod_X_mas (kernel.cu:938-
 *                    1042: p 1 | 0.1, e 2.5 | 2.0, rho from Eq_State1, cube
 *                    |x|, |y|, |z| <= 1), with the parameters' n_dust species
 *                    of dust on the gas sites as init_Sod_X_Dust places them
 *                    (kernel.cu:1505-1548, mass_ratio and R_dust of ds_params).
 *  DS_IC_DUSTY_SOD   the dusty Sod shock tube (no reference counterpart): the
 *                    ds_ic fields below.
 * A rejected first lattice point (the reference then writes Ind_gas[-1]) and
 * more gas particles than Maximum_particle (kernel.cu:1751) are DS_ERR_ARG. */
#define DS_IC_SOD_X_DUST 1
#define DS_IC_SOD_X_MAS 2
#define DS_IC_DUSTY_SOD 3

typedef struct ds_ic {
  int kind;      /* DS_IC_*                                                        */
  int reserved;
  /* DS_IC_DUSTY_SOD: tube [x0, x1] x [0, Ly] x [0, Lz], periodic in y and z.  The
     left state sits on a cubic lattice of spacing dx_left; the right lattice has
     round(Ly / (dx_left (rho_L / rho_R)^(1/3))) sites across and the same particle
     mass; h = h_factor x local spacing; gas sites at (i + lattice_offset) spacings
     from the lower faces, one dust particle per gas site half a spacing further
     (mass eps x the gas mass, constant stopping time t_s); particles within `wall`
     smoothing lengths of an x end frozen (Ind 1).  The run parameters: periodic
     y/z, per-particle h, CFL number cfl (or fixed_tau > 0), IDIC cells of
     idic_cells right-lattice spacings, neighbour cells of 1.001 h_max, stencil 2,
     FP64 (set precision and the like on the planned ds_params). */
  double dx_left, Ly, Lz; /* Lz <= 0 -> Ly                                          */
  double eps, t_s;
  double rho_L, p_L, rho_R, p_R, gamma;
  double h_factor;
  double x0, x1, wall, lattice_offset;
  double t_end, cfl, alpha, beta, av_eps;
  double idic_cells;
  double fixed_tau;
} ds_ic;

/* Defaults of a kind (DS_IC_DUSTY_SOD: Sod states 1, 1 | 0.125, 0.1; eps 1;
 * t_s 1e-3; gamma 1.4; h_factor 1.3; x in [-0.5, 0.5]; wall 2.5; offset 0.25;
 * t_end 0.2; cfl 0.3; alpha 1, beta 2, av_eps 0.01; idic_cells 2; dx_left and Ly
 * left 0 for the caller). */
ds_status ds_ic_init(ds_ic *ic, int kind);

/* "ic = sod_x_dust | sod_x_mas | dusty_sod" and "ic.<field> = value" extension
 * lines of an Init.txt (no "ic" line: DS_IC_SOD_X_DUST, as the reference). */
ds_status ds_ic_read_init_txt(const char *path, ds_ic *ic);

/* Host-side plan, no device work: the run parameters to create the context
 * with (out; precision, stencil, force_list and the like may be changed before
 * ds_create) and the particles per species (counts[1 + out->n_dust], gas
 * first).  init: the Init.txt parameters the reference generators read (box,
 * h, Particle_on_length, Type_of_state, Maximum_particle; for DS_IC_SOD_X_MAS
 * also n_dust, mass_ratio, R_dust); may be NULL for DS_IC_DUSTY_SOD. */
ds_status ds_ic_plan(const ds_ic *ic, const ds_params *init, ds_params *out, int *counts);

/* Generates tube `tube`'s particles on the device, in place of ds_set_gas /
 * ds_set_dust before the first step, or into a resident tube with the same
 * particle counts (the clock is kept).  The tube's own parameters are the
 * generator's init. */
ds_status ds_init_tube(ds_ctx *c, int tube, const ds_ic *ic);

/* One tube (the reference's single domain).  Replaces the reference's device
 * allocation and upload block (kernel.cu:1793-1926). */
ds_status ds_create(const ds_params *p, ds_ctx **out);

/* ntubes independent tubes advanced together (batched launches). */
ds_status ds_create_batch(int ntubes, const ds_params *p, ds_ctx **out);

/* Gas arrays of one tube, reference layout (data.h:19-20).  h may be NULL
 * (then h = params.h for every particle); ax, ay, az may be NULL (zero). */
ds_status ds_set_gas(ds_ctx *c, int tube, int n, const double *x, const double *y, const double *z,
                     const double *vx, const double *vy, const double *vz, const double *ax,
                     const double *ay, const double *az, const double *rho, const double *p,
                     const double *e, const double *mas, const double *h, const int *ind);

/* Dust species k (1..n_dust) of one tube, reference layout (data.h:49-55). */
ds_status ds_set_dust(ds_ctx *c, int tube, int species, int n, const double *x, const double *y,
                      const double *z, const double *vx, const double *vy, const double *vz,
                      const double *rho, const double *mas, const double *t_stop, const double *h,
                      const int *ind);

/* Carries tube src_tube of src's resident state (particles in their current
 * order, simulation time and step count) into tube dst_tube of dst, which must
 * not have stepped yet; the copy is device to device, made when dst is first
 * stepped, so src must stay alive until then.  Particle counts per species are
 * src's; parameters are dst's.  A batch is rebuilt this way when tubes join or
 * leave it (continuous batching), without the state leaving the GPU. */
ds_status ds_copy_tube(ds_ctx *dst, int dst_tube, ds_ctx *src, int src_tube);

/* Host buffers: pageable arrays go through the copy engines.  Pinned, mapped
 * ones (ds_host_alloc, cudaMallocHost) are read and written in place by
 * kernels over NVLink-C2C, in one pass per species: faster.  A resident upload
 * from pinned buffers reads them asynchronously, so keep them unchanged until
 * the next ds_step / ds_synchronize.  Downloads return when the data is in
 * host memory either way. */

/* Single-tube names the reference's host driver binds (tube 0). */
ds_status ds_upload_gas(ds_ctx *c, int n, const double *x, const double *y, const double *z,
                        const double *vx, const double *vy, const double *vz, const double *ax,
                        const double *ay, const double *az, const double *rho, const double *p,
                        const double *e, const double *mas, const double *h, const int *ind);
ds_status ds_upload_dust(ds_ctx *c, int species, int n, const double *x, const double *y,
                         const double *z, const double *vx, const double *vy, const double *vz,
                         const double *rho, const double *mas, const double *t_stop,
                         const double *h, const int *ind);

/* Advances every tube whose time is below its T_end by up to nsteps steps
 * (the body of the reference's do-while loop, kernel.cu:1929-2566).  State
 * stays on the device; returns after the device has finished. */
ds_status ds_step(ds_ctx *c, int nsteps);

/* Same, without waiting for the device (errors surface at the next sync). */
ds_status ds_step_async(ds_ctx *c, int nsteps);
ds_status ds_synchronize(ds_ctx *c);

/* Host arrays as the state of record, the way the reference's host keeps its
 * data.h arrays between steps and copies them to and from the GPU inside the
 * step (53 blocking cudaMemcpy calls in the step body, kernel.cu:1929-2527,
 * e.g. 2026-2027, 2268-2270, 2476-2482).  ds_bind_host binds caller-owned pinned arrays
 * (ds_host_alloc, cudaMallocHost, or cudaHostRegister'ed) to one species of
 * one tube: fields[0..14] = x, y, z, vx, vy, vz, ax, ay, az, rho, p, e, mas,
 * h, t_stop as in ds_get_fields, n = the species' particle count, ind its Ind.
 * ds_step_host then runs nsteps steps; each reads every bound array (the
 * caller may change them between calls) and writes back what the step can
 * change -- gas x..e (12 fields); dust x, y, z, vx, vy, vz, rho (with
 * DS_MODE_DUST_RHO) and t_stop (without DS_MODE_TSTOP_CONST) -- in the
 * caller's index order.  NULL entries are neither read nor written
 * (the resident values stay), and species left unbound stay resident.  Inside
 * a step the reads of the fields other than x, y, z overlap the cell sort,
 * and rho, p go back during the force sweep, ax, ay, az, t_stop during the
 * IDIC phase (kernels over NVLink-C2C on a second stream, all in one CUDA
 * graph).  Returns when the last step's results are in host memory.  Without
 * list reuse, results equal ds_upload_* + ds_step(1) + ds_download_* per
 * step, bit for bit (an upload re-sorts every tube).  With list reuse
 * (list_skin > 0, FP32 path) a step reads h, the masses and Ind with the
 * positions, and the start-of-step test measures the host's positions against
 * the recorded ones: a tube keeps its lists and slot order as a step on the
 * resident state would (its density sums start before the other fields have
 * arrived), so steps on unchanged host arrays equal ds_step(1) per step bit
 * for bit; a host edit of any particle's h or Ind makes its tube re-sort and
 * record.
 * fields == NULL unbinds the species.  ds_step / ds_get_* keep working on the
 * resident state in between. */
ds_status ds_bind_host(ds_ctx *c, int tube, int species, int n, double *const *fields, int *ind);
ds_status ds_step_host(ds_ctx *c, int nsteps);

/* Downloads in the caller's index order; any pointer may be NULL (skipped).
 * Before the first step they return the particles as set (or generated). */
ds_status ds_get_gas(ds_ctx *c, int tube, double *x, double *y, double *z, double *vx, double *vy,
                     double *vz, double *ax, double *ay, double *az, double *rho, double *p,
                     double *e, int *ind);
ds_status ds_get_dust(ds_ctx *c, int tube, int species, double *x, double *y, double *z, double *vx,
                      double *vy, double *vz, double *rho, double *t_stop, int *ind);
ds_status ds_download_gas(ds_ctx *c, double *x, double *y, double *z, double *vx, double *vy,
                          double *vz, double *ax, double *ay, double *az, double *rho, double *p,
                          double *e, int *ind);
ds_status ds_download_dust(ds_ctx *c, int species, double *x, double *y, double *z, double *vx,
                           double *vy, double *vz, double *rho, double *t_stop, int *ind);

/* Simulation time Tm, last step size and steps taken of one tube. */
ds_status ds_get_time(ds_ctx *c, int tube, double *Tm, double *dt_last, long long *nsteps);

/* Parity hook: for the particles' CURRENT positions, the raw cell key of each
 * particle (kernel.cu:1949), the reference's linked lists (head[ncells+1] =
 * Cell_*, next[n] = Nn_*, kernel.cu:1937-1955) reconstructed from the sorted
 * order, and per particle the candidates visited over the 27 offsets and the
 * number with 0 < r < 2h (IDIC.h:219-220), from the production sweep.  Any
 * pointer may be NULL.  *ncells receives Number_of_fihd_cells. */
ds_status ds_debug_cells(ds_ctx *c, int tube, int species, int *cell_key, int *head, int *next,
                         int *ncand, int *nnb, int *ncells);

/* Parity hook: the IDIC cell arrays of one species as left by the last step
 * (cells 0..Number_of_average_cell, kernel.cu:2060-2437): count[n] and
 * cells[12][n] = sums of Vx, Vy, Vz; sums of Ax, Ay, Az (gas) or of t_stop
 * (dust, first row); solved Vx, Vy, Vz; Psi x, y, z (gas) or mean t_stop and
 * eps (dust).  *ncells receives n.  Any pointer may be NULL. */
ds_status ds_debug_idic(ds_ctx *c, int tube, int species, int *count, double *cells, int *ncells);

/* The cell lists of one species as the last step built them, before it moved
 * the particles: what the reference's snapshot writer prints as Nn
 * (kernel.cu:261, 463; its lists are built at the top of the step,
 * kernel.cu:1937-1995).  Same layout as ds_debug_cells; no re-sort.  On the FP32
 * path a cell lists its particles in the path's own slot order. */
ds_status ds_step_lists(ds_ctx *c, int tube, int species, int *head, int *next, int *ncells);

/* Every field of one species in caller order: fields[0..14] receive x, y, z,
 * vx, vy, vz, ax, ay, az, rho, p, e, mas, h, t_stop (NULL entries skipped). */
ds_status ds_get_fields(ds_ctx *c, int tube, int species, double *const *fields, int *ind);

/* Global FP64 sums of one tube: out[0] mass, out[1..3] momentum, out[4] gas
 * internal energy sum m e, out[5] kinetic energy (all species). */
ds_status ds_conservation(ds_ctx *c, int tube, double *out6);

/* Dust self-density of every tube at the current positions (kernel.cu:2029-2043),
 * computed on demand: the reference computes it every step but only its snapshot
 * writer reads it (kernel.cu:2547-2562), so a host that writes snapshots calls
 * this before ds_get_dust / ds_download_dust at output times instead of paying
 * for it every step (DS_MODE_DUST_RHO).  Same sums as the per-step sweep. */
ds_status ds_dust_density(ds_ctx *c);

/* Binary checkpoint of one tube.  The reference has none: its text snapshots
 * print 8 decimals and cannot restart a run (kernel.cu:261).  The file holds the
 * tube's ds_params, its clock (Tm, last dt, step count) and every particle field
 * in caller order.  ds_checkpoint_params reads the parameters back, so a host can
 * create a matching context; ds_load_tube restores particles and clock, before
 * the first step or into a resident tube with the same particle counts.  On the
 * FP64 path the resumed run equals the uninterrupted one bit for bit. */
ds_status ds_save_tube(ds_ctx *c, int tube, const char *path);
ds_status ds_checkpoint_params(const char *path, ds_params *p);
ds_status ds_load_tube(ds_ctx *c, int tube, const char *path);

/* Runs nsteps steps back to back (the graph's kernels, launched one by one)
 * with CUDA events between phases on the context's stream; returns the total
 * device time and the per-phase sums in milliseconds: [0] keys, sort, reorder,
 * cell ranges, IDIC-key sort; [1] density sweeps with the EOS (and, on the
 * FP32 path, the force neighbour lists); [2] t_stop, step size, force sweep;
 * [3] IDIC reduce + solve, relax, move, energy.  phase_ms may be NULL: then
 * the steps are the captured graphs ds_step replays, between two events, and
 * only the total is returned. */
ds_status ds_step_timed(ds_ctx *c, int nsteps, float *total_ms, float *phase_ms);

/* Number of kernels one step launches (the library's own kernels). */
ds_status ds_kernels_per_step(ds_ctx *c, int *count);

/* List reuse (ds_params.list_skin): steps of the tube that re-sorted and
 * recorded its neighbour lists, and steps taken.  No counterpart in the
 * reference, which rebuilds its lists every step (kernel.cu:1937-1995). */
ds_status ds_list_stats(ds_ctx *c, int tube, long long *rebuilds, long long *steps);

/* Parity hook (FP32 path with force lists): the neighbour lists the density
 * sweep last recorded for the tube's gas, by caller index.  count[i] = the
 * entries of particle i (-1: its warp walks the cells instead, an entry beyond
 * the lists' capacity), nbr[i * cap + k] = the caller index of its k-th entry,
 * k < min(count[i], cap).  Tests use it to check that reused lists still hold
 * every pair within the cut-off.  No counterpart in the reference, whose
 * linked cell lists (kernel.cu:1937-1995) are walked afresh every step. */
ds_status ds_debug_force_lists(ds_ctx *c, int tube, int cap, int *count, int *nbr);

/* Split step, for one tube cut into x-slabs across processes (the host layer
 * in dustyshock3d_gb300/slab.py).  A slab's context holds its own particles
 * and frozen copies (Ind != 0) of the other slabs' gas within 2 h_max of its
 * boundaries ("ghosts").  One step is
 *   ds_step_density   the sort, the gas density and the EOS (and the dust
 *                     density); the ghosts' own densities are not computed;
 *   ds_get_cfl_min    the slab's CFL candidate min h / (c_s + |v|) over its
 *                     updated gas (+inf without CFL);
 *   ds_set_cfl_min    the minimum over all slabs (an allreduce(min) on the host);
 *   ds_set_gas_hydro  the ghosts' density and pressure as their owners computed
 *                     them (idx: caller indices of gas particles of the tube);
 *   ds_step_complete  t_stop, the step size, the force, the IDIC cell solve,
 *                     the update and the clock.
 * The reference runs one domain on one device (kernel.cu:1793); its step
 * (kernel.cu:1937-2566) is split after the density and EOS (kernel.cu:2011-2024)
 * so the ghosts' pressure can arrive before the force (kernel.cu:2233-2266).
 * Each call synchronises the context's stream. */
ds_status ds_step_density(ds_ctx *c);
ds_status ds_get_cfl_min(ds_ctx *c, int tube, double *dtmin);
ds_status ds_set_cfl_min(ds_ctx *c, int tube, double dtmin);
ds_status ds_set_gas_hydro(ds_ctx *c, int tube, int n, const int *idx, const double *rho, const double *p);
ds_status ds_step_complete(ds_ctx *c);

/* Set a tube's clock (time and steps taken), e.g. when a slab's state moves to
 * a larger context.  The reference keeps Tm in its time loop (kernel.cu:1929). */
ds_status ds_set_time(ds_ctx *c, int tube, double Tm, long long nsteps);

/* Host-side: the IDIC cell column (x index) of each position, computed as the
 * step computes it for the parameters' precision (FP64: the division of
 * kernel.cu:2116 with the proper grid's floor; FP32: one FMA with the
 * reciprocal width).  Slab boundaries fall on these columns, so every IDIC
 * cell's particles live in one slab. */
ds_status ds_idic_columns(const ds_params *p, int n, const double *x, int *col);

/* Device bytes held by the context, and particles per tube. */
ds_status ds_memory_bytes(ds_ctx *c, long long *bytes);

/* Sticky device flags (DS_FLAG_*) and the last error text. */
ds_status ds_last_error(ds_ctx *c, int *device_flags, char *msg, int msglen);

/* Allocation-free cell lists.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc (a host that hands all device
 * memory to its own pool allocator, or code that runs where an allocation
 * would be an error or would stall the device): builds, for n particles whose
 * positions are already in device memory, the raw cell key of each particle
 * (kernel.cu:1949) and the reference's linked lists -- head[c] = first
 * particle of cell c, next[p] = the following particle of p's cell in
 * ascending index, -1 at the end (kernel.cu:1937-1955) -- exactly as
 * ds_debug_cells reports them, without allocating anything.  The sort's
 * scratch is a static device array inside the library sized for
 * DS_NOALLOC_MAX_PARTICLES particles (about 4.7 MB per GPU that loads the
 * library, held until the process exits); larger n returns DS_ERR_ARG.
 * Inputs and outputs are caller-owned device arrays: d_cell_key[n],
 * d_next[n], d_head[head_len] with head_len >= Number_of_fihd_cells + 1.
 * The grid comes from p (cell width, box, DS_MODE_GRID_PROPER/PERIODIC_*).
 * Work is enqueued on `stream` (a cudaStream_t, NULL for the default stream)
 * and the call returns without waiting.  The first call on each device (and
 * the first after a cudaDeviceReset) loads the library's device code and its
 * static array into that device's context and resolves the array's device
 * address: the load itself takes device memory through the driver, so make
 * that first call before the host's pool takes the memory, and before any
 * stream capture.  Each launch's status is checked on its own; an earlier
 * error of another call on the thread is neither cleared nor reported.  All
 * calls share the one scratch array, so calls whose work overlaps on the GPU
 * race; serialise them. */
#define DS_NOALLOC_MAX_PARTICLES 262144
ds_status ds_cell_lists_noalloc(const ds_params *p, int n, const double *d_x, const double *d_y,
                                const double *d_z, int *d_cell_key, int *d_head, int head_len, int *d_next,
                                void *stream);

/* Pinned host memory for end-to-end copies (cudaMallocHost / cudaFreeHost). */
ds_status ds_host_alloc(void **ptr, long long bytes);
ds_status ds_host_free(void *ptr);

void ds_destroy(ds_ctx *c);

/* Library version string. */
const char *ds_version(void);

#ifdef __cplusplus
}
#endif
#endif
