// ds_kernels.cuh -- launch wrappers of the step kernels (ds_cells.cu,
// ds_sweep64.cu, ds_sweep32.cu).  Every wrapper only enqueues work on the
// given stream, so a whole step can be captured into a CUDA graph.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ds_common.cuh"

#define DS_CHUNK 128  // particles per chunk = threads per block of the per-particle kernels

// Per-key arrays of the IDIC cells (one key per tube, species and cell).
struct CellArrays {
  int *cnt;
  double *vx, *vy, *vz;     // velocity sums
  double *a0, *a1, *a2;     // gas: sums of A; dust: a0 = sum of t_stop
  double *nvx, *nvy, *nvz;  // solved cell velocities
  double *px, *py, *pz;     // gas: Psi; dust: px = mean t_stop, py = eps
  double *q0, *q1;          // FP32 path: relax coefficients (v_new = q0 v + q1 (...))
  int *start;               // first sorted IDIC slot of every key (run bounds)
};

// also zeroes the persistent sweeps' chunk counters (work: DS_NSWEEP ints, or nullptr)
void ds_launch_step_begin(const TubeDesc *tubes, TubeState *ts, int ntubes, int *work, cudaStream_t s);
// fast: FP32 path (reciprocal-multiply cell indices, slot-order scatters);
// otherwise the reference's divisions and caller-index order.
// List reuse (FP32 path): reuse_ts != nullptr gives each tube's decision of the
// step (TubeState::rebuild); a tube keeping its lists keeps its slot order:
// prev_skey, the previous sort's keys, become its keys, and the reorder copies
// it slot for slot.  pos_ref receives the FP32 offsets of re-sorted tubes.
void ds_launch_keys(const TubeDesc *tubes, const Chunk *chunks, int nchunks, DevState st, uint32_t *kin,
                    uint32_t *vin, bool fast, cudaStream_t s, const TubeState *reuse_ts = nullptr,
                    const uint32_t *prev_skey = nullptr, const int *slot_pid = nullptr);
void ds_launch_reorder(const TubeDesc *tubes, const Chunk *chunks, int nchunks, const uint32_t *order,
                       const uint32_t *skey, DevState src, DevState dst, float4 *pos32, float4 *vm32, int *idic_local,
                       uint32_t *ikin, uint32_t *ivin, int *slot_of_pid, int *ind_of_pid, int *flags, bool fast,
                       cudaStream_t s, const TubeState *reuse_ts = nullptr, float4 *pos_ref = nullptr,
                       const int *slot_pid = nullptr, float4 *pm32 = nullptr);
// A bound step with list reuse: pos32 and pm32 of the gas of the tubes that
// keep their lists, from the host's state in caller order (slot q holds
// particle slot_pid[q]), before the reorder.
void ds_launch_early_fp32(const TubeDesc *tubes, const Chunk *gas_chunks, int ngas_chunks, const TubeState *ts,
                          const uint32_t *skey, DevState cs, const int *slot_pid, float4 *pos32, float4 *pm32,
                          cudaStream_t s);
// run_if: skipped when *run_if == 0 (no tube re-sorted this step)
void ds_launch_cell_start(const uint32_t *skey, int n, int nkeys, int *cell_start, cudaStream_t s,
                          const int *run_if = nullptr);
// List reuse: the start-of-step test (displacements, per-cell statistics, the
// bound per tube) and the per-tube decision; *any = some tube re-sorts.
// slot_pid / res (a step on bound host arrays): st is the host's state in
// caller order, slot q of the recorded order holds particle slot_pid[q], res
// is the resident state the lists were recorded on.
void ds_launch_list_test(const TubeDesc *tubes, TubeState *ts, int ntubes, const Chunk *gas_chunks,
                         int ngas_chunks, DevState st, const uint32_t *skey, const float4 *pos_ref, float4 *disp,
                         const int *nseg_key0, const int *nseg_tube, const int *nseg_species, int nseg, int nkeys,
                         const int *cell_start, int xl, const unsigned char *krad, float4 *cellstat, int *force,
                         int *any, cudaStream_t s, const int *slot_pid = nullptr, DevState res = DevState{});
// split step: density and pressure of listed gas particles (caller indices idx;
// val = rho[0..n) then p[0..n)), with the force sweep's per-particle inputs
void ds_launch_set_hydro(const TubeDesc *tubes, int tube, int n, const int *idx, const double *val, const int *inv,
                         DevState st, double *cs64, double *pt64, float4 *hyd32, const float4 *pos32, bool fp32,
                         bool hpp, cudaStream_t s);
// the decision alone (with *force set: every tube re-sorts)
void ds_launch_list_decide(const TubeDesc *tubes, TubeState *ts, int ntubes, int *force, int *any, cudaStream_t s);
void ds_launch_idic_reduce(const uint32_t *ikey, const uint32_t *islot, int n, int nikeys, const int *seg_key0,
                           const int *seg_species, const int *seg_orphan, int nseg, DevState st, CellArrays ca,
                           bool fast, cudaStream_t s, int lanes = 4);
void ds_launch_idic_solve(const TubeDesc *tubes, const TubeState *ts, const int *tube_cell0, int ntubes,
                          int ncell_total, CellArrays ca, bool fast, cudaStream_t s);
void ds_launch_relax_move(const TubeDesc *tubes, const TubeState *ts, const Chunk *chunks, int nchunks,
                          DevState st, const int *idic_local, const double *edot, CellArrays ca, int *flags,
                          bool fast, cudaStream_t s);
void ds_launch_tstop(const TubeDesc *tubes, const TubeState *ts, const Chunk *chunks, int nchunks, DevState st,
                     const int *gas_slot_of_pid, int *flags, cudaStream_t s);
void ds_launch_dt(const TubeDesc *tubes, TubeState *ts, int ntubes, cudaStream_t s);
void ds_launch_step_end(TubeState *ts, int ntubes, cudaStream_t s);
void ds_launch_conservation(const TubeDesc *tubes, int tube, DevState st, double *out, cudaStream_t s);
void ds_launch_debug_lists(const TubeDesc *tubes, int tube, int species, int nseg_particles, int ncells,
                           DevState st, const int *cell_start, int xl, int *head, int *next, int *rawkey,
                           cudaStream_t s);

void ds_launch_cell_radius(const TubeDesc *tubes, const int *cell_start, int nkeys, int xl, const double *h,
                           double *wa, double *wb, const int *nseg_key0, const int *nseg_tube,
                           const int *nseg_species, int nseg, unsigned char *krad, cudaStream_t s,
                           const int *run_if = nullptr);
void ds_launch_origins(const TubeDesc &T, double *orig, cudaStream_t s);
void ds_launch_fill(double *a, int n, double v, cudaStream_t s);
void ds_launch_iota(int *a, int n, cudaStream_t s);

// Sweeps.  what: 0 = gas density + EOS (+ derived c, p/rho^2, CFL minimum),
// 1 = dust self-density, 2 = counts only (parity hook, any species).
void ds_launch_density64(const SweepArgs &a, bool hpp, bool proper, int what, cudaStream_t s);
void ds_launch_force64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s);
void ds_launch_counts64(const SweepArgs &a, bool hpp, bool proper, cudaStream_t s);
void ds_launch_density32(const SweepArgs &a, bool hpp, int what, int depth, cudaStream_t s);
void ds_launch_force32(const SweepArgs &a, bool hpp, int depth, cudaStream_t s);
void ds_launch_force32_list(const SweepArgs &a, bool hpp, cudaStream_t s);
void ds_launch_force32_walk(const SweepArgs &a, bool hpp, int depth, cudaStream_t s);
// blocks per SM of each FP32 sweep (DS_SW_*) for the persistent grids
void ds_sweep32_blocks_per_sm(bool hpp, int depth, bool list, int *bps);
// list reuse: the density of tubes keeping their lists, streamed from them
void ds_launch_density32_lst(const SweepArgs &a, bool hpp, cudaStream_t s);
// The density stream split for a step on bound host arrays: the sums before
// the reorder (cs: the host's state in caller order, slot i holding particle
// slot_pid[i]; Kahan pairs into dsum), the density and the rest after it.
void ds_launch_density32_lst_sums(const SweepArgs &a, bool hpp, DevState cs, const int *slot_pid, float2 *dsum,
                                  cudaStream_t s);
void ds_launch_density32_lst_finish(const SweepArgs &a, bool hpp, float2 *dsum, cudaStream_t s);
// parity hook: one tube's recorded force lists by caller index (a: gas chunks)
void ds_launch_debug_force_lists(const SweepArgs &a, int tube, int cap, int *count, int *nbr, cudaStream_t s);
