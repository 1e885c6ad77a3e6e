/*
 * geodesic_cuda.h — C ABI of the GB300 (sm_103a) compute backend for
 * GEODESIC-M, selected as `backend = "cuda"` beside "cpu" and "gpu".
 *
 * The entry points mirror the reference's `ComputeBackend` trait
 * (geodesic-core/src/backend.rs:11-23) plus the three engine free functions
 * the run loop calls directly (integrator::half_kick, constraint::
 * constrain_velocities, lib.rs:68-77 kinetic energy).  All arrays are plain
 * caller-owned host pointers in the reference's SoA layout (f64 x/y/z rows,
 * u32 indices); they are read or written only during the call.  Device
 * buffers are owned by the context.  Every call returns a gm_status (0 = ok).
 *
 * Thread safety: a context may be driven from any one thread at a time (the
 * trait is `Send`, not `Sync`); each entry point makes the context's device
 * current itself and uses the context's own stream.
 */
#ifndef GEODESIC_CUDA_H
#define GEODESIC_CUDA_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The Rust binding maps them onto the reference's errors:
 * NO_DEVICE -> BackendError::NoAdapter, OUT_OF_MEMORY ->
 * BackendError::OutOfGpuMemory, DEVICE -> BackendError::DeviceLost,
 * CONVERGENCE -> ConvergenceError::ConstraintSolver (details in
 * gm_convergence), NONFINITE -> NumericalError, others -> ConfigError. */
typedef enum {
    GM_OK = 0,
    GM_ERR_INVALID_ARGUMENT = 1,
    GM_ERR_NO_DEVICE = 2,
    GM_ERR_OUT_OF_MEMORY = 3,
    GM_ERR_DEVICE = 4,
    GM_ERR_CONVERGENCE = 5,
    GM_ERR_NONFINITE = 6,
    GM_ERR_LIST_OVERFLOW = 7,
    GM_ERR_UNSUPPORTED = 8,
    GM_ERR_FIXED_POINT_OVERFLOW = 9,
    GM_ERR_NOT_BUILT = 10
} gm_status;

/* Arithmetic of the force path. */
typedef enum {
    GM_PRECISION_MIXED = 0, /* FP32 pair/bonded math, int64 fixed-point sums, FP64 energy and integrator */
    GM_PRECISION_FP64 = 1   /* FP64 everywhere (int64 fixed-point sums) */
} gm_precision;

/* AtomData (geodesic-core/src/atoms.rs:3-12); element: 0 = hydrogen. */
typedef struct {
    int64_t n_atoms;
    const double *sigma, *epsilon, *mass, *charge;
    const uint8_t *element; /* may be NULL (no hydrogen information) */
} gm_atoms;

/* BondedTopology (geodesic-core/src/topology.rs:4-37). */
typedef struct {
    int64_t n_bonds;  const uint32_t *bond_i, *bond_j; const double *bond_k, *bond_r0;
    int64_t n_angles; const uint32_t *angle_i, *angle_j, *angle_k; const double *angle_kth, *angle_th0;
    int64_t n_diheds; const uint32_t *dihed_i, *dihed_j, *dihed_k, *dihed_l;
    const double *dihed_kphi; const uint32_t *dihed_n; const double *dihed_delta;
    int64_t n_constr; const uint32_t *constr_i, *constr_j; const double *constr_dsq;
    int64_t n_excl;   const uint32_t *excl_i, *excl_j;
} gm_topology;

/* SimParams (geodesic-core/src/params.rs:4-23), fields on the path. */
typedef struct {
    double box[3];
    int32_t periodic;
    int32_t precision;        /* gm_precision */
    double r_cutoff, r_skin, r_switch;
    uint32_t max_constr_iter;
    double constr_tol;
    /* beyond the reference (0 = off = reference behaviour) */
    int32_t coulomb;          /* q_i q_j 332.0522173 / r with the LJ switch */
    double scale14_lj, scale14_coul;
    int32_t device;           /* CUDA device ordinal */
    /* beyond the reference: with periodic, the displacement between the two
     * atoms of a bond, angle arm, dihedral bond vector, 1-4 pair or
     * constraint goes to the nearest periodic image, d - L round(d / L), the
     * reference's min_image (neighbor.rs:74-76) that its bonded and
     * constraint terms leave out (memory.md:140-144).  0 = off = reference.
     * The SHAKE warm start (gm_ws_record, gm_ws_enable) is unsupported with it. */
    int32_t bonded_min_image;
} gm_params;

/* ConvergenceError::ConstraintSolver (geodesic-core/src/error.rs:50-63). */
typedef struct {
    uint64_t step;
    int64_t constraint_idx, atom_i, atom_j;
    double residual;
    uint32_t max_iter;
} gm_convergence;

typedef struct gm_ctx gm_ctx;

/* CpuBackend::new / GpuBackend::try_new (cpu_backend.rs:50-83,
 * gpu_backend.rs:24-53).  Copies atoms and topology to the device.  Returns
 * NULL and sets *status on failure. */
gm_ctx *gm_create(const gm_atoms *atoms, const gm_topology *topo, const gm_params *params, int32_t *status);

/* Drop of the backend. */
int32_t gm_destroy(gm_ctx *ctx);

/* ComputeBackend::build_neighbor_list (backend.rs:14, neighbor.rs:8-55).
 * Wraps positions in place when periodic; the list is kept on the device. */
int32_t gm_build_list(gm_ctx *ctx, double *px, double *py, double *pz);

/* ComputeBackend::compute_forces + potential_energy (backend.rs:15,18,
 * cpu_backend.rs:92-182): bonded + nonbonded forces at the given positions
 * into fx/fy/fz (overwritten), total potential into *energy.  On failure the
 * forces are NaN-poisoned so the caller's finiteness check stops the run. */
int32_t gm_compute_forces(gm_ctx *ctx, const double *px, const double *py, const double *pz,
                          double *fx, double *fy, double *fz, double *energy);

/* ComputeBackend::needs_rebuild (backend.rs:21, neighbor.rs:60-72). */
int32_t gm_needs_rebuild(gm_ctx *ctx, const double *px, const double *py, const double *pz, int32_t *result);

/* ComputeBackend::geodesic_drift (backend.rs:16, integrator.rs:32-71):
 * r += dt v, SHAKE projection, v = (r_new - r_old)/dt.  On non-convergence
 * returns GM_ERR_CONVERGENCE with *err filled (positions left partially
 * corrected, as the reference does). */
int32_t gm_geodesic_drift(gm_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy, double *vz,
                          double dt, uint64_t step, gm_convergence *err);

/* integrator::half_kick (integrator.rs:14-21). */
int32_t gm_half_kick(gm_ctx *ctx, double *vx, double *vy, double *vz, const double *fx, const double *fy,
                     const double *fz, double dt_half);

/* constraint::constrain_velocities (constraint.rs:170-259), RATTLE. */
int32_t gm_constrain_velocities(gm_ctx *ctx, const double *px, const double *py, const double *pz,
                                double *vx, double *vy, double *vz, uint64_t step, gm_convergence *err);

/* lib.rs:68-77 */
int32_t gm_kinetic_energy(gm_ctx *ctx, const double *vx, const double *vy, const double *vz, double *ke);

/* ComputeBackend::n_threads (backend.rs:22): always 1 (gpu_backend.rs:99). */
int32_t gm_n_threads(const gm_ctx *ctx);

/* Copies the current half pair list out as the reference's NeighborList
 * pair_i/pair_j (topology.rs:42-55): i < j, sorted by (i, then j).  With
 * pair_i == NULL only *n_pairs is returned. */
int32_t gm_get_pairs(gm_ctx *ctx, int64_t cap, uint32_t *pair_i, uint32_t *pair_j, int64_t *n_pairs);

/* Device-resident BAB + RATTLE loop (lib.rs:292-323 without I/O): uploads
 * (p, v), runs n_steps steps with the list rebuilt on the device whenever an
 * atom moved more than half the skin, downloads (p, v) and the last forces
 * (fx/fy/fz may be NULL) and potential energy.  *n_rebuilds (nullable)
 * receives the number of list rebuilds. */
int32_t gm_steps(gm_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy, double *vz,
                 double dt, uint64_t first_step, int64_t n_steps, double *fx, double *fy, double *fz,
                 double *energy, int64_t *n_rebuilds, gm_convergence *err);

/* Copies the last error message (NUL-terminated, truncated to len). */
int32_t gm_last_error(const gm_ctx *ctx, char *buf, int64_t len);

/* ---- resident-state interface (benchmarks, batching) ------------------ */

/* Uploads positions and velocities to the device state.  The neighbour list
 * is kept (rebuilt later only if an atom moved more than half the skin), and
 * the resident forces stay valid when the positions equal the resident ones. */
int32_t gm_upload_state(gm_ctx *ctx, const double *px, const double *py, const double *pz,
                        const double *vx, const double *vy, const double *vz);
/* Downloads positions and velocities from the device state. */
int32_t gm_download_state(gm_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy, double *vz);
/* Runs n_steps BAB steps on the resident state (asynchronous on the
 * context's stream; call gm_synchronize to collect errors). */
int32_t gm_run_resident(gm_ctx *ctx, double dt, uint64_t first_step, int64_t n_steps);
/* Evaluates forces on the resident positions; first rebuilds the list when
 * an atom moved more than half the skin since the last build (the check is
 * one host synchronisation; the force launches are asynchronous). */
int32_t gm_forces_resident(gm_ctx *ctx);
/* Waits for the stream and reports device-side errors. */
int32_t gm_synchronize(gm_ctx *ctx, gm_convergence *err);
/* Average device time (ms, CUDA events on the context's stream) of one
 * launch of: which = 0 the pair kernel, 1 the bonded kernel, 2 the list
 * rebuild sequence, 3 one captured BAB step of length dt, 4 the pack kernel,
 * 5 the force evaluation of a step (pack, then the pair kernel beside the
 * bonded and 1-4 kernels), 6 the 1-4 kernel, 7 the list build kernel (with
 * its flag set/clear launches).  Runs on the resident state
 * (which = 3 advances it); forces are recomputed afterwards. */
int32_t gm_profile(gm_ctx *ctx, int32_t which, int32_t n_iter, double dt, double *avg_ms);
/* Runs n_steps resident BAB steps, each bracketed by CUDA events; with
 * flush_buf (a device buffer larger than L2) a memset of flush_bytes runs
 * between steps, outside the bracketed time.  *total_ms = sum of step times. */
int32_t gm_time_steps(gm_ctx *ctx, double dt, uint64_t first_step, int64_t n_steps, void *flush_buf,
                      int64_t flush_bytes, double *total_ms);
/* The context's cudaStream_t, for callers that time work on it. */
void *gm_stream(gm_ctx *ctx);
/* Counters: [0] pairs in the current list, [1] list rebuilds so far,
 * [2] list capacity per atom, [3] kernel launches issued so far,
 * [4] last SHAKE iteration count, [5] last RATTLE iteration count,
 * [6] kernel launches per captured step, [7] warps per 32-atom group in the
 * FP32 pair kernel, [8] resident steps with constraints, [9] / [10] the sum
 * of their SHAKE / RATTLE iteration counts, [11] warm-start solves recorded. */
int32_t gm_counters(const gm_ctx *ctx, int64_t *out, int64_t n);

/* ---- batches of independent systems (no reference counterpart) --------
 *
 * One context holding n_systems independent systems (the reference runs one
 * ComputeBackend per system): atoms[s], topos[s] describe system s with its
 * own atom indices; they share params.  The systems are concatenated in
 * order (system s's atoms at offsets [off[s], off[s+1]) of every per-atom
 * array the entry points above take), never interact, and advance together:
 * one graph launch per step covers all of them, with one kernel launch per
 * kernel for the whole batch, and each system's list is rebuilt only when
 * one of its own atoms moved more than half the skin.  Each system has its
 * own cell grid and Lennard-Jones type table (up to 64 types per system).
 * The SHAKE/RATTLE stop rule runs over the whole batch (every cluster
 * iterates to the batch's largest count, each converged to the tolerance). */
gm_ctx *gm_create_ensemble(int32_t n_systems, const gm_atoms *atoms, const gm_topology *topos,
                           const gm_params *params, int32_t *status);
/* off[0..n_systems]: the first atom of each system, then the atom count. */
int32_t gm_ensemble_info(const gm_ctx *ctx, int64_t *atom_offsets);
/* Per-system potential energy at the last force evaluation (int64 fixed-point
 * sums, so a system's value does not depend on the batch around it) and
 * kinetic energy of the resident velocities (lib.rs:68-77); NULL skips. */
int32_t gm_ensemble_energies(gm_ctx *ctx, double *e_pot, double *e_kin);

/* ---- trajectory frames (the run loop's frame output, lib.rs:325-331,
 * 347-361, recorded on the device) -------------------------------------
 *
 * With frame_interval > 0, every resident step (gm_run_resident, gm_steps,
 * gm_time_steps) whose completed step count is a multiple of frame_interval
 * records a frame into a device ring of `capacity` frames: the positions as
 * float32 rows x|y|z (the run loop's f32 conversion), the potential energy of
 * the step's force evaluation and the kinetic energy of its final velocities
 * (the sums of potential_energy / gm_kinetic_energy).  Frames due while the
 * ring is full are counted as lost.  0 turns recording off.  Changing the
 * setting recaptures the step graph. */
int32_t gm_frames_enable(gm_ctx *ctx, int32_t frame_interval, int32_t capacity);
/* Copies the frames recorded since the last call, oldest first, and empties
 * the ring: xyz [n][3][N] float32, steps [n], e_pot / e_kin [n] (kcal/mol);
 * any pointer may be NULL.  *n_frames = n; GM_ERR_INVALID_ARGUMENT (nothing
 * taken) when n > max_frames.  *n_lost (nullable): frames dropped on a full
 * ring. */
int32_t gm_frames_take(gm_ctx *ctx, int64_t max_frames, float *xyz, uint64_t *steps, double *e_pot, double *e_kin,
                       int64_t *n_frames, int64_t *n_lost);

/* ---- autotuner (no reference counterpart) ------------------------------
 *
 * Times the context's pair kernel (mixed or FP64) on the current list
 * (reps launches per candidate, CUDA events on the context's stream) over
 * warps per 32-atom group (1-16: list columns per warp), warps per block (2,
 * 4, 8) and grid (one work item per warp, or a persistent grid of 2-16
 * blocks per SM), and keeps the fastest.  In the persistent step form
 * (gm_step_form) the split is then timed again on the persistent kernel's
 * force phase and the fastest kept.  Every candidate computes the same force
 * bits (fixed 32-entry chunks folded into int64 sums).  choice (nullable):
 * split, warps per block, grid (0 = one item per warp). */
int32_t gm_autotune(gm_ctx *ctx, int32_t reps, int64_t *choice);
/* Sets the pair kernel's launch shape directly (a choice gm_autotune returned
 * earlier, e.g. cached across runs): split 1-16, warps per block 2, 4 or 8,
 * grid 0 (one work item per warp) or a block count.  The forces are the same
 * bits for every shape. */
int32_t gm_pair_shape(gm_ctx *ctx, int32_t split, int32_t warps_per_block, int32_t grid);

/* ---- step form (no reference counterpart) ------------------------------
 *
 * How the resident steps of an unconstrained mixed-precision context are
 * issued (gm_steps, gm_run_resident, gm_time_steps):
 *   GM_STEP_GRAPH       one captured graph per step: the fused
 *                       kick/drift/check/pack kernel, the rebuild IF node,
 *                       the pair kernel beside the bonded / 1-4 kernel.
 *   GM_STEP_PERSISTENT  one captured graph per step holding ONE persistent
 *                       cooperative launch (forces at the current positions
 *                       from a single work queue of pair items and bonded /
 *                       1-4 chunks over every system of an ensemble, a grid
 *                       barrier, then kick/drift/check/pack) and the rebuild
 *                       IF node.  The forces at the final positions are
 *                       evaluated by the force kernels after the last launch.
 * Both forms give the same bits.  GM_ERR_UNSUPPORTED for an FP64 or
 * constrained context; with trajectory frames enabled the graph form runs.
 * The default is GM_STEP_PERSISTENT (the kernel graph for FP64 and
 * constrained contexts).  In mixed precision with GM_STEP_PERSISTENT every
 * force evaluation outside the persistent launches (gm_compute_forces, list
 * builds, the constrained step graph) runs as the persistent kernel's force
 * phase alone: one launch over the same work queue, the same bits. */
enum { GM_STEP_GRAPH = 0, GM_STEP_PERSISTENT = 1 };
int32_t gm_step_form(gm_ctx *ctx, int32_t form);
/* Error-path test of the persistent form's grid barrier: the next call that
 * runs persistent steps starts with the barrier's arrival count far past the
 * grid, so no block can release it.  Every block waits out the barrier's
 * poll limit (a fraction of a second), records the timeout and returns; the
 * call returns GM_ERR_DEVICE with nothing stepped, and the context is usable
 * afterwards.  GM_ERR_UNSUPPORTED unless the context steps in the
 * persistent form. */
int32_t gm_stall_next_barrier(gm_ctx *ctx);

/* ---- constraint warm start (no reference counterpart) ------------------
 *
 * A 12-64-64-1 SiLU network (BF16 matmul weights and activations, FP32
 * sums) predicts each constraint's total SHAKE multiplier Lambda (the sum of
 * the Jacobi lambdas of constraint.rs:62-152) from 12 rotation-invariant
 * features of the constraint and of the constraints sharing its atoms: with
 * r = r_ref, d = r_trial, (d.d - d0^2)/d0^2, d.r/d0^2, d0, 1/m_i, 1/m_j, the
 * constraint counts on i and j, t1 (below), the first-order coupling
 * sum_l (1/m_a)/w cos(r_k, r_l) s_k s_l t1_l w_k/w_l over the constraints l
 * sharing an atom a (s = +1 at the constraint's i, -1 at its j, w =
 * 1/m_i + 1/m_j), the sum of the squared coupling coefficients, the largest
 * |cos| and the sum of the neighbours' t1.  With the warm start on, each
 * SHAKE solve first moves the atoms once with the predicted multipliers (the
 * Jacobi update formula) and then runs the unchanged iteration to the same
 * tolerance, so the result meets the same convergence test.  Parameters:
 * 5057 FP32 values (W1[12][64], b1[64], W2[64][64], b2[64], w3[64], b3);
 * norm: 26 FP32 values (feature means[12], scales[12], target mean, scale).
 * The network output is the standardised correction t - t1, where t =
 * Lambda * 2 (1/m_i + 1/m_j) and t1 = (|r_trial|^2 - d0^2) / (r_trial .
 * r_ref) is the first Jacobi step of a cold solve. */

/* Records (raw features, target t - t1) of every constraint at every stride-th
 * resident step (gm_run_resident / gm_time_steps / gm_steps), up to
 * cap_steps solves; cap_steps = 0 stops recording and keeps the samples. */
int32_t gm_ws_record(gm_ctx *ctx, int64_t cap_steps, int32_t stride);
/* Copies up to cap recorded samples (feat: [cap][12], target: [cap]). */
int32_t gm_ws_samples(gm_ctx *ctx, int64_t cap, float *feat, float *target, int64_t *n_samples);
/* Trains the network on the GPU from a seeded Glorot start: feature and
 * target statistics over the recorded samples, then iters Adam steps
 * (cosine-decayed lr) on batches of blocks x 128 samples drawn by a seeded
 * hash.  *final_loss: mean squared error of the last batch (standardised). */
int32_t gm_ws_train(gm_ctx *ctx, int64_t iters, int32_t blocks, double lr, uint64_t seed, double *final_loss);
/* Uses (1) or stops using (0) the network as the SHAKE warm start. */
int32_t gm_ws_enable(gm_ctx *ctx, int32_t on);
/* Gets and/or sets the parameters (5057) and norm (26); NULL skips. */
int32_t gm_ws_params(gm_ctx *ctx, float *get_params, float *get_norm, const float *set_params, const float *set_norm);
/* Network output for m standardised inputs x[m][12] (host). */
int32_t gm_ws_forward(gm_ctx *ctx, const float *x, int64_t m, float *y);
/* Gradient (5057) of the mean squared error over m standardised samples
 * (x[m][12], t[m]) by the training kernels, and the loss. */
int32_t gm_ws_gradient(gm_ctx *ctx, const float *x, const float *t, int64_t m, float *grad, double *loss);
/* Raw features ([C][12]), predicted multipliers and multiplier totals of the
 * last solve that computed them (NULL skips). */
int32_t gm_ws_last(gm_ctx *ctx, float *feat, double *lam0, double *lam_sum);

/* ---- allocation-free list build ---------------------------------------- */

/* Largest system gm_build_pairs_static accepts, and the size of the one
 * static device array (per device) that holds its scratch. */
#define GM_STATIC_MAX_ATOMS 16384
#define GM_STATIC_SCRATCH_BYTES (1280u * 1024u)

/* No reference counterpart.  Builds the half neighbour list of a system of
 * at most GM_STATIC_MAX_ATOMS atoms without allocating device memory: no
 * context, no cudaMalloc/cudaFree, no allocating library call; the scratch
 * is a static __device__ array of GM_STATIC_SCRATCH_BYTES.  It serves
 * callers that cannot allocate when they need the list: a host engine whose
 * device memory is held by its own pool, or a step running beside other
 * streams, where cudaFree waits for the whole device.
 *
 * All pointers but params and n_pairs are DEVICE pointers on params->device,
 * which is current during the call; the caller's current device is restored
 * before it returns.  d_pos: x|y|z rows of n_atoms doubles, wrapped into the
 * box in place when periodic (as gm_build_list does).  d_excl_start
 * (n_atoms + 1) / d_excl: exclusions as CSR, both directions, each row
 * ascending (both NULL for none).  The pairs (i < j, |r_ij| <= r_skin by the
 * reference's FP64 test, excluded pairs left out) go to d_pair_i/d_pair_j,
 * sorted by (i, then j): the same list gm_get_pairs returns.  *n_pairs
 * (host) receives the count; with d_pair_i == NULL only the count is
 * computed.  If the count exceeds max_pairs nothing is written and
 * GM_ERR_LIST_OVERFLOW is returned; after any other error return the pair
 * buffers are untouched as well.  n_atoms > GM_STATIC_MAX_ATOMS returns
 * GM_ERR_UNSUPPORTED before any device call.  Runs on `stream` (a
 * cudaStream_t; NULL = the default stream) and returns after it finished.
 *
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress, which also loads the module there); make that first
 * call before any stream capture.  All calls on one device share the one
 * scratch array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. */
int32_t gm_build_pairs_static(double *d_pos, int32_t n_atoms, const int32_t *d_excl_start, const int32_t *d_excl,
                              const gm_params *params, uint32_t *d_pair_i, uint32_t *d_pair_j, int64_t max_pairs,
                              int64_t *n_pairs, void *stream);

#ifdef __cplusplus
}
#endif
#endif
