// gm_internal.cuh — definitions shared by the CUDA translation units of the
// GB300 backend: fixed-point force format, device status word, cell-grid
// description and the launchers each kernel file exports.
//
// Data layout in HBM (one system, N atoms):
//   * FP64 state in the caller's atom order: pos/vel/ref as x|y|z rows of N.
//   * int64 fixed-point force accumulators F (x|y|z rows, caller order),
//     value = F * 2^-40 kcal/mol/A.  Integer sums are associative, so
//     atomics from any thread order give bit-identical totals.
//   * Cell-sorted copies for the pair kernel: perm[s] = caller index of
//     sorted slot s; hi[s] = (x-o, y-o, z-o rounded to multiples of 2^-8 A,
//     Q_hi), lo[s] = (FP32 remainders of the same, Q_lo with the type in its
//     low 8 bits), Q = sqrt(k_C) q as a double-float; hi+lo carries each
//     coordinate to ~2^-33 A; FP64 mode keeps a sorted double4 copy.
//   * Full (symmetric) neighbour list in warp-interleaved columns: the 32
//     atoms of group g own a slab of 32*cap ints; entry e of lane l sits at
//     g*32*cap + e*32 + l, so one list row is a 128-byte coalesced load.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "geodesic_cuda.h"
#include "gm_df.h"
#include "gm_exact_math.h"

#define GM_FIX_SCALE 1099511627776.0        // 2^40
#define GM_FIX_INV (1.0 / 1099511627776.0)  // 2^-40
constexpr double GM_FORCE_TO_ACCEL = 20.455 * 20.455;  // kcal/mol/A/amu -> A/ps^2 (integrator.rs:9)
#define GM_FIX_SCALE_F 1099511627776.0f
#define GM_FIX_LIMIT 4194304.0              // 2^22: |contribution| must stay below

// Ceiling on distinct (sigma, epsilon) parameter pairs (the type sits in 8
// bits of a slot record; a single system's pair table of 16 B entries lives
// in shared memory while it fits in 48 KB, in L1 otherwise).
#define GM_MAX_TYPES 64
#define GM_WARP 32
#define GM_MAX_SPLIT 16      // largest number of warps per 32-atom group
// The list build runs GM_NSEG warps per 32-atom group, one per z layer of the
// 5 x 5 x (span + 4) cell box the group's candidates come from (cells are at
// least half the list radius wide).  Each warp fills its own staging segment;
// the block then concatenates the segments, layer by layer, into each lane's
// list column.
#define GM_NSEG 5
// Threads per block of the bonded and 1-4 kernels.
#define GM_BONDED_THREADS 64
// List columns are ordered by build-time distance in GM_NBUCKET buckets; the
// build stages a slot index with its bucket in the top bits.
#define GM_NBUCKET 4
#define GM_BUCKET_SHIFT 27
#define GM_SLOT_MASK ((1 << GM_BUCKET_SHIFT) - 1)  // slots per context stay below 2^27

// Device status bits (DevStatus::error).
enum : unsigned int {
    GM_DEV_NONFINITE_POS = 1u << 0,
    GM_DEV_NONFINITE_FORCE = 1u << 1,
    GM_DEV_FIX_OVERFLOW = 1u << 2,
    GM_DEV_LIST_OVERFLOW = 1u << 3,
    GM_DEV_SHAKE_FAIL = 1u << 4,
    GM_DEV_RATTLE_FAIL = 1u << 5,
    GM_DEV_EXTENT = 1u << 6,       // non-periodic extent too large for min-image
    GM_DEV_CELL_OVERFLOW = 1u << 7,
    GM_DEV_ITER_MISMATCH = 1u << 8,
    GM_DEV_BARRIER_TIMEOUT = 1u << 9,  // a grid barrier of the persistent step kernel gave up waiting
};

struct DevStatus {
    unsigned int error;
    unsigned int rebuild;          // 1 when the list must be rebuilt
    unsigned int blocks_done;      // last-block-done counter of the rebuild check
    unsigned int shake_T;          // iteration count of the last SHAKE call
    unsigned int rattle_T;
    unsigned int differs;          // uploaded positions differ from the resident ones
    unsigned long long n_rebuilds;
    unsigned long long step;       // current step of the resident loop
    unsigned long long fail_step;  // first step whose projection failed (init ~0)
    unsigned long long c_steps;    // resident steps with constraints
    unsigned long long shake_sum;  // sum of their SHAKE iteration counts
    unsigned long long rattle_sum; // sum of their RATTLE iteration counts
    unsigned int rec_n;            // warm-start samples recorded (in solves)
    unsigned int bad_pending;      // non-finite positions seen by the fused step kernel, moved to
                                   // error by its last block
    unsigned int max_count;        // largest list length the list build met (sizes a regrowth)
    unsigned int max_layer;        // largest staging (one z layer) length it met
    unsigned int tail_pending;     // unconstrained resident steps: the last step's closing half-kick
                                   // is still to do (the next step's first kernel or the finalizer)
    unsigned long long rebuild_base;  // n_rebuilds when the current call's status was reset
    unsigned int frame_n;          // trajectory frames recorded since they were last taken
    unsigned int frame_lost;       // frames due while the ring was full
};

struct GridInfo {
    double origin[3];   // coordinate origin of the float copies
    float lo[3];        // grid lower corner, origin-relative
    float inv_w[3];     // 1 / cell width
    float box[3], inv_box[3];
    int nc[3];
    int ncell;
    int periodic;
    int full[3];        // scan the whole dimension (periodic, fewer than 5 cells)
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ long long gm_to_fix(double v) { return __double2ll_rn(v * GM_FIX_SCALE); }

// A float force contribution to fixed point; flags non-finite / overflow.
__device__ __forceinline__ long long gm_to_fix_checked(float v, unsigned int &bad) {
    if (!isfinite(v)) { bad |= GM_DEV_NONFINITE_FORCE; return 0; }
    if (fabsf(v) >= (float)GM_FIX_LIMIT) { bad |= GM_DEV_FIX_OVERFLOW; return 0; }
    return gm_f2fix(v);
}
__device__ __forceinline__ long long gm_to_fix_checked(double v, unsigned int &bad) {
    if (!isfinite(v)) bad |= GM_DEV_NONFINITE_FORCE;
    else if (fabs(v) >= GM_FIX_LIMIT) bad |= GM_DEV_FIX_OVERFLOW;
    return __double2ll_rn(v * GM_FIX_SCALE);
}

__device__ __forceinline__ void gm_atomic_fix_add(long long *p, long long v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(p), static_cast<unsigned long long>(v));
}

// Per-system energies of a batch: int64 fixed point at 2^-32 kcal/mol, so the
// sum is independent of the order contributions arrive in.
constexpr double GM_EFIX_SCALE = 4294967296.0;

// Adds each lane's energy e to its system sy (sy < 0: nothing); one atomic
// per warp when the warp's lanes share a system.  All 32 lanes must call.
__device__ __forceinline__ void gm_add_sys_energy(long long *e_sys, int sy, double e) {
    const long long q = sy >= 0 ? __double2ll_rn(e * GM_EFIX_SCALE) : 0ll;
    const int s0 = __shfl_sync(0xffffffffu, sy, 0);
    if (__all_sync(0xffffffffu, sy == s0 || sy < 0) && s0 >= 0) {
        long long t = q;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((threadIdx.x & 31) == 0) gm_atomic_fix_add(e_sys + s0, t);
    } else if (sy >= 0 && q != 0) {
        gm_atomic_fix_add(e_sys + sy, q);
    }
}

// Sum of x[0..n) by a block of 256 threads: per-thread strided partial sums,
// then a tree over the block (fixed order; every caller gets the same bits).
__device__ __forceinline__ double gm_block_sum256(const double *x, int n, double *s) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) acc += x[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    return s[0];
}

// Both float4 of a slot's (hi, lo) coordinate pair in one 256-bit load
// through the read-only path (the pair is 32-byte aligned).
__device__ __forceinline__ void gm_ld_coord(const float4 *p, float4 &h, float4 &l) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(h.x), "=f"(h.y), "=f"(h.z), "=f"(h.w), "=f"(l.x), "=f"(l.y), "=f"(l.z), "=f"(l.w)
        : "l"(p));
}

// A slot's atom type, kept in the low 8 bits of its Q_lo (the low part of a
// double-float charge; those bits are below 2^-39 of Q).
__device__ __forceinline__ int gm_slot_type(float qlo) { return __float_as_int(qlo) & 0xff; }

// Per atom: (Q_hi, Q_lo | type), Q = sqrt(k_C) q, built on the host.
// The slot record of an atom at FP64 offset (ox, oy, oz) from its system's
// grid origin: coordinates rounded to the 2^-8 A grid (differences of two
// such values, and their squares below 16 A, are exact in FP32) and the FP32
// remainders.
__device__ __forceinline__ void gm_pack_record(float4 *rec, double ox, double oy, double oz, float2 qw) {
    const float hx = rintf((float)ox * 256.f) * (1.f / 256.f);
    const float hy = rintf((float)oy * 256.f) * (1.f / 256.f);
    const float hz = rintf((float)oz * 256.f) * (1.f / 256.f);
    rec[0] = make_float4(hx, hy, hz, qw.x);
    rec[1] = make_float4((float)(ox - (double)hx), (float)(oy - (double)hy), (float)(oz - (double)hz), qw.y);
}

// ------------------------------------------------------- launcher exports

struct ListArgs {
    int n;                   // atoms, all systems
    int n_slots;             // sorted slots: each system's atoms padded to a multiple of 32
    int n_sys;               // systems in the context
    int cap;                 // list entries per atom
    int cap_seg;             // staging entries per atom and z layer
    const double *pos;       // FP64 x|y|z rows of n atoms, caller order
    float4 *coord;           // per slot two float4 written by gm_pack_record
    double4 *pos64s;         // per slot FP64 copy (FP64 mode) or nullptr
    int *type_sorted;        // per slot types (FP64 mode)
    int *perm;               // slot -> atom (global index), -1 on padding slots
    int *slot_of;            // atom -> slot (or nullptr)
    int *cell_of;            // atom -> cell of its system
    int *cell_sorted;        // slot -> cell of its system
    int *cell_count, *cell_start, *cell_cursor;  // system s at sys_cell_off[s] (cell_start: ncell + 1 entries)
    int *tmp_atom;           // slot -> atom of the system, before the in-cell rank
    const int *type;         // caller order
    const float2 *qw;        // caller order: (Q_hi, Q_lo | type), see gm_pack_record
    const double *charge64;  // caller order (FP64 mode)
    const int *excl_start, *excl;   // caller-order CSR (both directions, sorted)
    int *list, *count, *gmax;
    int *stage;              // [group][layer][entry][lane], cap_seg entries per layer
    double *ref;             // FP64 x|y|z copy at each system's build
    long long *force;        // zeroed with the pack
    GridInfo *grid;          // one per system
    DevStatus *status;
    double r_list, r_cut, r_switch, box[3];
    int periodic;
    double *bbox_scratch;    // [n_sys][bbox_blocks][9] (min, max, sum per dimension)
    int bbox_blocks, max_sys_atoms;
    // systems: atoms [sys_atom_off[s], +1), slots [sys_slot_off[s], +1) (32-aligned),
    // cells [sys_cell_off[s], +1) (the system's cell budget + 1)
    const int *sys_atom_off, *sys_slot_off, *sys_cell_off;
    const int *atom_sys;     // atom -> system
    const int *group_sys;    // 32-slot group -> system
    unsigned int *sys_flag;  // 1: rebuild the system's list at the next rebuild
};

// set (every system) or clear the rebuild flags; clearing also clears status->rebuild
void gm_launch_flags(const ListArgs &a, bool set, cudaStream_t s);
void gm_launch_wrap(const ListArgs &a, double *pos, cudaStream_t s);
void gm_launch_grid(const ListArgs &a, cudaStream_t s);
void gm_launch_bin(const ListArgs &a, cudaStream_t s);
void gm_launch_build(const ListArgs &a, cudaStream_t s);
void gm_launch_pack(const ListArgs &a, bool fp64, cudaStream_t s);

// Constants of the mixed pair kernel; the low parts complete double-floats.
struct PairConst {
    float rc2, rsw2;          // cutoff^2, switch radius^2 (FP32 tests)
    float rsw, rsw_lo;        // switch radius
    float inv_w, inv_w_lo;    // 1 / (cutoff - switch radius)
    float mds, mds_lo;        // -30 / (cutoff - switch radius): dS/dr = mds u^2 (1 - u)^2
    float box[3], box_lo[3], inv_box[3];
};

struct ForceArgs {
    int n, n_groups, cap;
    int n_slots;             // n_groups * 32 (each system padded to whole groups)
    const int *group_sys, *atom_sys;
    long long *e_sys;        // per-system potential energy, fixed point 2^-32 kcal/mol (batches), or nullptr
    int split;               // warps per 32-atom group in the FP32 pair kernel
    int pair_warps;          // warps per block of the FP32 pair kernel (2, 4, 8)
    int pair_grid;           // blocks of the FP32 pair kernel (0: one work item per warp; fewer: persistent)
    const float4 *coord;     // per slot (hi, lo) pairs: one 32-byte sector per gathered atom
    const double4 *pos64s;
    const int *type_sorted;  // FP64 mode
    const int *perm;
    const int *list, *count, *gmax;
    int ntypes;
    const float4 *tab32;     // (sigma_ij^2, 24 epsilon_ij) per type pair, each a double-float (hi, lo)
    const double2 *tab64;    // (sigma_ij, epsilon_ij)
    PairConst pc;            // the mixed pair kernel's constants
    double rc2_64, rsw_64, rc_64, inv_wsw_64;
    int coulomb;
    float box[3], inv_box[3];
    double box64[3];
    int periodic;
    int bonded_mi;  // periodic && bonded_min_image: bonded and 1-4 differences at the nearest image
    long long *force;
    double *epart;           // per pair-kernel warp (n_groups * split), then bonded, then 1-4
    DevStatus *status;
    const double *pos;       // caller order FP64 (bonded)
    // bonded, caller order
    int n_bonds, n_angles, n_diheds;
    const int *bond_i, *bond_j; const double *bond_k, *bond_r0;
    const int *angle_i, *angle_j, *angle_k; const double *angle_kth, *angle_th0;
    const int *dihed_i, *dihed_j, *dihed_k, *dihed_l; const double *dihed_kphi; const int *dihed_n;
    const double *dihed_delta;
    const double2 *dihed_cs;  // (cos delta, sin delta) per dihedral
    double *epart_bonded;    // per block
    int bonded_blocks;
    // scaled 1-4 pairs
    int n14; const int *p14_i, *p14_j; double scale14_lj, scale14_coul;
    const double *sigma, *epsilon, *charge64;
    const double4 *p14par;   // per 1-4 pair: (sigma_ij, 4 eps_ij s_lj, 24 eps_ij s_lj, k_C q_i q_j s_coul)
    double *epart14; int blocks14;
    double *energy;          // total
    int n_epart_total;       // n_groups * split + bonded_blocks + blocks14 entries
};

void gm_launch_pair(const ForceArgs &a, bool fp64, cudaStream_t s);
void gm_launch_bonded(const ForceArgs &a, bool fp64, cudaStream_t s);
void gm_launch_pair14(const ForceArgs &a, bool fp64, cudaStream_t s);
// the bonded terms and the 1-4 pairs in one launch
void gm_launch_bonded_pair14(const ForceArgs &a, bool fp64, cudaStream_t s);
void gm_launch_energy(const ForceArgs &a, cudaStream_t s);
int gm_bonded_blocks(int n_bonds, int n_angles, int n_diheds);

struct ClusterArgs {
    int n_clusters;
    int n_single;                         // clusters [0, n_single): one constraint on two atoms
    int n_star_end;                       // [n_single, n_star_end): 2-8 constraints sharing one centre atom
    int n_warp_end;                       // [n_star_end, n_warp_end): other clusters, 2-32 constraints, <= 32 atoms
    const int *cl_cstart, *cl_cons;       // cluster -> constraints (ascending)
    const int *cl_astart, *cl_atoms;      // cluster -> atoms
    const int *cl_acstart, *cl_acons;     // cluster-atom slot -> signed constraint refs (ascending)
    const int *constr_i, *constr_j;
    const double *constr_dsq;
    const double *inv_mass;               // 1.0 / mass (caller order)
    double *lam;                          // per constraint scratch
    double *lam_sum;                      // per constraint accumulated multiplier (nullptr: not kept)
    const double *lam0;                   // per constraint warm-start multiplier (nullptr: cold start)
    double *rvec;                         // per constraint reference vector (3 x C)
    int *cl_iters;                        // per cluster iteration count
    double *cl_worst;                     // per cluster last max |lambda|
    int *cl_worst_idx;                    // per cluster constraint of that max
    int n_constr;
    unsigned int max_iter;
    double tol;
    DevStatus *status;
    int mi;                               // constraint differences at the nearest image of box64
    double box64[3];
};

// d taken to the nearest periodic image of a box of length L: the reference's
// min_image, d - L * round(d / L) with round half away from zero; each
// operation rounded on its own (never contracted into an FMA, whatever the
// translation unit's -fmad setting), so the bits are the reference's
__device__ __forceinline__ double gm_min_image(double d, double L) {
    return __dsub_rn(d, __dmul_rn(L, round(__ddiv_rn(d, L))));
}

void gm_launch_half_kick(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                         const DevStatus *st, cudaStream_t s);
void gm_launch_half_kick_f64(int n, double *vel, const double *force, const double *inv_mass, double dt_half,
                             cudaStream_t s);
void gm_launch_drift(int n, double *pos, double *vel, double *dref, double dt, bool resync, const DevStatus *st,
                     cudaStream_t s);
void gm_launch_resync(int n, const double *pos, double *vel, const double *dref, double dt, const DevStatus *st,
                      cudaStream_t s);
void gm_launch_check(int n, const double *pos, const double *ref, double thr_sq, DevStatus *st,
                     unsigned long long cond_handle, int blocks, const int *atom_sys, unsigned int *sys_flag,
                     cudaStream_t s);
void gm_launch_shake(const ClusterArgs &c, int n_atoms, const double *dref, double *pos, cudaStream_t s);
// the same solve in two halves, so the warm start can run in between:
// prepare (reset T, reference vectors, multiplier sums) and the iterations
// (warm-start displacement when c.lam0 is set, then both phases)
void gm_launch_shake_prepare(const ClusterArgs &c, int n_atoms, const double *dref, cudaStream_t s);
int gm_launch_shake_solve(const ClusterArgs &c, int n_atoms, double *pos, cudaStream_t s);
void gm_launch_rattle(const ClusterArgs &c, int n_atoms, const double *pos, double *vel, cudaStream_t s);
void gm_launch_step(DevStatus *st, cudaStream_t s);
// Unconstrained step: half-kicks (the previous step's closing one and this
// step's opening one) + drift (with the velocity resync) + rebuild check +
// coordinate pack in one launch.  Each atom gets the same operations in the
// same order as the separate kernels.
// The pack kernel's per-atom work (FP32 (hi, lo) copies relative to the
// system's grid origin, FP64 copies in FP64 mode, forces cleared), done by the
// fused step kernel for the force evaluation that follows it.
struct PackArgs {
    float4 *coord;
    double4 *pos64s;
    int *type_sorted;
    const int *slot_of;
    const GridInfo *grid;
    const int *type;
    const float2 *qw;
    const double *charge64;
    int fp64;
};
// The persistent step kernel (gm_step.cu): one cooperative launch per
// unconstrained mixed-precision step.  Its force phase hands out work items
// (pair items and 32-term bonded / 1-4 chunks) from `ticket`; one grid
// barrier separates it from the kick / drift / rebuild check / pack phase.
struct StepSync {
    unsigned int arrive;  // blocks arrived at the grid barrier
    unsigned int gen;     // barrier generation
    unsigned int ticket;  // next work item of the force phase
    unsigned int fresh;   // nonzero: the forces at the current positions are summed already (skip the phase)
};
struct StepArgs {
    int n;
    double *pos, *vel, *dref;
    const double *inv_mass, *ref;
    double dt_half, dt, inv_dt, thr_sq;
    unsigned long long cond;   // graph conditional handle of the rebuild, or 0
    const int *atom_sys;
    unsigned int *sys_flag;
    StepSync *sync;
};
// Blocks of the cooperative grid (all co-resident); 0 when the form does not apply.
int gm_step_persistent_blocks(const ForceArgs &fa);
void gm_launch_step_persistent(const ForceArgs &fa, const StepArgs &sa, const PackArgs &pk, int blocks,
                               cudaStream_t s);
// The persistent kernel's force phase alone, with energies (the force
// kernels' partials, the same bits), as a plain launch: pair items and bonded
// / 1-4 blocks from one queue.  The queue words must be zero.
void gm_launch_forces_persistent(const ForceArgs &fa, StepSync *sync, int blocks, cudaStream_t s);
void gm_launch_kick_drift_check(int n, double *pos, double *vel, double *dref, long long *force,
                                const double *inv_mass, double dt_half, double dt, const double *ref, double thr_sq,
                                DevStatus *st, unsigned long long cond, const int *atom_sys, unsigned int *sys_flag,
                                const PackArgs &pk, cudaStream_t s);
// Trajectory frames recorded on the device during resident steps.
struct FrameArgs {
    int interval;                // a frame when the completed step count is a multiple (0: none)
    int cap;                     // frames the ring holds
    float *xyz;                  // [cap][3][n] positions as float32
    unsigned long long *step;    // [cap] step of each frame
    double *energy;              // [cap][2] potential and kinetic energy (kcal/mol)
    double *partial;             // [kFrameBlocks] kinetic partial sums
    const double *epart;         // energy partials of the last force evaluation
    int n_epart;
};
constexpr int GM_FRAME_BLOCKS = 64;  // the kinetic reduction's grid (as gm_kinetic_energy's)
// Records a frame when the step just completed is due: positions as float32,
// the kinetic energy of the step's final velocities (its closing half-kick
// applied when still pending, in the finalizer's arithmetic; the reduction of
// gm_kinetic_energy) and the potential energy (the energy kernel's sum).
void gm_launch_frame(int n, const double *pos, const double *vel, const long long *force, const double *inv_mass,
                     const double *mass, double dt_half, DevStatus *st, const FrameArgs &f, cudaStream_t s);
// The closing half-kick and step count of the last unconstrained resident
// step, when one is pending (a no-op otherwise).
void gm_launch_kick_tail(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                         DevStatus *st, cudaStream_t s);
void gm_launch_kinetic(int n, const double *vel, const double *mass, double *partials, int blocks, double *out,
                       cudaStream_t s);
void gm_launch_forces_out(int n, const long long *force, double *out, cudaStream_t s);
void gm_launch_differs(int n, const double *a, const double *b, unsigned int *flag, cudaStream_t s);
// The per-call status reset on the device: counters kept, per-call fields
// cleared, the step set when set_step, n_rebuilds noted as the call's base.
void gm_launch_status_reset(DevStatus *st, int set_step, unsigned long long step, cudaStream_t s);
int gm_check_blocks(int n);

// ---- constraint warm start (gm_mlp.cu) -----------------------------------
// A 12-64-64-1 SiLU network over per-constraint features predicts the
// constraint's total SHAKE multiplier, as a correction to the first Jacobi
// step (t = Lambda * 2 (1/m_i + 1/m_j) = t1 + network).  FP32 master parameters, laid out as
// W1[12][64], b1[64], W2[64][64], b2[64], w3[64], b3; the matmul weights and
// the activations are rounded to BF16, sums are FP32.  norm holds the
// feature means[12], feature scales[12], target mean, target scale.
constexpr int GM_WS_IN = 12, GM_WS_H = 64;
constexpr int GM_WS_OFF_W1 = 0, GM_WS_OFF_B1 = 768, GM_WS_OFF_W2 = 832, GM_WS_OFF_B2 = 4928, GM_WS_OFF_W3 = 4992,
              GM_WS_OFF_B3 = 5056, GM_WS_NPAR = 5057, GM_WS_NNORM = 26;
constexpr int GM_WS_TILE = 128;  // samples per block of the training kernel

// Features of constraint k = (i, j), d0^2 = dsq, r = ref_i - ref_j, d =
// trial_i - trial_j, w = 1/m_i + 1/m_j:
//  0 (d.d - d0^2) / d0^2   1 d.r / d0^2   2 d0   3 1/m_i   4 1/m_j
//  5, 6 constraints on i, on j   7 t1 = (d.d - d0^2) / d.r (the first Jacobi
//  step times 2 w)   8 c1 = sum over the other constraints l on a shared
//  atom a of (1/m_a) / w_k cos(r_k, r_l) s_k s_l t1_l w_k / w_l (the first
//  order coupling; s = +1 where a is the constraint's i, -1 where it is j)
//  9 sum of the squared coupling coefficients   10 max |cos|   11 sum of t1_l
//  (8-11 in FP32)
struct WsFeatureArgs {
    int n_constr, n_atoms;
    const int *constr_i, *constr_j;
    const double *constr_dsq, *inv_mass;
    const int *atom_cstart, *atom_cref;  // per-atom constraints (CSR; ref k: atom is i, -k-1: atom is j)
    const double *pos, *dref;    // trial and reference positions
    float *feat;                 // [n_constr][12] raw features
    double *scale;               // 2 (1/m_i + 1/m_j) per constraint
    double *t1;                  // first Jacobi step of a cold solve, times scale
    float4 *unit;                // (reference bond direction, t1) per constraint (FP32), for the coupling pass
    const float *w;              // 1/m_i + 1/m_j per constraint, FP32 (each mass rounded first)
};
// Two launches per solve: every constraint's raw features, t1 and scale, and
// with infer the network on the tensor cores (fused with the coupling pass)
// and the predicted multipliers lam0[k] = (t1[k] + y_k * t_scale + t_mean) /
// scale[k].  `packed`: the parameters and standardisation as gm_launch_ws_pack
// left them.
void gm_launch_ws_predict(const WsFeatureArgs &a, const void *packed, double *lam0, bool infer, cudaStream_t s);
// The inference's parameter block (gm_ws_packed_bytes bytes), written from
// the parameters and the input standardisation; run after every change of
// either.
size_t gm_ws_packed_bytes();
void gm_launch_ws_pack(const float *params, const float *norm, void *packed, cudaStream_t s);
// The network's output y for m standardised inputs x[m][12] (same kernels).
void gm_launch_ws_forward(int m, const float *x, const float *params, float *y, cudaStream_t s);
// records raw features and targets lam_sum * scale - t1 into slot rec_n when
// step % stride == 0 (resident steps), then advances rec_n
void gm_launch_ws_record(int n_constr, const float *feat, const double *lam_sum, const double *scale, const double *t1,
                         float *rec_feat, float *rec_t, int stride, int cap_slots, DevStatus *st, cudaStream_t s);
// feature/target statistics over n samples into norm (device, deterministic)
void gm_launch_ws_stats(long long n, const float *feat, const float *t, double *partial, int blocks, float *norm,
                        cudaStream_t s);
// one forward/backward pass over a batch of blocks x 128 samples; sample b*128+s
// is idx ? idx[...] : hash(seed, iter, .) % n.  Writes per-block gradients
// and loss into partial[blocks][NPAR + 1]; rows past n_valid count nothing.
void gm_launch_ws_grad(long long n, const float *feat, const float *t, const float *norm, bool standardized,
                       const float *params, int blocks, unsigned long long seed, long long iter, long long n_valid,
                       float *partial, cudaStream_t s);
// fixed-order sum of the block gradients; Adam step when m != nullptr,
// otherwise the summed gradient (and loss) go to grad_out
void gm_launch_ws_update(int blocks, const float *partial, float *params, float *m, float *v, float lr, float b1,
                         float b2, float eps, int t, float *grad_out, cudaStream_t s);
