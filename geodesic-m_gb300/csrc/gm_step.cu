// gm_step.cu — the unconstrained mixed-precision BAB step (lib.rs:292-323
// without constraints) as one persistent cooperative launch per step.
//
// Launch k of a run starts from the positions x_k that launch k-1 left (and
// the list that the graph's conditional rebuild left after it):
//   1. forces F(x_k): every warp takes work items from one queue: the pair
//      items of the mixed kernel (pair_item_mixed, a 32-atom group's share of
//      list columns) and 128-term chunks of the bonded terms and 1-4 pairs,
//      spread evenly through the queue so that each SM mixes FP32 pair work
//      with FP64 bonded work.  Skipped when the forces at x_k are summed
//      already (the first launch of a call: the call starts with current
//      forces).
//   2. one grid barrier (bounded: a block that waits too long records
//      GM_DEV_BARRIER_TIMEOUT and returns).
//   3. per atom, grid-strided: the closing half-kick of step k-1 (when
//      pending) and the opening half-kick of step k with F(x_k), the drift to
//      x_{k+1}, the velocity resync, the pack of x_{k+1}, the zeroing of the
//      force sums and the rebuild check; the last block sets the graph's
//      rebuild condition.
// The graph that holds the launch has one more node, the IF node of the list
// rebuild.  After the last launch of a call the forces F(x_n) are evaluated
// by this kernel's force phase alone (the STEP = false instantiation, with
// energies) and the closing half-kick by the tail kernel, so a call ends as
// in the kernel-graph form.
//
// The launch performs the kernel-graph form's operations in the same order:
// force sums are integer sums (the order of the work items changes no bit),
// and phase 3 is written with explicit round-to-nearest operations, so it
// rounds like the integrator kernels, which are compiled without
// contraction.  Energies are not evaluated inside the loop (the force
// evaluation after the last launch sums them): the pair items and the
// bonded chunks add forces only.
#include "gm_force_terms.cuh"

namespace {

constexpr int kStepThreads = 128;
constexpr int kStepMinBlocks = 6;  // 24 warps per SM: at most 80 registers a thread
constexpr int kTermsPerTicket = 128;  // bonded terms (or 1-4 pairs) per work item, 32 per lane pass
// ~64 ns per poll: about a quarter of a second before a block gives up
constexpr unsigned kBarrierPolls = 1u << 22;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of a cooperative launch (every block is resident).  The
// generation is read before arriving, the last block to arrive resets the
// count and advances the generation.  Returns false (and records the
// timeout) when the generation did not advance within kBarrierPolls polls.
__device__ bool grid_barrier(StepSync *sy, DevStatus *st) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = ld_acquire(&sy->gen);
        __threadfence();
        if (atomicAdd(&sy->arrive, 1u) == gridDim.x - 1) {
            atomicExch(&sy->arrive, 0u);
            __threadfence();
            atomicAdd(&sy->gen, 1u);
        } else {
            for (unsigned it = 0; ld_acquire(&sy->gen) == g; it++) {
                if (it >= kBarrierPolls) {
                    atomicOr(&st->error, (unsigned)GM_DEV_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// A 64-term block of bonded terms (or 1-4 pairs) by one warp, two terms a
// lane, with the energy partial and the per-system energies of term_block
// (gm_force.cu): lane l holds terms l and l + 32, and the shuffle-down tree
// adds in the order of its shared-memory tree, so the partial has the same
// bits.
template <bool MI, bool P14>
__device__ __forceinline__ void term_block_warp(const ForceArgs &fa, int blk, int lane, unsigned &bad) {
    int f0 = -1, f1 = -1;
    const int t = blk * GM_BONDED_THREADS + lane;
    const double e0 = P14 ? pair14_term<MI>(fa, t, bad, f0) : bonded_term<MI>(fa, t, bad, f0);
    const double e1 = P14 ? pair14_term<MI>(fa, t + 32, bad, f1) : bonded_term<MI>(fa, t + 32, bad, f1);
    if (fa.e_sys) {
        gm_add_sys_energy(fa.e_sys, f0 >= 0 ? fa.atom_sys[f0] : -1, e0);
        gm_add_sys_energy(fa.e_sys, f1 >= 0 ? fa.atom_sys[f1] : -1, e1);
    }
    double v = e0 + e1;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0 && blk < (P14 ? fa.blocks14 : fa.bonded_blocks)) (P14 ? fa.epart14 : fa.epart_bonded)[blk] = v;
}

// STEP: one BAB step (phases 1-3 above, a cooperative launch).  !STEP: phase
// 1 alone with energies (the pair items' partials, the 64-term blocks'
// partials and the per-system energies of the force kernels, the same bits),
// a plain launch; its last warp clears the queue words.
template <bool PERIODIC, bool COULOMB, bool BATCH, bool MI, bool STEP>
__global__ void __launch_bounds__(kStepThreads, kStepMinBlocks)
step_persistent_kernel(ForceArgs fa, StepArgs sa, PackArgs pk) {
    extern __shared__ float4 s_tab[];
    DevStatus *st = fa.status;
    StepSync *sy = sa.sync;
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    // read by every block before the barrier; block 0 clears it after
    const bool fresh = STEP && sy->fresh != 0;
    // ---- 1. forces at the current positions
    if (!fresh) {
        if (!BATCH) {
            for (int t = threadIdx.x; t < fa.ntypes * fa.ntypes; t += blockDim.x) s_tab[t] = fa.tab32[t];
            __syncthreads();
        }
        // tickets: n_pair pair items and nbw bonded tickets (kTermsPerTicket
        // bonded terms or 1-4 pairs each), the bonded ones at t = k * stride
        const int n_pair = fa.n_groups * fa.split;
        const int cb = (fa.n_bonds + fa.n_angles + fa.n_diheds + kTermsPerTicket - 1) / kTermsPerTicket;
        const int c14 = (fa.n14 + kTermsPerTicket - 1) / kTermsPerTicket;
        const int nbw = cb + c14, total = n_pair + nbw;
        const int stride = nbw > 0 ? total / nbw : 1;
        for (;;) {
            int t = 0;
            if (lane == 0) t = (int)atomicAdd(&sy->ticket, 1u);
            t = __shfl_sync(full, t, 0);
            if (t >= total) break;
            const int q = t / stride, r = t - q * stride;
            if (r == 0 && q < nbw) {
                unsigned bad = 0;
                const bool b14 = q >= cb;
                if (STEP) {
                    int first = -1;
                    const int base = (b14 ? q - cb : q) * kTermsPerTicket + lane;
                    for (int u = 0; u < kTermsPerTicket; u += 32) {
                        if (b14) pair14_term<MI>(fa, base + u, bad, first);
                        else bonded_term<MI>(fa, base + u, bad, first);
                    }
                } else {
                    const int blk0 = (b14 ? q - cb : q) * (kTermsPerTicket / GM_BONDED_THREADS);
                    for (int h = 0; h < kTermsPerTicket / GM_BONDED_THREADS; h++) {
                        if (b14) term_block_warp<MI, true>(fa, blk0 + h, lane, bad);
                        else term_block_warp<MI, false>(fa, blk0 + h, lane, bad);
                    }
                }
                bad = __reduce_or_sync(full, bad);
                if (bad && lane == 0) atomicOr(&st->error, bad);
            } else {
                // bonded tickets at or before t: min(q + 1, nbw)
                const int item = t - min(q + 1, nbw);
                pair_item_mixed<PERIODIC, COULOMB, BATCH, !STEP>(
                    item, lane, fa.n, fa.cap, fa.split, fa.coord, fa.perm, fa.list, fa.count, fa.gmax, fa.ntypes,
                    fa.tab32, s_tab, fa.pc, fa.force, fa.epart, st, fa.group_sys, STEP ? nullptr : fa.e_sys);
            }
        }
    }
    if (!STEP) {
        // the last warp out leaves the queue words at zero for the next launch
        if (lane == 0) {
            __threadfence();
            const unsigned warps = gridDim.x * (blockDim.x / 32);
            if (atomicAdd(&sy->arrive, 1u) == warps - 1) {
                atomicExch(&sy->ticket, 0u);
                atomicExch(&sy->arrive, 0u);
            }
        }
        return;
    }
    // ---- 2. every force is summed
    if (!grid_barrier(sy, st)) return;
    // ---- 3. kick, drift, pack, rebuild check (kick_drift_check_kernel's
    // operations, one atom at a time)
    const bool err0 = ld_acquire(&st->error) != 0, tail0 = ld_acquire(&st->tail_pending) != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sy->ticket = 0;
        sy->fresh = 0;
    }
    const int n = sa.n;
    int need = 0, bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double np[3];
        if (!err0) {
            const double inv_m = sa.inv_mass[i];
            for (int d = 0; d < 3; d++) {
                const double f = __dmul_rn((double)__ldcg(fa.force + d * n + i), GM_FIX_INV);
                const double kick = __dmul_rn(__dmul_rn(__dmul_rn(sa.dt_half, f), inv_m), GM_FORCE_TO_ACCEL);
                double v = sa.vel[d * n + i];
                if (tail0) v = __dadd_rn(v, kick);
                v = __dadd_rn(v, kick);
                const double p = sa.pos[d * n + i];
                sa.dref[d * n + i] = p;
                np[d] = __dadd_rn(p, __dmul_rn(sa.dt, v));
                sa.pos[d * n + i] = np[d];
                sa.vel[d * n + i] = gm_div_by_dt(__dsub_rn(np[d], p), sa.dt, sa.inv_dt);
            }
        } else {
            for (int d = 0; d < 3; d++) np[d] = sa.pos[d * n + i];
        }
        const int sl = pk.slot_of[i];
        const GridInfo *g = pk.grid + sa.atom_sys[i];
        gm_pack_record(pk.coord + 2 * sl, __dsub_rn(np[0], g->origin[0]), __dsub_rn(np[1], g->origin[1]),
                       __dsub_rn(np[2], g->origin[2]), pk.qw[i]);
        for (int d = 0; d < 3; d++) fa.force[d * n + i] = 0;
        bad |= !(isfinite(np[0]) && isfinite(np[1]) && isfinite(np[2]));
        const double dx = __dsub_rn(np[0], sa.ref[i]), dy = __dsub_rn(np[1], sa.ref[n + i]),
                     dz = __dsub_rn(np[2], sa.ref[2 * n + i]);
        const bool moved = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)) > sa.thr_sq;
        if (moved) {
            sa.sys_flag[sa.atom_sys[i]] = 1u;
            need = 1;
        }
    }
    need = __syncthreads_or(need);
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        if (need) atomicOr(&st->rebuild, 1u);
        if (bad) atomicOr(&st->bad_pending, 1u);
        __threadfence();
        const unsigned done = atomicAdd(&st->blocks_done, 1u);
        if (done == gridDim.x - 1) {
            __threadfence();
            const unsigned r = atomicOr(&st->rebuild, 0u);
            st->blocks_done = 0;
            if (atomicExch(&st->bad_pending, 0u)) atomicOr(&st->error, (unsigned)GM_DEV_NONFINITE_POS);
            const unsigned e = atomicOr(&st->error, 0u);
            if (sa.cond) cudaGraphSetConditional((cudaGraphConditionalHandle)sa.cond, (r && !e) ? 1u : 0u);
            if (!err0) {
                if (tail0) st->step += 1;
                st->tail_pending = 1u;
            }
        }
    }
}

using StepKernel = void (*)(ForceArgs, StepArgs, PackArgs);

template <bool STEP>
StepKernel pick(const ForceArgs &fa, bool gtab) {
#define GM_STEPK(P, Q, B, M) return step_persistent_kernel<P, Q, B, M, STEP>
#define GM_STEPB(P, Q, M) { if (gtab) GM_STEPK(P, Q, true, M); else GM_STEPK(P, Q, false, M); }
#define GM_STEPQ(P, M) { if (fa.coulomb) GM_STEPB(P, true, M) else GM_STEPB(P, false, M) }
    if (fa.bonded_mi) GM_STEPQ(true, true)
    if (fa.periodic) GM_STEPQ(true, false)
    GM_STEPQ(false, false)
#undef GM_STEPQ
#undef GM_STEPB
#undef GM_STEPK
}

// A batch reads its [system][type][type] tables through L1, as does a single
// system whose table passes 48 KB.
bool global_table(const ForceArgs &fa) {
    return fa.e_sys != nullptr || sizeof(float4) * (size_t)fa.ntypes * fa.ntypes > 48 * 1024;
}

}  // namespace

int gm_step_persistent_blocks(const ForceArgs &fa) {
    const bool gtab = global_table(fa);
    const size_t smem = gtab ? 0 : sizeof(float4) * (size_t)fa.ntypes * fa.ntypes;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pick<true>(fa, gtab), kStepThreads, smem) != cudaSuccess)
        return 0;
    return per_sm * sms;
}

void gm_launch_step_persistent(const ForceArgs &fa, const StepArgs &sa, const PackArgs &pk, int blocks,
                               cudaStream_t s) {
    const bool gtab = global_table(fa);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(kStepThreads);
    cfg.dynamicSmemBytes = gtab ? 0 : sizeof(float4) * (size_t)fa.ntypes * fa.ntypes;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, pick<true>(fa, gtab), fa, sa, pk);
}

void gm_launch_forces_persistent(const ForceArgs &fa, StepSync *sync, int blocks, cudaStream_t s) {
    const bool gtab = global_table(fa);
    StepArgs sa{};
    sa.sync = sync;
    PackArgs pk{};
    const size_t smem = gtab ? 0 : sizeof(float4) * (size_t)fa.ntypes * fa.ntypes;
    pick<false>(fa, gtab)<<<blocks, kStepThreads, smem, s>>>(fa, sa, pk);
}
