// gm_force.cu — force and energy kernels.
//
// Nonbonded (force/nonbonded.rs:20-82 physics): one lane per cell-sorted atom
// i walks its own column of the symmetric neighbour list, gathers each j's
// (hi, lo) record, one 32-byte sector, with one 256-bit load through the
// read-only path (four entries' gathers in flight before their arithmetic)
// and accumulates the force on i only, so no atomics are needed per pair and
// every atom's sum has a fixed order.  In mixed precision the pair arithmetic
// is double-float on the FP32 pipe (pair_kernel_mixed); per-lane sums over
// chunks of 32 entries are folded into int64 fixed point (2^-40 kcal/mol/A),
// and the energy into FP64.  Each pair is evaluated by both of its atoms (the
// list is symmetric), the energy total is halved.
// Bonded terms (force/bonded.rs) and the scaled 1-4 pairs use one thread per
// term, FP64 arithmetic in both precisions, and int64 atomics; integer
// addition is associative, so the result is run-to-run identical.
#include "gm_force_terms.cuh"

namespace {

constexpr double kCoulomb64 = 332.0522173;

// Mixed-precision nonbonded kernel: warps stride over the work items
// (pair_item_mixed); a grid smaller than the work makes it persistent, every
// item is computed the same either way.  A single system keeps its type table
// in shared memory; a batch reads its [system][type][type] tables through L1.
template <bool PERIODIC, bool COULOMB, bool BATCH, int W>
__global__ void __launch_bounds__(W * 32)
pair_kernel_mixed(int n, int n_slots, int cap, int split, const float4 *__restrict__ coord,
                  const int *__restrict__ perm, const int *__restrict__ list, const int *__restrict__ count,
                  const int *__restrict__ gmax, int ntypes, const float4 *__restrict__ tab, PairConst k,
                  long long *__restrict__ force, double *__restrict__ epart, DevStatus *st,
                  const int *__restrict__ group_sys, long long *e_sys) {
    extern __shared__ float4 s_tab[];
    if (!BATCH) {
        for (int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x) s_tab[t] = tab[t];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int n_work = (n_slots / 32) * split;
    for (int wid = blockIdx.x * W + (threadIdx.x >> 5); wid < n_work; wid += gridDim.x * W)
        pair_item_mixed<PERIODIC, COULOMB, BATCH>(wid, lane, n, cap, split, coord, perm, list, count, gmax, ntypes,
                                                  tab, s_tab, k, force, epart, st, group_sys, e_sys);
}

// FP64 nonbonded kernel (the FP64 path): the reference's arithmetic
// (force/nonbonded.rs:20-82) in FP64 on the sorted FP64 copies.  The same
// work split as the mixed kernel (a 32-atom group's columns over `split`
// warps, 2/4/8 warps per block, optional persistent grid), and the same
// summation: FP64 sums over chunks of 32 entries folded into int64, so every
// launch shape gives the same bits.
template <bool PERIODIC, bool COULOMB, bool BATCH, int W>
__global__ void __launch_bounds__(W * 32)
pair_kernel_f64(int n, int n_slots, int cap, int split, const double4 *__restrict__ p64,
                const int *__restrict__ type_s, const int *__restrict__ perm, const int *__restrict__ list,
                const int *__restrict__ count, const int *__restrict__ gmax, int ntypes,
                const double2 *__restrict__ tab, double rc2, double rsw, double rc, double bx, double by, double bz,
                long long *__restrict__ force, double *__restrict__ epart, DevStatus *st,
                const int *__restrict__ group_sys, long long *e_sys) {
    extern __shared__ double2 s_tab64[];
    if (!BATCH) {
        for (int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x) s_tab64[t] = tab[t];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const double wsw = rc - rsw;
    const int n_work = (n_slots / 32) * split;
    for (int wid = blockIdx.x * W + (threadIdx.x >> 5); wid < n_work; wid += gridDim.x * W) {
    const int group = wid / split, part = wid - group * split;
    const int s = group * 32 + lane;
    const int atom = perm[s];  // -1 on a padding slot
    const bool valid = atom >= 0;
    double4 mi = make_double4(0, 0, 0, 0);
    int cnt = 0, ti = 0;
    if (valid) { mi = p64[s]; cnt = count[s]; ti = type_s[s]; }
    const double2 *trow = (BATCH ? tab + (size_t)group_sys[group] * ntypes * ntypes : s_tab64) + ti * ntypes;
    const double qi = mi.w * kCoulomb64;
    const int gm = gmax[group];
    const int per = ((gm + split - 1) / split + kChunk - 1) / kChunk * kChunk;
    const int e_begin = part * per, e_end = min(gm, e_begin + per);
    const int *L = list + (size_t)group * 32 * cap + lane;
    long long ax = 0, ay = 0, az = 0;
    double eacc = 0.0;
    unsigned int bad = 0;
    for (int e0 = e_begin; e0 < e_end; e0 += kChunk) {
        double fx = 0, fy = 0, fz = 0;
        const int e1 = min(e0 + kChunk, min(e_end, cnt));
        for (int e = e0; e < e1; e++) {
            const int j = __ldg(L + (size_t)e * 32);
            const double4 pj = p64[j];
            double dx = pj.x - mi.x, dy = pj.y - mi.y, dz = pj.z - mi.z;
            if (PERIODIC) {
                dx = gm_min_image(dx, bx);
                dy = gm_min_image(dy, by);
                dz = gm_min_image(dz, bz);
            }
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > rc2 || r2 == 0.0) continue;
            const double r = sqrt(r2);
            const double rinv = 1.0 / r;
            const double2 p = trow[type_s[j]];
            double v = 0.0, fr = 0.0;  // fr = F_r (radial magnitude)
            if (p.y != 0.0) {
                const double sr = p.x * rinv;
                const double s2 = sr * sr, s4 = s2 * s2, s6 = s2 * s4, s12 = s6 * s6;
                v = 4.0 * p.y * (s12 - s6);
                fr = 24.0 * p.y * rinv * (2.0 * s12 - s6);
            }
            if (COULOMB) {
                const double vc = qi * pj.w * rinv;
                v += vc;
                fr += vc * rinv;
            }
            if (r > rsw) {
                const double u = (r - rsw) / wsw;
                const double u2 = u * u;
                const double sw = 1.0 - 10.0 * u2 * u + 15.0 * u2 * u2 - 6.0 * u2 * u2 * u;
                const double dsw = -30.0 * u2 * (1.0 - u) * (1.0 - u) / wsw;
                fr = fr * sw - v * dsw;
                v *= sw;
            }
            const double g = fr * rinv;
            fx -= g * dx;
            fy -= g * dy;
            fz -= g * dz;
            eacc += v;
        }
        ax += gm_to_fix_checked(fx, bad);
        ay += gm_to_fix_checked(fy, bad);
        az += gm_to_fix_checked(fz, bad);
    }
    if (valid && e_begin < e_end) {
        gm_atomic_fix_add(force + atom, ax);
        gm_atomic_fix_add(force + n + atom, ay);
        gm_atomic_fix_add(force + 2 * n + atom, az);
    }
    for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
    if (lane == 0) epart[wid] = 0.5 * eacc;
    if (e_sys && lane == 0) gm_atomic_fix_add(e_sys + group_sys[group], __double2ll_rn(0.5 * eacc * GM_EFIX_SCALE));
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && lane == 0) atomicOr(&st->error, bad);
    }
}

// One block of GM_BONDED_THREADS bonded terms (or 1-4 pairs) with a
// fixed-order block reduction of the energy into its partial.
template <bool MI, bool P14>
__device__ __forceinline__ void term_block(const ForceArgs &a, int blk) {
    const int t = blk * blockDim.x + threadIdx.x;
    unsigned bad = 0;
    int first = -1;
    const double e = P14 ? pair14_term<MI>(a, t, bad, first) : bonded_term<MI>(a, t, bad, first);
    __shared__ double se[GM_BONDED_THREADS];
    se[threadIdx.x] = e;
    __syncthreads();
    for (int s2 = GM_BONDED_THREADS / 2; s2 > 0; s2 >>= 1) {
        if (threadIdx.x < s2) se[threadIdx.x] += se[threadIdx.x + s2];
        __syncthreads();
    }
    if (threadIdx.x == 0) (P14 ? a.epart14 : a.epart_bonded)[blk] = se[0];
    if (a.e_sys) gm_add_sys_energy(a.e_sys, first >= 0 ? a.atom_sys[first] : -1, e);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(&a.status->error, bad);
}
template <bool MI>
__device__ __forceinline__ void bonded_block(const ForceArgs &a, int blk) { term_block<MI, false>(a, blk); }
template <bool MI>
__device__ __forceinline__ void pair14_block(const ForceArgs &a, int blk) { term_block<MI, true>(a, blk); }

template <bool MI>
__global__ void __launch_bounds__(GM_BONDED_THREADS) bonded_kernel(ForceArgs a) { bonded_block<MI>(a, blockIdx.x); }
template <bool MI>
__global__ void __launch_bounds__(GM_BONDED_THREADS) pair14_kernel(ForceArgs a) { pair14_block<MI>(a, blockIdx.x); }
// Both in one persistent launch: the grid strides over the virtual blocks
// of GM_BONDED_THREADS terms, the first bonded_blocks of them bonded terms,
// the rest 1-4 pairs (independent work; integer force sums; each virtual
// block writes its own energy partial, so the grid size changes no bits).
template <bool MI>
__global__ void __launch_bounds__(GM_BONDED_THREADS) bonded_pair14_kernel(ForceArgs a) {
    const int total = a.bonded_blocks + a.blocks14;
    for (int vb = blockIdx.x; vb < total; vb += gridDim.x) {
        if (vb < a.bonded_blocks) bonded_block<MI>(a, vb);
        else pair14_block<MI>(a, vb - a.bonded_blocks);
    }
}

// Fixed-order sum of all energy partials (pair groups, bonded blocks, 1-4
// blocks) into the FP64 total: deterministic for a given launch shape.
__global__ void __launch_bounds__(256) energy_kernel(const double *epart, int n, double *out) {
    __shared__ double s[256];
    const double e = gm_block_sum256(epart, n, s);
    if (threadIdx.x == 0) *out = e;
}

}  // namespace

int gm_bonded_blocks(int nb, int na, int nd) {
    const long long t = (long long)nb + na + nd;
    return (int)((t + GM_BONDED_THREADS - 1) / GM_BONDED_THREADS);
}

void gm_launch_pair(const ForceArgs &a, bool fp64, cudaStream_t s) {
    if (a.n == 0) return;
    const bool batch = a.e_sys != nullptr;
    if (!fp64) {
        const int W = a.pair_warps == 2 || a.pair_warps == 8 ? a.pair_warps : 4;
        int blocks32 = (a.n_groups * a.split + W - 1) / W;
        if (a.pair_grid > 0 && a.pair_grid < blocks32) blocks32 = a.pair_grid;
        // a table past 48 KB is read through L1 like a batch's tables (a
        // single system's group_sys is all zero)
        const size_t tab_bytes = sizeof(float4) * (size_t)a.ntypes * a.ntypes;
        const bool gtab = batch || tab_bytes > 48 * 1024;
        const size_t smem = gtab ? 0 : tab_bytes;
#define GM_PAIRMW(P, Q, B, WW)                                                                              \
    pair_kernel_mixed<P, Q, B, WW><<<blocks32, WW * 32, smem, s>>>(                                          \
        a.n, a.n_slots, a.cap, a.split, a.coord, a.perm, a.list, a.count, a.gmax, a.ntypes, a.tab32, a.pc,    \
        a.force, a.epart, a.status, a.group_sys, a.e_sys)
#define GM_PAIRM(P, Q, B) { if (W == 2) GM_PAIRMW(P, Q, B, 2); else if (W == 8) GM_PAIRMW(P, Q, B, 8); \
                            else GM_PAIRMW(P, Q, B, 4); }
#define GM_PAIRMB(P, Q) { if (gtab) GM_PAIRM(P, Q, true) else GM_PAIRM(P, Q, false) }
        if (a.periodic) { if (a.coulomb) GM_PAIRMB(true, true) else GM_PAIRMB(true, false) }
        else { if (a.coulomb) GM_PAIRMB(false, true) else GM_PAIRMB(false, false) }
#undef GM_PAIRMB
#undef GM_PAIRM
#undef GM_PAIRMW
    } else {
        const int W = a.pair_warps == 2 || a.pair_warps == 8 ? a.pair_warps : 4;
        int blocks64 = (a.n_groups * a.split + W - 1) / W;
        if (a.pair_grid > 0 && a.pair_grid < blocks64) blocks64 = a.pair_grid;
        const size_t tab_bytes = sizeof(double2) * (size_t)a.ntypes * a.ntypes;
        const bool gtab = batch || tab_bytes > 48 * 1024;
        const size_t smem = gtab ? 0 : tab_bytes;
#define GM_PAIR64W(P, Q, B, WW)                                                                                   \
    pair_kernel_f64<P, Q, B, WW><<<blocks64, WW * 32, smem, s>>>(                                                  \
        a.n, a.n_slots, a.cap, a.split, a.pos64s, a.type_sorted, a.perm, a.list, a.count, a.gmax, a.ntypes, a.tab64, \
        a.rc2_64, a.rsw_64, a.rc_64, a.box64[0], a.box64[1], a.box64[2], a.force, a.epart, a.status, a.group_sys, \
        a.e_sys)
#define GM_PAIR64(P, Q, B) { if (W == 2) GM_PAIR64W(P, Q, B, 2); else if (W == 8) GM_PAIR64W(P, Q, B, 8); \
                             else GM_PAIR64W(P, Q, B, 4); }
#define GM_PAIR64B(P, Q) { if (gtab) GM_PAIR64(P, Q, true) else GM_PAIR64(P, Q, false) }
        if (a.periodic) { if (a.coulomb) GM_PAIR64B(true, true) else GM_PAIR64B(true, false) }
        else { if (a.coulomb) GM_PAIR64B(false, true) else GM_PAIR64B(false, false) }
#undef GM_PAIR64B
#undef GM_PAIR64
#undef GM_PAIR64W
    }
}

// The bonded and 1-4 kernels are FP64 in both precisions (fp64 selects the
// pair kernel only).
void gm_launch_bonded(const ForceArgs &a, bool, cudaStream_t s) {
    if (a.bonded_blocks == 0) return;
    if (a.bonded_mi) bonded_kernel<true><<<a.bonded_blocks, GM_BONDED_THREADS, 0, s>>>(a);
    else bonded_kernel<false><<<a.bonded_blocks, GM_BONDED_THREADS, 0, s>>>(a);
}

// The bonded / 1-4 kernel runs beside the pair kernel on a second stream:
// two small blocks per SM (persistent), launched at the device's highest
// priority, so that every SM keeps its FP64 pipe busy with these terms while
// the registers the blocks leave free hold the pair kernel's blocks (FP32).
// Measured on the 50k system (one graph step): one block per SM 0.227 ms,
// two 0.223 ms, four 0.227 ms, one block per 64 terms 0.248 ms.
void gm_launch_bonded_pair14(const ForceArgs &a, bool, cudaStream_t s) {
    const int blocks = a.bonded_blocks + a.blocks14;
    if (blocks == 0) return;
    static int prio = [] {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        return greatest;
    }();
    static int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(blocks < 2 * sms ? blocks : 2 * sms));
    cfg.blockDim = dim3(GM_BONDED_THREADS);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = prio;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (a.bonded_mi) cudaLaunchKernelEx(&cfg, bonded_pair14_kernel<true>, a);
    else cudaLaunchKernelEx(&cfg, bonded_pair14_kernel<false>, a);
}

void gm_launch_pair14(const ForceArgs &a, bool, cudaStream_t s) {
    if (a.blocks14 == 0) return;
    if (a.bonded_mi) pair14_kernel<true><<<a.blocks14, GM_BONDED_THREADS, 0, s>>>(a);
    else pair14_kernel<false><<<a.blocks14, GM_BONDED_THREADS, 0, s>>>(a);
}

void gm_launch_energy(const ForceArgs &a, cudaStream_t s) {
    energy_kernel<<<1, 256, 0, s>>>(a.epart, a.n_epart_total, a.energy);
}
