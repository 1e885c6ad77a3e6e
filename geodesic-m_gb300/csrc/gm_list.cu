// gm_list.cu — Verlet list build on the device (neighbor.rs:8-55 semantics),
// for one system or a batch of independent systems in one context.
//
// Pipeline at each rebuild (all on the context's stream, no host sync):
//   wrap (periodic only) -> bbox partials -> grid setup -> cell assignment +
//   counting-sort histogram -> scan -> scatter -> in-cell rank by caller
//   index (deterministic order) -> pack -> list build.
// Every kernel runs over all systems at once (blockIdx.y = system) and skips
// the systems whose rebuild flag is clear, so a batch rebuilds only the
// systems that need it.  Each system owns a range of atoms, a 32-aligned
// range of sorted slots (padding slots have perm = -1 and no list), a range
// of cells and its own grid; perm and the list entries hold global indices.
// The list build gives each warp 32 consecutive cell-sorted atoms of one
// system and one z layer of their candidate cell box (five warps per group,
// each filling its own list segment); the warp streams the candidates of
// each cell row of its layer through shared memory and each lane tests them
// against its own atom.  The
// test runs in FP32 on hi+lo coordinates; candidates within `margin` of the
// list radius are re-decided with the reference's exact FP64 expression
// (min-image, then dx*dx + dy*dy + dz*dz, no fused multiply-add), so the pair
// set equals the reference's bit for bit.
#include <algorithm>
#include <cfloat>
#include <climits>

#include "gm_internal.cuh"

namespace {


__device__ __forceinline__ double exact_min_image(double d, double L) {
    // neighbor.rs:74-76: d - L * round(d / L), no contraction
    return __dsub_rn(d, __dmul_rn(L, round(__ddiv_rn(d, L))));
}

__device__ __forceinline__ double exact_wrap(double x, double L) {
    // neighbor.rs:86-88: x - L * floor(x / L)
    return __dsub_rn(x, __dmul_rn(L, floor(__ddiv_rn(x, L))));
}

// Atom range of system blockIdx.y, or false when it keeps its list.
__device__ __forceinline__ bool sys_atoms(const ListArgs &a, int &a0, int &a1) {
    const int s = blockIdx.y;
    if (!a.sys_flag[s]) return false;
    a0 = a.sys_atom_off[s];
    a1 = a.sys_atom_off[s + 1];
    return true;
}

__global__ void set_flags_kernel(ListArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_sys) a.sys_flag[s] = 1u;
}

__global__ void clear_flags_kernel(ListArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_sys) a.sys_flag[s] = 0u;
    if (s == 0) a.status->rebuild = 0u;
}

__global__ void wrap_kernel(ListArgs a, double *pos) {
    int a0, a1;
    if (!sys_atoms(a, a0, a1)) return;
    const int n = a.n;
    for (int i = a0 + blockIdx.x * blockDim.x + threadIdx.x; i < a1; i += gridDim.x * blockDim.x) {
        pos[i] = exact_wrap(pos[i], a.box[0]);
        pos[n + i] = exact_wrap(pos[n + i], a.box[1]);
        pos[2 * n + i] = exact_wrap(pos[2 * n + i], a.box[2]);
    }
}

// Partial-sum blocks of a system's bbox: as many as a context holding only
// that system uses, so a system's grid (and its FP32 copies) come out the
// same alone or in a batch.
__device__ __forceinline__ int bbox_blocks_of(int n_atoms, int cap) {
    const int b = (n_atoms + 255) / 256;
    return b < 1 ? 1 : (b > cap ? cap : b);
}

// Per block and system: min x,y,z, max x,y,z and the sum x,y,z.
__global__ void bbox_kernel(ListArgs a) {
    __shared__ double sm[9][256];
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX}, sum[3] = {0, 0, 0};
    int a0, a1;
    if (!sys_atoms(a, a0, a1)) return;  // uniform per block
    const int nb = bbox_blocks_of(a1 - a0, 256);
    if ((int)blockIdx.x >= nb) return;
    const int n = a.n;
    for (int i = a0 + blockIdx.x * blockDim.x + threadIdx.x; i < a1; i += nb * blockDim.x) {
        for (int d = 0; d < 3; d++) {
            double v = a.pos[d * n + i];
            mn[d] = fmin(mn[d], v);
            mx[d] = fmax(mx[d], v);
            if (v == v) sum[d] += v;
        }
    }
    for (int d = 0; d < 3; d++) {
        sm[d][threadIdx.x] = mn[d];
        sm[3 + d][threadIdx.x] = mx[d];
        sm[6 + d][threadIdx.x] = sum[d];
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int d = 0; d < 3; d++) {
                sm[d][threadIdx.x] = fmin(sm[d][threadIdx.x], sm[d][threadIdx.x + s]);
                sm[3 + d][threadIdx.x] = fmax(sm[3 + d][threadIdx.x], sm[3 + d][threadIdx.x + s]);
                sm[6 + d][threadIdx.x] += sm[6 + d][threadIdx.x + s];
            }
        __syncthreads();
    }
    if (threadIdx.x < 9)
        a.bbox_scratch[((size_t)blockIdx.y * a.bbox_blocks + blockIdx.x) * 9 + threadIdx.x] = sm[threadIdx.x][0];
}

// One block per system: reduce its bbox partials, then lay out its grid.
__global__ void grid_kernel(ListArgs a, int blocks) {
    const int sys = blockIdx.x;
    if (!a.sys_flag[sys]) return;
    __shared__ double red[9][256];
    const double *partial = a.bbox_scratch + (size_t)sys * blocks * 9;
    const int nb = a.periodic ? 0 : bbox_blocks_of(a.sys_atom_off[sys + 1] - a.sys_atom_off[sys], 256);
    for (int v = 0; v < 9; v++) {
        double acc = v < 3 ? DBL_MAX : (v < 6 ? -DBL_MAX : 0.0);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const double x = partial[b * 9 + v];
            acc = v < 3 ? fmin(acc, x) : (v < 6 ? fmax(acc, x) : acc + x);
        }
        red[v][threadIdx.x] = acc;
    }
    __syncthreads();
    __shared__ int s_ncell;
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k)
            for (int v = 0; v < 9; v++) {
                const double x = red[v][threadIdx.x + k];
                red[v][threadIdx.x] = v < 3 ? fmin(red[v][threadIdx.x], x)
                                            : (v < 6 ? fmax(red[v][threadIdx.x], x) : red[v][threadIdx.x] + x);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
    GridInfo *g = a.grid + sys;
    const int n_atoms = a.sys_atom_off[sys + 1] - a.sys_atom_off[sys];
    const int max_cells = a.sys_cell_off[sys + 1] - a.sys_cell_off[sys] - 1;
    const double box[3] = {a.box[0], a.box[1], a.box[2]};
    const double wmin = a.r_list * 0.5 * (1.0 + 1e-5) + 1e-6;
    int nc[3];
    double w[3], lo[3];
    g->periodic = a.periodic;
    for (int d = 0; d < 3; d++) {
        g->box[d] = (float)box[d];
        g->inv_box[d] = (float)(1.0 / box[d]);
    }
    if (a.periodic) {
        for (int d = 0; d < 3; d++) {
            nc[d] = (int)floor(box[d] / wmin);
            if (nc[d] < 1) nc[d] = 1;
            g->origin[d] = 0.5 * box[d];
            lo[d] = -0.5 * box[d];
        }
    } else {
        double mn[3], mx[3], sum[3];
        for (int d = 0; d < 3; d++) { mn[d] = red[d][0]; mx[d] = red[3 + d][0]; sum[d] = red[6 + d][0]; }
        // The grid covers a core cube around the mean position, at the finest
        // cell width the allocation allows; atoms outside it (evaporated atoms
        // of a droplet in vacuum) are clamped into the edge cells.  Clamping is
        // 1-Lipschitz on cell indices, so the 5x5x5 stencil still finds every
        // pair, and a few outliers no longer coarsen the whole grid.
        const int per_dim = (int)floor(cbrt((double)max_cells));
        for (int d = 0; d < 3; d++) {
            double ext = mx[d] - mn[d];
            if (!(ext == ext) || mx[d] < mn[d]) { ext = 0.0; mn[d] = mx[d] = 0.0; sum[d] = 0.0; }
            // min-image of the reference folds pairs farther apart than box/2;
            // the cell search assumes it never does
            if (ext + a.r_list >= 0.5 * box[d]) atomicOr(&a.status->error, (unsigned)GM_DEV_EXTENT);
            const double mean = n_atoms > 0 ? sum[d] / n_atoms : 0.0;
            const double half = 0.5 * per_dim * wmin;
            double lo_c = fmax(mn[d], mean - half), hi_c = fmin(mx[d], mean + half);
            if (!(hi_c >= lo_c)) { lo_c = mn[d]; hi_c = mx[d]; }
            const double pad = 1e-3 * (1.0 + (hi_c - lo_c));
            g->origin[d] = 0.5 * (lo_c + hi_c);
            lo[d] = (lo_c - g->origin[d]) - pad;
            nc[d] = (int)floor((hi_c - lo_c + 2.0 * pad) / wmin);
            if (nc[d] < 1) nc[d] = 1;
        }
    }
    // keep the cell count within the allocation by coarsening the grid
    // (coarser cells only widen the 5x5x5 search, never miss a pair)
    while ((long long)nc[0] * nc[1] * nc[2] > max_cells) {
        for (int d = 0; d < 3; d++) nc[d] = nc[d] > 1 ? (nc[d] * 3) / 4 : 1;
    }
    for (int d = 0; d < 3; d++) {
        double span = a.periodic ? box[d] : -2.0 * lo[d];
        w[d] = span / nc[d];
        g->nc[d] = nc[d];
        g->lo[d] = (float)lo[d];
        g->inv_w[d] = (float)(1.0 / w[d]);
        g->full[d] = a.periodic && nc[d] < 5;
    }
    g->ncell = nc[0] * nc[1] * nc[2];  // <= max_cells by construction
    atomicAdd(&a.status->n_rebuilds, 1ull);
    s_ncell = min(g->ncell, max_cells);
    }
    // the cells the new grid uses (the only ones assign and the scan touch)
    __syncthreads();
    const int c0 = a.sys_cell_off[sys];
    for (int c = c0 + threadIdx.x; c < c0 + s_ncell; c += blockDim.x) {
        a.cell_count[c] = 0;
        a.cell_cursor[c] = 0;
    }
}


__device__ __forceinline__ int cell_coord(float h, float lo, float inv_w, int nc) {
    float t = floorf((h - lo) * inv_w);
    int c = (int)t;  // NaN converts to 0
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

__global__ void assign_kernel(ListArgs a) {
    int a0, a1;
    if (!sys_atoms(a, a0, a1)) return;
    const GridInfo *g = a.grid + blockIdx.y;
    const int coff = a.sys_cell_off[blockIdx.y];
    const int max_cells = a.sys_cell_off[blockIdx.y + 1] - coff - 1;
    const int n = a.n;
    for (int i = a0 + blockIdx.x * blockDim.x + threadIdx.x; i < a1; i += gridDim.x * blockDim.x) {
        int c3[3];
        for (int d = 0; d < 3; d++) {
            double x = a.pos[d * n + i];
            a.ref[d * n + i] = x;  // NeighborList::ref_{x,y,z} (neighbor.rs:48-50)
            c3[d] = cell_coord((float)(x - g->origin[d]), g->lo[d], g->inv_w[d], g->nc[d]);
        }
        int c = (c3[2] * g->nc[1] + c3[1]) * g->nc[0] + c3[0];
        if (c < 0 || c >= max_cells) {
            atomicOr(&a.status->error, (unsigned)GM_DEV_CELL_OVERFLOW);
            c = 0;
        }
        a.cell_of[i] = c;
        atomicAdd(&a.cell_count[coff + c], 1);
    }
}

// Exclusive scan of one value per thread over a block (a multiple of 32
// threads, at most 1024), with the block total.
__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        int t = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_sums[lane] = t;
    }
    __syncthreads();
    const int excl = x - v + (w > 0 ? warp_sums[w - 1] : 0);
    total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

__device__ __forceinline__ int sys_ncell(const ListArgs &a, int s) {
    const int max_cells = a.sys_cell_off[s + 1] - a.sys_cell_off[s] - 1;
    return min(a.grid[s].ncell, max_cells);
}

// Exclusive scan of each system's cell counts into cell_start[0..ncell], one
// block per system walking its cells in chunks of 4096 with a running carry
// (a few chunks for the grids of these systems).
__global__ void __launch_bounds__(1024) scan_cells_kernel(ListArgs a) {
    __shared__ int warp_sums[32];
    const int s = blockIdx.x;
    if (!a.sys_flag[s]) return;
    const int ncell = sys_ncell(a, s), coff = a.sys_cell_off[s];
    int carry = 0;
    for (int base = 0; base <= ncell; base += 4 * (int)blockDim.x) {
        const int i0 = base + 4 * (int)threadIdx.x;
        int v[4], sum = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[k] = i0 + k < ncell ? a.cell_count[coff + i0 + k] : 0;
            sum += v[k];
        }
        int total;
        int run = carry + block_exclusive_scan(sum, warp_sums, total);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (i0 + k <= ncell) a.cell_start[coff + i0 + k] = run;
            run += v[k];
        }
        carry += total;
    }
}



__global__ void scatter_kernel(ListArgs a) {
    int a0, a1;
    if (!sys_atoms(a, a0, a1)) return;
    const int coff = a.sys_cell_off[blockIdx.y], soff = a.sys_slot_off[blockIdx.y];
    for (int i = a0 + blockIdx.x * blockDim.x + threadIdx.x; i < a1; i += gridDim.x * blockDim.x) {
        const int c = a.cell_of[i];
        const int slot = a.cell_start[coff + c] + atomicAdd(&a.cell_cursor[coff + c], 1);
        a.tmp_atom[soff + slot] = i - a0;
    }
}

// Within a cell, atoms are ordered by caller index: the rank of an atom is
// the number of cell members with a smaller index.  Independent of the
// atomic order of the scatter, so the sorted layout is deterministic.
__global__ void rank_kernel(ListArgs a) {
    int a0, a1;
    if (!sys_atoms(a, a0, a1)) return;
    const int coff = a.sys_cell_off[blockIdx.y], soff = a.sys_slot_off[blockIdx.y];
    const int ns = a1 - a0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        const int at = a.tmp_atom[soff + k];
        const int c = a.cell_of[a0 + at];
        const int s0 = a.cell_start[coff + c], s1 = a.cell_start[coff + c + 1];
        if (s1 - s0 > 65536) {
            // no physical system packs this many atoms into one half cell; keep
            // the quadratic rank bounded and report it
            atomicOr(&a.status->error, (unsigned)GM_DEV_CELL_OVERFLOW);
            a.perm[soff + k] = a0 + at;
            a.cell_sorted[soff + k] = c;
            if (a.slot_of) a.slot_of[a0 + at] = soff + k;
            continue;
        }
        int rank = 0;
        for (int m = s0; m < s1; m++) rank += a.tmp_atom[soff + m] < at;
        a.perm[soff + s0 + rank] = a0 + at;
        a.cell_sorted[soff + s0 + rank] = c;
        if (a.slot_of) a.slot_of[a0 + at] = soff + s0 + rank;
    }
}

// Every slot of every system, every force evaluation: the slot records
// relative to the system's grid origin, and the force accumulators cleared.
__global__ void pack_kernel(ListArgs a, bool fp64) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n_slots) return;
    const int at = a.perm[s];
    if (at < 0) return;  // padding slot
    const int n = a.n;
    const GridInfo *g = a.grid + a.atom_sys[at];
    const double x = a.pos[at], y = a.pos[n + at], z = a.pos[2 * n + at];
    gm_pack_record(a.coord + 2 * s, x - g->origin[0], y - g->origin[1], z - g->origin[2], a.qw[at]);
    if (fp64) {
        a.pos64s[s] = make_double4(x, y, z, a.charge64[at]);
        a.type_sorted[s] = a.type[at];
    }
    a.force[at] = 0;
    a.force[n + at] = 0;
    a.force[2 * n + at] = 0;
}

struct Range { int lo, hi, nc, wrap; };

__device__ __forceinline__ Range dim_range(int mn, int mx, int nc, int periodic, int full) {
    Range r;
    r.nc = nc;
    if (full) { r.lo = 0; r.hi = nc - 1; r.wrap = 0; return r; }
    r.lo = mn - 2;
    r.hi = mx + 2;
    if (periodic) {
        if (r.hi - r.lo + 1 >= nc) { r.lo = 0; r.hi = nc - 1; r.wrap = 0; }
        else r.wrap = 1;
    } else {
        r.lo = r.lo < 0 ? 0 : r.lo;
        r.hi = r.hi >= nc ? nc - 1 : r.hi;
        r.wrap = 0;
    }
    return r;
}

__device__ __forceinline__ int wrapi(int c, int nc) { return c < 0 ? c + nc : (c >= nc ? c - nc : c); }

// FP32 squared distance of a staged candidate from the lane's atom (both
// relative to the group's first atom), with the periodic image; every
// product-sum is an explicit FMA, so the candidate test and the bucket of an
// accepted candidate see the same value.
template <bool PERIODIC>
__device__ __forceinline__ float rel_r2(float4 c, float mx, float my, float mz, const GridInfo &g) {
    float dx = c.x - mx, dy = c.y - my, dz = c.z - mz;
    if (PERIODIC) {
        dx = fmaf(-g.box[0], rintf(dx * g.inv_box[0]), dx);
        dy = fmaf(-g.box[1], rintf(dy * g.inv_box[1]), dy);
        dz = fmaf(-g.box[2], rintf(dz * g.inv_box[2]), dz);
    }
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// One block per group, one warp per z layer: warp `seg` tests the candidates
// of z layer `seg` of each row box its lanes need and stages them; the block
// then concatenates the layers into each lane's list column.
// Each lane's column is written in distance-bucket order (GM_NBUCKET buckets
// of the build-time distance, bounds in bucket_r2): inside the switch radius,
// the switch band, the shell beyond the cutoff.  Within a bucket the entries
// keep the single-warp sweep order.  The pair kernel's lanes then meet the
// same kind of pair at the same entry and branch together.
template <bool PERIODIC>
__global__ void __launch_bounds__(GM_NSEG * 32)
build_kernel(ListArgs a, float rl2_lo, float rl2_hi, double rl2_64, float3 bucket_r2) {
    // candidates of the current batch: coordinates relative to the group's
    // first atom (FP32; the rounding, under 1e-5 A for candidates within a
    // few list radii, stays far inside the FP64 re-decision margin) and
    // caller indices
    __shared__ float4 s_rel[GM_NSEG][32];
    __shared__ int s_orig[GM_NSEG][32];
    __shared__ int s_cnt[GM_NSEG][GM_NBUCKET][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int group = blockIdx.x, seg = wib;
    const int gseg = group * GM_NSEG + seg;
    if (group * 32 >= a.n_slots) return;
    const int sys = a.group_sys[group];
    if (!a.sys_flag[sys]) return;  // block-uniform: the system keeps its list
    // the unrolled candidate loop below reads all 32 staging entries
    s_rel[wib][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    s_orig[wib][lane] = 0;
    const int soff = a.sys_slot_off[sys], coff = a.sys_cell_off[sys];
    const int ns = a.sys_atom_off[sys + 1] - a.sys_atom_off[sys];
    const int s = group * 32 + lane;
    const bool valid = s - soff < ns;
    const GridInfo g = a.grid[sys];
    const int n = a.n;
    const int cap = a.cap;
    const int *__restrict__ cell_start = a.cell_start + coff;
    // the reference point: the group's first slot (always an atom: systems
    // start on a group boundary)
    float4 rh, rl;
    gm_ld_coord(a.coord + 2 * group * 32, rh, rl);
    float mx = 0.f, my = 0.f, mz = 0.f;
    int my_orig = -1, my_cell = 0;
    if (valid) {
        float4 mh, ml;
        gm_ld_coord(a.coord + 2 * s, mh, ml);
        mx = (mh.x - rh.x) + (ml.x - rl.x);
        my = (mh.y - rh.y) + (ml.y - rl.y);
        mz = (mh.z - rh.z) + (ml.z - rl.z);
        my_orig = a.perm[s];
        my_cell = a.cell_sorted[s];
    }
    // own exclusions (caller indices, ascending); up to 8 kept in registers
    int e0 = 0, e1 = 0;
    int ex[8];
    if (valid) { e0 = a.excl_start[my_orig]; e1 = a.excl_start[my_orig + 1]; }
    const int ne = e1 - e0;
#pragma unroll
    for (int k = 0; k < 8; k++) ex[k] = (k < ne) ? a.excl[e0 + k] : -1;
    // the exclusions span [ex_lo, ex_hi] in caller index: candidates outside
    // skip the scan
    const int ex_lo = ne > 0 ? ex[0] : INT_MAX, ex_hi = ne > 0 ? a.excl[e1 - 1] : INT_MIN;
    // Candidate regions, one per distinct cell row (cy, cz) among the lanes:
    // a group of 32 sorted atoms usually lies in one row of cells, sometimes
    // straddles the end of a row.  Sweeping each row's own 5 x 5 x (span + 4)
    // box keeps the regions tight (one box over both rows would cover the
    // whole row); a lane tests only the candidates of its own row's box, so
    // it never meets a candidate twice.  This warp takes z layer `seg` of
    // each box.
    const int cx = my_cell % g.nc[0], cy = (my_cell / g.nc[0]) % g.nc[1], cz = my_cell / (g.nc[0] * g.nc[1]);
    const int row_id = valid ? cz * g.nc[1] + cy : -1;
    const int cap_seg = a.cap_seg;
    int *my_stage = a.stage + (size_t)gseg * 32 * cap_seg + lane;
    int cnt = 0;
    int nb[GM_NBUCKET] = {0, 0, 0, 0};  // staged entries per bucket
    const double bx[3] = {a.box[0], a.box[1], a.box[2]};
    unsigned remaining = __ballot_sync(0xffffffffu, valid);
    while (remaining) {
        const int leader = __ffs(remaining) - 1;
        const int R = __shfl_sync(0xffffffffu, row_id, leader);
        const bool mine = valid && row_id == R;
        remaining &= ~__ballot_sync(0xffffffffu, mine);
        const int xmin = __reduce_min_sync(0xffffffffu, mine ? cx : INT_MAX);
        const int xmax = __reduce_max_sync(0xffffffffu, mine ? cx : INT_MIN);
        const int yR = R % g.nc[1], zR = R / g.nc[1];
        Range rx = dim_range(xmin, xmax, g.nc[0], g.periodic, g.full[0]);
        Range ry = dim_range(yR, yR, g.nc[1], g.periodic, g.full[1]);
        Range rz = dim_range(zR, zR, g.nc[2], g.periodic, g.full[2]);
        const int zz = rz.lo + seg;
        if (zz > rz.hi) continue;  // warp-uniform
        const int z = rz.wrap ? wrapi(zz, g.nc[2]) : zz;
        for (int yy = ry.lo; yy <= ry.hi; yy++) {
            const int y = ry.wrap ? wrapi(yy, g.nc[1]) : yy;
            // the x extent as one or two runs of consecutive cells
            int seg_lo[2], seg_hi[2], nrun;
            if (!rx.wrap) { seg_lo[0] = rx.lo; seg_hi[0] = rx.hi; nrun = 1; }
            else if (rx.lo < 0) { seg_lo[0] = rx.lo + g.nc[0]; seg_hi[0] = g.nc[0] - 1; seg_lo[1] = 0; seg_hi[1] = rx.hi; nrun = 2; }
            else if (rx.hi >= g.nc[0]) { seg_lo[0] = rx.lo; seg_hi[0] = g.nc[0] - 1; seg_lo[1] = 0; seg_hi[1] = rx.hi - g.nc[0]; nrun = 2; }
            else { seg_lo[0] = rx.lo; seg_hi[0] = rx.hi; nrun = 1; }
            for (int sg = 0; sg < nrun; sg++) {
                const int row = (z * g.nc[1] + y) * g.nc[0];
                // the system's slots, made global
                const int b0 = soff + cell_start[row + seg_lo[sg]], b1 = soff + cell_start[row + seg_hi[sg] + 1];
                for (int base = b0; base < b1; base += 32) {
                    const int t = base + lane;
                    __syncwarp();
                    if (t < b1) {
                        float4 ch, cl;
                        gm_ld_coord(a.coord + 2 * t, ch, cl);
                        s_rel[wib][lane] = make_float4((ch.x - rh.x) + (cl.x - rl.x), (ch.y - rh.y) + (cl.y - rl.y),
                                                       (ch.z - rh.z) + (cl.z - rl.z), 0.f);
                        s_orig[wib][lane] = a.perm[t];
                    }
                    __syncwarp();
                    if (!mine) continue;
                    const int m = min(32, b1 - base);
                    // distance tests of all 32 staged candidates: bit k of
                    // `near` within the list radius plus the margin, of `sure`
                    // within it minus the margin
                    unsigned near = 0, sure = 0;
#pragma unroll
                    for (int k = 0; k < 32; k++) {
                        const float r2 = rel_r2<PERIODIC>(s_rel[wib][k], mx, my, mz, g);
                        near |= (r2 <= rl2_hi ? 1u : 0u) << k;
                        sure |= (r2 <= rl2_lo ? 1u : 0u) << k;
                    }
                    near &= m < 32 ? (1u << m) - 1u : 0xffffffffu;
                    const int self = s - base;
                    if (self >= 0 && self < 32) near &= ~(1u << self);
                    // the accepted candidates, in order
                    while (near) {
                        const int k = __ffs(near) - 1;
                        near &= near - 1;
                        const int jo = s_orig[wib][k];
                        bool in = (sure >> k) & 1u;
                        if (!in) {
                            // the reference's own FP64 decision
                            double ex_ = exact_min_image(__dsub_rn(a.pos[jo], a.pos[my_orig]), bx[0]);
                            double ey_ = exact_min_image(__dsub_rn(a.pos[n + jo], a.pos[n + my_orig]), bx[1]);
                            double ez_ = exact_min_image(__dsub_rn(a.pos[2 * n + jo], a.pos[2 * n + my_orig]), bx[2]);
                            double rr = __dadd_rn(__dadd_rn(__dmul_rn(ex_, ex_), __dmul_rn(ey_, ey_)), __dmul_rn(ez_, ez_));
                            in = rr <= rl2_64;
                        }
                        if (!in) continue;
                        if (jo >= ex_lo && jo <= ex_hi) {
                            bool excluded = false;
#pragma unroll
                            for (int q = 0; q < 8; q++) excluded |= (ex[q] == jo);
                            if (ne > 8)
                                for (int q = e0 + 8; q < e1; q++) excluded |= (a.excl[q] == jo);
                            if (excluded) continue;
                        }
                        // the distance bucket, for accepted candidates only
                        // (the same r2 as the test above)
                        const float r2 = rel_r2<PERIODIC>(s_rel[wib][k], mx, my, mz, g);
                        const int bk = (r2 > bucket_r2.x ? 1 : 0) + (r2 > bucket_r2.y ? 1 : 0) + (r2 > bucket_r2.z ? 1 : 0);
                        if (cnt < cap_seg) {
                            my_stage[(size_t)cnt * 32] = (base + k) | (bk << GM_BUCKET_SHIFT);
#pragma unroll
                            for (int q = 0; q < GM_NBUCKET; q++) nb[q] += bk == q;
                        }
                        cnt++;
                    }
                }
            }
        }
    }
    // concatenate the layers: lane l's layer k goes after its layers < k
    int lmax = cnt;
    for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if (lane == 0) atomicMax(&a.status->max_layer, (unsigned)lmax);
    const int staged = cnt < cap_seg ? cnt : cap_seg;
#pragma unroll
    for (int q = 0; q < GM_NBUCKET; q++) s_cnt[seg][q][lane] = nb[q];
    __syncthreads();
    // this layer's first position in each bucket: the earlier buckets of all
    // layers, then this bucket of the earlier layers
    int off[GM_NBUCKET];
    int total = 0;
#pragma unroll
    for (int q = 0; q < GM_NBUCKET; q++) {
        int before = 0, all = 0;
#pragma unroll
        for (int k = 0; k < GM_NSEG; k++) {
            const int ck = s_cnt[k][q][lane];
            before += k < seg ? ck : 0;
            all += ck;
        }
        off[q] = total + before;
        total += all;
    }
    int smax = staged;
    for (int o = 16; o > 0; o >>= 1) smax = max(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    int *my_list = a.list + (size_t)group * 32 * cap + lane;
    for (int e = 0; e < smax; e++) {
        if (e < staged) {
            const int v = my_stage[(size_t)e * 32];
            const int bk = v >> GM_BUCKET_SHIFT;
            int pos = 0;
#pragma unroll
            for (int q = 0; q < GM_NBUCKET; q++) {
                if (bk == q) { pos = off[q]; off[q]++; }
            }
            if (pos < cap) my_list[(size_t)pos * 32] = v & GM_SLOT_MASK;
        }
    }
    if (seg == 0) {
        if (valid) a.count[s] = total < cap ? total : cap;
        if (valid && (cnt > cap_seg || total > cap)) atomicOr(&a.status->error, (unsigned)GM_DEV_LIST_OVERFLOW);
        int c = valid ? (total < cap ? total : cap) : 0;
        int tm = valid ? total : 0;
        for (int o = 16; o > 0; o >>= 1) {
            c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
            tm = max(tm, __shfl_xor_sync(0xffffffffu, tm, o));
        }
        if (lane == 0) {
            a.gmax[group] = c;
            atomicMax(&a.status->max_count, (unsigned)tm);
        }
    } else if (valid && cnt > cap_seg) {
        atomicOr(&a.status->error, (unsigned)GM_DEV_LIST_OVERFLOW);
    }
}

// Per-system launch shape: x covers the largest system, y the systems.
dim3 sys_grid(const ListArgs &a, int per_block, int cap_blocks) {
    int bx = (a.max_sys_atoms + per_block - 1) / per_block;
    bx = bx < 1 ? 1 : (bx > cap_blocks ? cap_blocks : bx);
    return dim3((unsigned)bx, (unsigned)a.n_sys, 1);
}

}  // namespace

void gm_launch_flags(const ListArgs &a, bool set, cudaStream_t s) {
    if (set) set_flags_kernel<<<(a.n_sys + 255) / 256, 256, 0, s>>>(a);
    else clear_flags_kernel<<<(a.n_sys + 255) / 256, 256, 0, s>>>(a);
}

void gm_launch_wrap(const ListArgs &a, double *pos, cudaStream_t s) {
    if (!a.periodic || a.n == 0) return;
    wrap_kernel<<<sys_grid(a, 256, 4096), 256, 0, s>>>(a, pos);
}

void gm_launch_grid(const ListArgs &a, cudaStream_t s) {
    if (!a.periodic && a.n > 0) bbox_kernel<<<dim3((unsigned)a.bbox_blocks, (unsigned)a.n_sys), 256, 0, s>>>(a);
    grid_kernel<<<a.n_sys, 256, 0, s>>>(a, a.bbox_blocks);
}

void gm_launch_bin(const ListArgs &a, cudaStream_t s) {
    // the grid kernel cleared the cells
    if (a.n > 0) assign_kernel<<<sys_grid(a, 256, 4096), 256, 0, s>>>(a);
    scan_cells_kernel<<<a.n_sys, 1024, 0, s>>>(a);
    if (a.n > 0) {
        scatter_kernel<<<sys_grid(a, 256, 4096), 256, 0, s>>>(a);
        rank_kernel<<<sys_grid(a, 256, 4096), 256, 0, s>>>(a);
    }
}

void gm_launch_pack(const ListArgs &a, bool fp64, cudaStream_t s) {
    if (a.n_slots == 0) return;
    pack_kernel<<<(a.n_slots + 255) / 256, 256, 0, s>>>(a, fp64);
}

void gm_launch_build(const ListArgs &a, cudaStream_t s) {
    if (a.n_slots == 0) return;
    const int groups = a.n_slots / 32;
    const double rl2 = a.r_list * a.r_list;  // neighbor.rs:25
    const double margin = 1e-3 * (rl2 > 144.0 ? rl2 / 144.0 : 1.0);
    // bucket bounds: the switch radius, the cutoff, halfway to the list radius
    const double rsh = 0.5 * (a.r_cut + a.r_list);
    const float3 bk = make_float3((float)(a.r_switch * a.r_switch), (float)(a.r_cut * a.r_cut), (float)(rsh * rsh));
    if (a.periodic)
        build_kernel<true><<<groups, GM_NSEG * 32, 0, s>>>(a, (float)(rl2 - margin), (float)(rl2 + margin), rl2, bk);
    else
        build_kernel<false><<<groups, GM_NSEG * 32, 0, s>>>(a, (float)(rl2 - margin), (float)(rl2 + margin), rl2, bk);
}
