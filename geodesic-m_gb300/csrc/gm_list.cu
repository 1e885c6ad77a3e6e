// gm_list.cu — Verlet list build on the device (neighbor.rs:8-55 semantics).
//
// Pipeline at each rebuild (all on the context's stream, no host sync):
//   wrap (periodic only) -> bbox partials -> grid setup -> cell assignment +
//   counting-sort histogram -> scan -> scatter -> in-cell rank by caller
//   index (deterministic order) -> pack -> list build.
// The list build gives each warp 32 consecutive cell-sorted atoms; the warp
// streams every candidate in the union of their 5x5x5 half-cell stencils
// through shared memory and each lane tests it against its own atom.  The
// test runs in FP32 on hi+lo coordinates; candidates within `margin` of the
// list radius are re-decided with the reference's exact FP64 expression
// (min-image, then dx*dx + dy*dy + dz*dz, no fused multiply-add), so the pair
// set equals the reference's bit for bit.
#include <cfloat>

#include "gm_internal.cuh"

namespace {

constexpr int kBuildWarps = 4;

__device__ __forceinline__ double exact_min_image(double d, double L) {
    // neighbor.rs:74-76: d - L * round(d / L), no contraction
    return __dsub_rn(d, __dmul_rn(L, round(__ddiv_rn(d, L))));
}

__device__ __forceinline__ double exact_wrap(double x, double L) {
    // neighbor.rs:86-88: x - L * floor(x / L)
    return __dsub_rn(x, __dmul_rn(L, floor(__ddiv_rn(x, L))));
}

__global__ void wrap_kernel(int n, double *pos, double b0, double b1, double b2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = exact_wrap(pos[i], b0);
    pos[n + i] = exact_wrap(pos[n + i], b1);
    pos[2 * n + i] = exact_wrap(pos[2 * n + i], b2);
}

// Per block: min x,y,z, max x,y,z and the sum x,y,z of the positions.
__global__ void bbox_kernel(int n, const double *pos, double *partial) {
    __shared__ double sm[9][256];
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX}, sum[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int d = 0; d < 3; d++) {
            double v = pos[d * n + i];
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
    if (threadIdx.x < 9) partial[blockIdx.x * 9 + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void grid_kernel(const double *partial, int blocks, GridInfo *g, DevStatus *st, double r_list,
                            double b0, double b1, double b2, int periodic, int max_cells, int n_atoms) {
    // reduce the per-block bbox partials with the whole block first
    __shared__ double red[9][256];
    for (int v = 0; v < 9; v++) {
        double acc = v < 3 ? DBL_MAX : (v < 6 ? -DBL_MAX : 0.0);
        for (int b = threadIdx.x; b < blocks; b += blockDim.x) {
            const double x = partial[b * 9 + v];
            acc = v < 3 ? fmin(acc, x) : (v < 6 ? fmax(acc, x) : acc + x);
        }
        red[v][threadIdx.x] = acc;
    }
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k)
            for (int v = 0; v < 9; v++) {
                const double x = red[v][threadIdx.x + k];
                red[v][threadIdx.x] = v < 3 ? fmin(red[v][threadIdx.x], x)
                                            : (v < 6 ? fmax(red[v][threadIdx.x], x) : red[v][threadIdx.x] + x);
            }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double box[3] = {b0, b1, b2};
    const double wmin = r_list * 0.5 * (1.0 + 1e-5) + 1e-6;
    int nc[3];
    double w[3], lo[3];
    g->periodic = periodic;
    for (int d = 0; d < 3; d++) {
        g->box[d] = (float)box[d];
        g->inv_box[d] = (float)(1.0 / box[d]);
    }
    if (periodic) {
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
            if (ext + r_list >= 0.5 * box[d]) atomicOr(&st->error, (unsigned)GM_DEV_EXTENT);
            const double mean = n_atoms > 0 ? sum[d] / n_atoms : 0.0;
            const double half = 0.5 * per_dim * wmin;
            double a = fmax(mn[d], mean - half), b = fmin(mx[d], mean + half);
            if (!(b >= a)) { a = mn[d]; b = mx[d]; }
            const double pad = 1e-3 * (1.0 + (b - a));
            g->origin[d] = 0.5 * (a + b);
            lo[d] = (a - g->origin[d]) - pad;
            nc[d] = (int)floor((b - a + 2.0 * pad) / wmin);
            if (nc[d] < 1) nc[d] = 1;
        }
    }
    // keep the cell count within the allocation by coarsening the grid
    // (coarser cells only widen the 5x5x5 search, never miss a pair)
    while ((long long)nc[0] * nc[1] * nc[2] > max_cells) {
        for (int d = 0; d < 3; d++) nc[d] = nc[d] > 1 ? (nc[d] * 3) / 4 : 1;
    }
    for (int d = 0; d < 3; d++) {
        double span = periodic ? box[d] : -2.0 * lo[d];
        w[d] = span / nc[d];
        g->nc[d] = nc[d];
        g->lo[d] = (float)lo[d];
        g->inv_w[d] = (float)(1.0 / w[d]);
        g->full[d] = periodic && nc[d] < 5;
    }
    g->ncell = nc[0] * nc[1] * nc[2];  // <= max_cells by construction
    st->rebuild = 0;
    st->n_rebuilds += 1;
}

__device__ __forceinline__ int cell_coord(float h, float lo, float inv_w, int nc) {
    float t = floorf((h - lo) * inv_w);
    int c = (int)t;  // NaN converts to 0
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

__global__ void assign_kernel(int n, const double *pos, double *ref, const GridInfo *g, int *cell_of,
                              int *cell_count, int max_cells, DevStatus *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c3[3];
    for (int d = 0; d < 3; d++) {
        double x = pos[d * n + i];
        ref[d * n + i] = x;  // NeighborList::ref_{x,y,z} (neighbor.rs:48-50)
        c3[d] = cell_coord((float)(x - g->origin[d]), g->lo[d], g->inv_w[d], g->nc[d]);
    }
    int c = (c3[2] * g->nc[1] + c3[1]) * g->nc[0] + c3[0];
    if (c < 0 || c >= max_cells) {
        atomicOr(&st->error, (unsigned)GM_DEV_CELL_OVERFLOW);
        c = 0;
    }
    cell_of[i] = c;
    atomicAdd(&cell_count[c], 1);
}

// Exclusive scan of cell_count[0..ncell) into cell_start[0..ncell], in three
// launches: per-block scans of 1024 cells with block totals, a scan of the
// totals in one block, then the block offsets added back.
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

__global__ void scan_local_kernel(const GridInfo *g, const int *cell_count, int *cell_start, int *block_sums,
                                  int max_cells) {
    __shared__ int warp_sums[32];
    const int ncell = min(g->ncell, max_cells);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x >= ncell + 1) return;  // whole block idle (uniform)
    const int v = i < ncell ? cell_count[i] : 0;
    int total;
    const int excl = block_exclusive_scan(v, warp_sums, total);
    if (i <= ncell) cell_start[i] = excl;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void scan_blocks_kernel(const GridInfo *g, int *block_sums, int max_cells) {
    __shared__ int warp_sums[32];
    const int ncell = min(g->ncell, max_cells);
    const int nblocks = (ncell + 1 + 1023) / 1024;
    int carry = 0;
    for (int base = 0; base < nblocks; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < nblocks ? block_sums[i] : 0;
        int total;
        const int excl = block_exclusive_scan(v, warp_sums, total);
        if (i < nblocks) block_sums[i] = excl + carry;
        carry += total;
    }
}

__global__ void scan_add_kernel(const GridInfo *g, int *cell_start, const int *block_sums, int max_cells) {
    const int ncell = min(g->ncell, max_cells);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= ncell) cell_start[i] += block_sums[blockIdx.x];
}

__global__ void scatter_kernel(int n, const int *cell_of, const int *cell_start, int *cell_cursor, int *tmp_atom) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell_of[i];
    int slot = cell_start[c] + atomicAdd(&cell_cursor[c], 1);
    tmp_atom[slot] = i;
}

// Within a cell, atoms are ordered by caller index: the rank of an atom is
// the number of cell members with a smaller index.  Independent of the
// atomic order of the scatter, so the sorted layout is deterministic.
__global__ void rank_kernel(int n, const int *cell_of, const int *cell_start, const int *tmp_atom, int *perm,
                            int *cell_sorted, DevStatus *st) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int a = tmp_atom[k];
    int c = cell_of[a];
    int s0 = cell_start[c], s1 = cell_start[c + 1];
    if (s1 - s0 > 65536) {
        // no physical system packs this many atoms into one half cell; keep
        // the quadratic rank bounded and report it
        atomicOr(&st->error, (unsigned)GM_DEV_CELL_OVERFLOW);
        perm[k] = a;
        cell_sorted[k] = c;
        return;
    }
    int rank = 0;
    for (int m = s0; m < s1; m++) rank += tmp_atom[m] < a;
    perm[s0 + rank] = a;
    cell_sorted[s0 + rank] = c;
}

__global__ void pack_kernel(int n, const double *pos, const int *perm, const int *type, const float *charge,
                            const GridInfo *g, float4 *hi, float4 *lo, double4 *pos64s, int *type_sorted,
                            const double *charge64, long long *force) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int a = perm[s];
    double x = pos[a], y = pos[n + a], z = pos[2 * n + a];
    double dx = x - g->origin[0], dy = y - g->origin[1], dz = z - g->origin[2];
    float hx = (float)dx, hy = (float)dy, hz = (float)dz;
    hi[s] = make_float4(hx, hy, hz, __int_as_float(type[a]));
    lo[s] = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz), charge[a]);
    if (pos64s) {
        pos64s[s] = make_double4(x, y, z, charge64[a]);
        type_sorted[s] = type[a];
    }
    force[a] = 0;
    force[n + a] = 0;
    force[2 * n + a] = 0;
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

__global__ void __launch_bounds__(kBuildWarps * 32)
build_kernel(int n, int cap, const float4 *__restrict__ hi, const float4 *__restrict__ lo,
             const int *__restrict__ perm, const int *__restrict__ cell_sorted, const int *__restrict__ cell_start,
             const GridInfo *__restrict__ gp, const double *__restrict__ pos, const int *__restrict__ excl_start,
             const int *__restrict__ excl, int *__restrict__ list, int *__restrict__ count, int *__restrict__ gmax,
             DevStatus *st, float rl2_lo, float rl2_hi, double rl2_64, double b0, double b1, double b2) {
    __shared__ float4 s_hi[kBuildWarps][32];
    __shared__ float4 s_lo[kBuildWarps][32];
    __shared__ int s_orig[kBuildWarps][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int group = blockIdx.x * kBuildWarps + wib;
    const int s = group * 32 + lane;
    if (group * 32 >= n) return;
    const bool valid = s < n;
    const GridInfo g = *gp;
    float4 mh = make_float4(0.f, 0.f, 0.f, 0.f), ml = mh;
    int my_orig = -1, my_cell = 0;
    if (valid) {
        mh = hi[s];
        ml = lo[s];
        my_orig = perm[s];
        my_cell = cell_sorted[s];
    }
    // own exclusions (caller indices, ascending); up to 8 kept in registers
    int e0 = 0, e1 = 0;
    int ex[8];
    if (valid) { e0 = excl_start[my_orig]; e1 = excl_start[my_orig + 1]; }
    const int ne = e1 - e0;
#pragma unroll
    for (int k = 0; k < 8; k++) ex[k] = (k < ne) ? excl[e0 + k] : -1;
    // Candidate regions, one per distinct cell row (cy, cz) among the lanes:
    // a group of 32 sorted atoms usually lies in one row of cells, sometimes
    // straddles the end of a row.  Sweeping each row's own 5 x 5 x (span + 4)
    // box keeps the regions tight (one box over both rows would cover the
    // whole row); a lane tests only the candidates of its own row's box, so
    // it never meets a candidate twice.
    const int cx = my_cell % g.nc[0], cy = (my_cell / g.nc[0]) % g.nc[1], cz = my_cell / (g.nc[0] * g.nc[1]);
    const int row_id = valid ? cz * g.nc[1] + cy : -1;
    int *my_list = list + (size_t)group * 32 * cap + lane;
    int cnt = 0;
    const double bx[3] = {b0, b1, b2};
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
        for (int zz = rz.lo; zz <= rz.hi; zz++) {
            const int z = rz.wrap ? wrapi(zz, g.nc[2]) : zz;
            for (int yy = ry.lo; yy <= ry.hi; yy++) {
                const int y = ry.wrap ? wrapi(yy, g.nc[1]) : yy;
                // the x extent as one or two runs of consecutive cells
                int seg_lo[2], seg_hi[2], nseg;
                if (!rx.wrap) { seg_lo[0] = rx.lo; seg_hi[0] = rx.hi; nseg = 1; }
                else if (rx.lo < 0) { seg_lo[0] = rx.lo + g.nc[0]; seg_hi[0] = g.nc[0] - 1; seg_lo[1] = 0; seg_hi[1] = rx.hi; nseg = 2; }
                else if (rx.hi >= g.nc[0]) { seg_lo[0] = rx.lo; seg_hi[0] = g.nc[0] - 1; seg_lo[1] = 0; seg_hi[1] = rx.hi - g.nc[0]; nseg = 2; }
                else { seg_lo[0] = rx.lo; seg_hi[0] = rx.hi; nseg = 1; }
                for (int sg = 0; sg < nseg; sg++) {
                    const int row = (z * g.nc[1] + y) * g.nc[0];
                    const int a0 = cell_start[row + seg_lo[sg]], a1 = cell_start[row + seg_hi[sg] + 1];
                    for (int base = a0; base < a1; base += 32) {
                        const int t = base + lane;
                        __syncwarp();
                        if (t < a1) {
                            s_hi[wib][lane] = hi[t];
                            s_lo[wib][lane] = lo[t];
                            s_orig[wib][lane] = perm[t];
                        }
                        __syncwarp();
                        if (!mine) continue;
                        const int m = min(32, a1 - base);
                        for (int k = 0; k < m; k++) {
                            const int j = base + k;
                            if (j == s) continue;
                            const float4 ch = s_hi[wib][k], cl = s_lo[wib][k];
                            float dx = (ch.x - mh.x) + (cl.x - ml.x);
                            float dy = (ch.y - mh.y) + (cl.y - ml.y);
                            float dz = (ch.z - mh.z) + (cl.z - ml.z);
                            if (g.periodic) {
                                dx -= g.box[0] * rintf(dx * g.inv_box[0]);
                                dy -= g.box[1] * rintf(dy * g.inv_box[1]);
                                dz -= g.box[2] * rintf(dz * g.inv_box[2]);
                            }
                            const float r2 = dx * dx + dy * dy + dz * dz;
                            if (r2 > rl2_hi) continue;
                            const int jo = s_orig[wib][k];
                            bool in = r2 <= rl2_lo;
                            if (!in) {
                                // the reference's own FP64 decision
                                double ex_ = exact_min_image(__dsub_rn(pos[jo], pos[my_orig]), bx[0]);
                                double ey_ = exact_min_image(__dsub_rn(pos[n + jo], pos[n + my_orig]), bx[1]);
                                double ez_ = exact_min_image(__dsub_rn(pos[2 * n + jo], pos[2 * n + my_orig]), bx[2]);
                                double rr = __dadd_rn(__dadd_rn(__dmul_rn(ex_, ex_), __dmul_rn(ey_, ey_)), __dmul_rn(ez_, ez_));
                                in = rr <= rl2_64;
                            }
                            if (!in) continue;
                            bool excluded = false;
#pragma unroll
                            for (int q = 0; q < 8; q++) excluded |= (ex[q] == jo);
                            if (ne > 8)
                                for (int q = e0 + 8; q < e1; q++) excluded |= (excl[q] == jo);
                            if (excluded) continue;
                            if (cnt < cap) my_list[(size_t)cnt * 32] = j;
                            cnt++;
                        }
                    }
                }
            }
        }
    }
    if (valid) {
        count[s] = cnt < cap ? cnt : cap;
        if (cnt > cap) atomicOr(&st->error, (unsigned)GM_DEV_LIST_OVERFLOW);
    }
    int c = valid ? (cnt < cap ? cnt : cap) : 0;
    for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
    if (lane == 0) gmax[group] = c;
}

}  // namespace

void gm_launch_wrap(const ListArgs &a, double *pos, cudaStream_t s) {
    if (!a.periodic || a.n == 0) return;
    wrap_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a.n, pos, a.box[0], a.box[1], a.box[2]);
}

void gm_launch_grid(const ListArgs &a, cudaStream_t s) {
    if (!a.periodic && a.n > 0) bbox_kernel<<<a.bbox_blocks, 256, 0, s>>>(a.n, a.pos, a.bbox_scratch);
    grid_kernel<<<1, 256, 0, s>>>(a.bbox_scratch, a.periodic || a.n == 0 ? 0 : a.bbox_blocks, a.grid, a.status,
                                 a.r_list, a.box[0], a.box[1], a.box[2], a.periodic, a.max_cells, a.n);
}

void gm_launch_bin(const ListArgs &a, cudaStream_t s) {
    cudaMemsetAsync(a.cell_count, 0, sizeof(int) * (size_t)a.max_cells, s);
    cudaMemsetAsync(a.cell_cursor, 0, sizeof(int) * (size_t)a.max_cells, s);
    const int nb = (a.n + 255) / 256;
    if (a.n > 0)
        assign_kernel<<<nb, 256, 0, s>>>(a.n, a.pos, a.ref, a.grid, a.cell_of, a.cell_count, a.max_cells, a.status);
    const int scan_blocks = (a.max_cells + 1 + 1023) / 1024;
    scan_local_kernel<<<scan_blocks, 1024, 0, s>>>(a.grid, a.cell_count, a.cell_start, a.scan_scratch, a.max_cells);
    scan_blocks_kernel<<<1, 1024, 0, s>>>(a.grid, a.scan_scratch, a.max_cells);
    scan_add_kernel<<<scan_blocks, 1024, 0, s>>>(a.grid, a.cell_start, a.scan_scratch, a.max_cells);
    if (a.n > 0) {
        scatter_kernel<<<nb, 256, 0, s>>>(a.n, a.cell_of, a.cell_start, a.cell_cursor, a.tmp_atom);
        rank_kernel<<<nb, 256, 0, s>>>(a.n, a.cell_of, a.cell_start, a.tmp_atom, a.perm, a.cell_sorted, a.status);
    }
}

void gm_launch_pack(const ListArgs &a, bool fp64, cudaStream_t s) {
    if (a.n == 0) return;
    pack_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a.n, a.pos, a.perm, a.type, a.charge, a.grid, a.hi, a.lo,
                                                   fp64 ? a.pos64s : nullptr, a.type_sorted, a.charge64, a.force);
}

void gm_launch_build(const ListArgs &a, cudaStream_t s) {
    if (a.n == 0) return;
    const int groups = (a.n + 31) / 32;
    const double rl2 = a.r_list * a.r_list;  // neighbor.rs:25
    const double margin = 1e-3 * (rl2 > 144.0 ? rl2 / 144.0 : 1.0);
    build_kernel<<<(groups + kBuildWarps - 1) / kBuildWarps, kBuildWarps * 32, 0, s>>>(
        a.n, a.cap, a.hi, a.lo, a.perm, a.cell_sorted, a.cell_start, a.grid, a.pos, a.excl_start, a.excl, a.list,
        a.count, a.gmax, a.status, (float)(rl2 - margin), (float)(rl2 + margin), rl2, a.box[0], a.box[1], a.box[2]);
}
