// gm_static_list.cu — gm_build_pairs_static: the half neighbour list of a
// small system built without allocating device memory.
//
// Every gm_ctx entry point works on buffers that gm_create allocated.  This
// one is for callers that cannot allocate at the time they need a pair list:
// a host engine whose device memory is all held by its own pool (a caching
// allocator that already owns the free memory, so a cudaMalloc fails or
// forces the pool to be emptied), and code inside a running step that shares
// the device with other streams, where cudaFree (and a cudaMalloc that has to
// grow the heap) waits for the whole device.  Such a caller passes its own
// device buffers for positions, exclusions and pairs; the scratch the build
// needs (cell grid, counting sort, per-atom row counts) lives in one
// file-scope __device__ array whose size is fixed at compile time.
//
// The cell grid and counting sort are the same launches as the context's list
// build; the pair test is the reference's FP64 one (neighbor.rs:25-42:
// min-image difference, r^2 <= r_skin^2, exclusions skipped), applied to
// every candidate, so the pair set equals gm_get_pairs's for the same input.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "gm_internal.cuh"

namespace {

constexpr int kMaxAtoms = GM_STATIC_MAX_ATOMS;
constexpr int kMaxCells = 32768;
constexpr int kBboxBlocks = (kMaxAtoms + 255) / 256;
constexpr int kMaxDevices = 64;

// Layout of the scratch array.  What accumulates starts at zero: the status
// word is cleared by a memset, and the cell counts and cursors by the grid
// launch; every other field is written in full before it is read.
struct Scratch {
    double bbox[9 * kBboxBlocks];
    double ref[3 * kMaxAtoms];
    GridInfo grid;
    DevStatus status;
    int cell_count[kMaxCells], cell_cursor[kMaxCells], cell_start[kMaxCells + 1];
    int cell_of[kMaxAtoms], tmp_atom[kMaxAtoms], perm[kMaxAtoms], cell_sorted[kMaxAtoms];
    int row_count[kMaxAtoms], row_start[kMaxAtoms + 1];
    // the one system's tables (atoms, slots, cells) and rebuild flag
    int sys_atom_off[2], sys_slot_off[2], sys_cell_off[2];
    unsigned int sys_flag[1];
};
static_assert(sizeof(Scratch) <= GM_STATIC_SCRATCH_BYTES, "scratch layout exceeds GM_STATIC_SCRATCH_BYTES");

// One copy per device (a __device__ variable exists once in each context).
static __device__ __align__(256) unsigned char g_scratch[GM_STATIC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch on `device` (which is current), looked up on
// the first call for that device.
int scratch_for(int device, Scratch **out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "gm_build_pairs_static: cudaGetSymbolAddress failed on device %d: %s\n", device,
                         cudaGetErrorString(e));
            return GM_ERR_DEVICE;
        }
        g_scratch_ptr[device] = p;
    }
    *out = static_cast<Scratch *>(g_scratch_ptr[device]);
    return GM_OK;
}

__device__ __forceinline__ double min_image(double d, double L) {
    // neighbor.rs:74-76: d - L * round(d / L), no contraction
    return __dsub_rn(d, __dmul_rn(L, round(__ddiv_rn(d, L))));
}

// Cells searched along one axis around cell c: two on each side (cells are
// at least half the list radius wide), the whole axis when that would meet
// itself around a periodic box.
__device__ __forceinline__ void axis_cells(int c, int nc, int periodic, int full, int &lo, int &hi) {
    if (full) { lo = 0; hi = nc - 1; return; }
    lo = c - 2;
    hi = c + 2;
    if (periodic) {
        if (hi - lo + 1 >= nc) { lo = 0; hi = nc - 1; }
    } else {
        lo = lo < 0 ? 0 : lo;
        hi = hi >= nc ? nc - 1 : hi;
    }
}

__device__ __forceinline__ bool in_row(const int *excl, int lo, int hi, int j) {
    // exclusion rows are ascending: binary search
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int v = excl[mid];
        if (v == j) return true;
        if (v < j) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

struct PairTest {
    int n;
    const double *pos;
    const Scratch *S;
    const int *excl_start, *excl;
    double rl2, box[3];
};

// Calls f(j) for every j > i in the list radius of atom i that is not
// excluded, in cell order.
template <class F>
__device__ void for_each_partner(const PairTest &t, int i, F &&f) {
    const GridInfo &g = t.S->grid;
    const int n = t.n;
    const int c = t.S->cell_of[i];
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    int xlo, xhi, ylo, yhi, zlo, zhi;
    axis_cells(cx, g.nc[0], g.periodic, g.full[0], xlo, xhi);
    axis_cells(cy, g.nc[1], g.periodic, g.full[1], ylo, yhi);
    axis_cells(cz, g.nc[2], g.periodic, g.full[2], zlo, zhi);
    const double xi = t.pos[i], yi = t.pos[n + i], zi = t.pos[2 * n + i];
    const int e0 = t.excl_start ? t.excl_start[i] : 0, e1 = t.excl_start ? t.excl_start[i + 1] : 0;
    for (int zz = zlo; zz <= zhi; zz++) {
        const int z = (zz + g.nc[2]) % g.nc[2];
        for (int yy = ylo; yy <= yhi; yy++) {
            const int y = (yy + g.nc[1]) % g.nc[1];
            for (int xx = xlo; xx <= xhi; xx++) {
                const int x = (xx + g.nc[0]) % g.nc[0];
                const int cell = (z * g.nc[1] + y) * g.nc[0] + x;
                const int a1 = t.S->cell_start[cell + 1];
                for (int k = t.S->cell_start[cell]; k < a1; k++) {
                    const int j = t.S->perm[k];
                    if (j <= i) continue;
                    const double dx = min_image(__dsub_rn(t.pos[j], xi), t.box[0]);
                    const double dy = min_image(__dsub_rn(t.pos[n + j], yi), t.box[1]);
                    const double dz = min_image(__dsub_rn(t.pos[2 * n + j], zi), t.box[2]);
                    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                    if (!(r2 <= t.rl2)) continue;
                    if (e1 > e0 && in_row(t.excl, e0, e1, j)) continue;
                    f(j);
                }
            }
        }
    }
}

__global__ void count_rows_kernel(PairTest t, Scratch *S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t.n) return;
    const int n = t.n;
    if (!isfinite(t.pos[i]) || !isfinite(t.pos[n + i]) || !isfinite(t.pos[2 * n + i]))
        atomicOr(&S->status.error, (unsigned)GM_DEV_NONFINITE_POS);
    int cnt = 0;
    for_each_partner(t, i, [&](int) { cnt++; });
    S->row_count[i] = cnt;
}

// Exclusive scan of the row counts into row_start[0..n] in one block of 1024
// threads, each owning a run of consecutive rows.  n <= 16384 pairs per row
// bound the total below 2^31.
__global__ void scan_rows_kernel(int n, Scratch *S) {
    __shared__ int warp_tot[32];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(b + per, n);
    int local = 0;
    for (int r = b; r < e; r++) local += S->row_count[r];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        warp_tot[lane] = v;
    }
    __syncthreads();
    int run = incl - local + (w > 0 ? warp_tot[w - 1] : 0);
    for (int r = b; r < e; r++) {
        S->row_start[r] = run;
        run += S->row_count[r];
    }
    if (threadIdx.x == blockDim.x - 1) S->row_start[n] = warp_tot[(blockDim.x >> 5) - 1];
}

// Writes row i at row_start[i], kept ascending in j by insertion as it is
// filled.  Nothing is written when the total exceeds the caller's capacity,
// nor after an earlier launch of the build raised an error (non-finite
// positions, an extent or cell overflow), so an error return leaves the
// caller's pair buffers untouched.
__global__ void emit_rows_kernel(PairTest t, uint32_t *pair_i, uint32_t *pair_j, long long max_pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t.n || t.S->status.error || (long long)t.S->row_start[t.n] > max_pairs) return;
    const int base = t.S->row_start[i];
    int k = 0;
    for_each_partner(t, i, [&](int j) {
        int p = base + k;
        while (p > base && pair_j[p - 1] > (uint32_t)j) {
            pair_j[p] = pair_j[p - 1];
            p--;
        }
        pair_j[p] = (uint32_t)j;
        pair_i[base + k] = (uint32_t)i;
        k++;
    });
}

bool positive_finite(double v) { return std::isfinite(v) && v > 0.0; }

// Makes `device` current for the call and gives the caller back the device
// it had current, on every return path.
struct CurrentDevice {
    int prev = -1;
    bool changed = false;
    cudaError_t enter(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev == device) return cudaSuccess;
        e = cudaSetDevice(device);
        changed = e == cudaSuccess;
        return e;
    }
    ~CurrentDevice() {
        if (changed) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int32_t gm_build_pairs_static(double *d_pos, int32_t n_atoms, const int32_t *d_excl_start,
                                         const int32_t *d_excl, const gm_params *params, uint32_t *d_pair_i,
                                         uint32_t *d_pair_j, int64_t max_pairs, int64_t *n_pairs, void *stream) {
    if (!params || !n_pairs) return GM_ERR_INVALID_ARGUMENT;
    *n_pairs = 0;
    if (n_atoms < 0 || max_pairs < 0) return GM_ERR_INVALID_ARGUMENT;
    if (n_atoms > kMaxAtoms) {
        std::fprintf(stderr, "gm_build_pairs_static: %d atoms exceed the static scratch limit of %d atoms\n",
                     (int)n_atoms, kMaxAtoms);
        return GM_ERR_UNSUPPORTED;
    }
    if ((d_pair_i == nullptr) != (d_pair_j == nullptr) || (d_excl_start == nullptr) != (d_excl == nullptr))
        return GM_ERR_INVALID_ARGUMENT;
    if (!positive_finite(params->r_skin) || !positive_finite(params->box[0]) || !positive_finite(params->box[1]) ||
        !positive_finite(params->box[2]))
        return GM_ERR_INVALID_ARGUMENT;
    if (params->device < 0 || params->device >= kMaxDevices) return GM_ERR_INVALID_ARGUMENT;
    if (n_atoms == 0) return GM_OK;
    if (!d_pos) return GM_ERR_INVALID_ARGUMENT;
    CurrentDevice current;
    if (current.enter(params->device) != cudaSuccess) return GM_ERR_NO_DEVICE;
    Scratch *S = nullptr;
    int rc = scratch_for(params->device, &S);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int n = n_atoms;

    // the one system: atoms [0, n), slots [0, n) (no list is built, so no
    // padding is needed), the whole cell budget
    const int tables[6] = {0, n, 0, n, 0, kMaxCells + 1};
    if (cudaMemcpyAsync(S->sys_atom_off, tables, sizeof(tables), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return GM_ERR_DEVICE;
    ListArgs a{};
    a.n = n;
    a.n_slots = n;
    a.n_sys = 1;
    a.sys_atom_off = S->sys_atom_off;
    a.sys_slot_off = S->sys_slot_off;
    a.sys_cell_off = S->sys_cell_off;
    a.sys_flag = S->sys_flag;
    a.max_sys_atoms = n;
    a.pos = d_pos;
    a.ref = S->ref;
    a.perm = S->perm;
    a.cell_of = S->cell_of;
    a.cell_sorted = S->cell_sorted;
    a.cell_count = S->cell_count;
    a.cell_start = S->cell_start;
    a.cell_cursor = S->cell_cursor;
    a.tmp_atom = S->tmp_atom;
    a.grid = &S->grid;
    a.status = &S->status;
    a.r_list = params->r_skin;
    for (int d = 0; d < 3; d++) a.box[d] = params->box[d];
    a.periodic = params->periodic ? 1 : 0;
    a.bbox_scratch = S->bbox;
    a.bbox_blocks = (n + 255) / 256 < kBboxBlocks ? (n + 255) / 256 : kBboxBlocks;

    if (cudaMemsetAsync(&S->status, 0, sizeof(DevStatus), s) != cudaSuccess) return GM_ERR_DEVICE;
    gm_launch_flags(a, true, s);
    gm_launch_wrap(a, d_pos, s);  // neighbor.rs:10-16
    gm_launch_grid(a, s);
    gm_launch_bin(a, s);

    PairTest t;
    t.n = n;
    t.pos = d_pos;
    t.S = S;
    t.excl_start = d_excl_start;
    t.excl = d_excl;
    t.rl2 = params->r_skin * params->r_skin;  // neighbor.rs:25
    for (int d = 0; d < 3; d++) t.box[d] = params->box[d];
    const int blocks = (n + 127) / 128;
    count_rows_kernel<<<blocks, 128, 0, s>>>(t, S);
    scan_rows_kernel<<<1, 1024, 0, s>>>(n, S);
    if (d_pair_i) emit_rows_kernel<<<blocks, 128, 0, s>>>(t, d_pair_i, d_pair_j, (long long)max_pairs);
    if (cudaGetLastError() != cudaSuccess) return GM_ERR_DEVICE;

    unsigned int err = 0;
    int total = 0;
    if (cudaMemcpyAsync(&err, &S->status.error, sizeof(err), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&total, &S->row_start[n], sizeof(total), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GM_ERR_DEVICE;
    if (err & GM_DEV_NONFINITE_POS) return GM_ERR_NONFINITE;
    if (err & (GM_DEV_EXTENT | GM_DEV_CELL_OVERFLOW)) return GM_ERR_UNSUPPORTED;
    if (err) return GM_ERR_DEVICE;
    *n_pairs = total;
    if (d_pair_i && total > max_pairs) return GM_ERR_LIST_OVERFLOW;
    return GM_OK;
}
