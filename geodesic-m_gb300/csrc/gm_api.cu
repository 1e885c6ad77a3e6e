// gm_api.cu — the backend context and the C ABI (include/geodesic_cuda.h).
//
// gm_ctx mirrors the reference's CpuBackend/GpuBackend (cpu_backend.rs:25-37,
// gpu_backend.rs:11-22): it owns the atoms, the topology, the neighbour list
// and the force buffer, on the device.  Host entry points upload the caller's
// arrays, run the kernels on the context's stream and copy results back;
// the resident entry points keep everything on the device and run the BAB
// loop as a CUDA graph, one captured step per launch: without constraints the
// fused kernel (the previous step's closing half-kick, this step's opening
// one, drift, rebuild check, coordinate pack), an IF node holding the list
// rebuild, and the forces (pair kernel beside the bonded/1-4 kernel); with
// constraints half-kick, drift, SHAKE, check, the IF node, forces,
// half-kick, RATTLE.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <utility>
#include <vector>

#include "gm_internal.cuh"

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct gm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // bonded/1-4 branch beside the pair kernel
    // gm_steps' host copies beside the device work: the velocity upload
    // beside the position check, the position download beside the final
    // force evaluation
    cudaStream_t xfer = nullptr;
    cudaEvent_t ev_xfer_in = nullptr, ev_xfer_out = nullptr;
    gm_params p{};
    int n = 0;
    bool fp64 = false;
    std::string err;
    long long launches = 0;
    std::vector<void *> allocs;

    // atoms
    int ntypes = 0;
    double *d_mass = nullptr, *d_inv_mass = nullptr, *d_sigma = nullptr, *d_eps = nullptr, *d_charge64 = nullptr;
    int *d_type = nullptr;
    float2 *d_qw = nullptr;  // per atom (Q_hi, Q_lo | type) of the mixed pair kernel's slot records
    float4 *d_tab32 = nullptr;
    double2 *d_tab64 = nullptr;
    // state
    double *d_pos = nullptr, *d_vel = nullptr, *d_ref = nullptr, *d_dref = nullptr, *d_fout = nullptr,
           *d_host_f = nullptr;
    long long *d_force = nullptr;
    // sorted / cells
    float4 *d_coord = nullptr;  // two float4 per slot (hi, lo)
    double4 *d_pos64s = nullptr;
    int *d_type_sorted = nullptr;
    int *d_perm = nullptr, *d_cell_of = nullptr, *d_cell_sorted = nullptr, *d_cell_count = nullptr,
        *d_cell_start = nullptr, *d_cell_cursor = nullptr, *d_tmp_atom = nullptr, *d_slot_of = nullptr;
    long long total_cells = 0;     // cell budget of all systems
    // systems of a batch (one for a plain context)
    int n_sys = 1, n_slots = 0, max_sys_atoms = 0;
    std::vector<int> h_atom_off;
    int *d_sys_atom_off = nullptr, *d_sys_slot_off = nullptr, *d_sys_cell_off = nullptr, *d_atom_sys = nullptr,
        *d_group_sys = nullptr;
    unsigned int *d_sys_flag = nullptr;
    long long *d_e_sys = nullptr;  // per-system energies (batches)
    GridInfo *d_grid = nullptr;
    double *d_bbox = nullptr;
    int bbox_blocks = 0;
    // list
    int cap = 0, cap_seg = 0, n_groups = 0;  // list entries per atom; staging entries per atom and z layer
    int split = 1;                   // warps per group in the pair kernel
    int pair_warps = 4, pair_grid = 0;  // FP32 pair kernel block size and grid (0: one item per warp)
    int *d_list = nullptr, *d_count = nullptr, *d_gmax = nullptr, *d_stage = nullptr;
    bool built = false;
    // exclusions
    int *d_excl_start = nullptr, *d_excl = nullptr;
    // bonded
    int n_bonds = 0, n_angles = 0, n_diheds = 0, bonded_blocks = 0;
    int *d_bi = nullptr, *d_bj = nullptr, *d_ai = nullptr, *d_aj = nullptr, *d_ak = nullptr, *d_di = nullptr,
        *d_dj = nullptr, *d_dk = nullptr, *d_dl = nullptr, *d_dn = nullptr;
    double *d_bk = nullptr, *d_br0 = nullptr, *d_akth = nullptr, *d_ath0 = nullptr, *d_dkphi = nullptr,
           *d_ddelta = nullptr;
    double2 *d_dcs = nullptr;  // (cos delta, sin delta) per dihedral
    double4 *d_p14par = nullptr;  // per 1-4 pair (sigma, 4 eps s_lj, 24 eps s_lj, k_C q_i q_j s_coul)
    // 1-4
    int n14 = 0, blocks14 = 0;
    int *d_p14i = nullptr, *d_p14j = nullptr;
    // constraints
    int n_constr = 0, n_clusters = 0, n_single = 0, n_star_end = 0, n_warp_end = 0;
    int *d_ci = nullptr, *d_cj = nullptr, *d_cl_cstart = nullptr, *d_cl_cons = nullptr, *d_cl_astart = nullptr,
        *d_cl_atoms = nullptr, *d_cl_acstart = nullptr, *d_cl_acons = nullptr, *d_cl_iters = nullptr,
        *d_cl_worst_idx = nullptr;
    double *d_cdsq = nullptr, *d_lam = nullptr, *d_rvec = nullptr, *d_cl_worst = nullptr;
    std::vector<int> h_ci, h_cj;
    // constraint warm start (gm_mlp.cu)
    bool ws_on = false, ws_model = false;
    int ws_rec_stride = 0, ws_rec_cap = 0;
    int *d_atom_cstart = nullptr, *d_atom_cref = nullptr;
    float4 *d_ws_unit = nullptr;
    float *d_ws_w = nullptr;
    unsigned char *d_ws_packed = nullptr;  // the parameters in the inference's layout (gm_launch_ws_pack)
    float *d_ws_params = nullptr, *d_ws_norm = nullptr, *d_ws_m = nullptr, *d_ws_v = nullptr, *d_ws_feat = nullptr,
          *d_rec_feat = nullptr, *d_rec_t = nullptr, *d_ws_partial = nullptr, *d_ws_out = nullptr;
    double *d_ws_scale = nullptr, *d_ws_t1 = nullptr, *d_ws_lam0 = nullptr, *d_lam_sum = nullptr,
           *d_ws_stats = nullptr;
    int ws_partial_blocks = 0;
    // energy
    double *d_epart = nullptr, *d_energy = nullptr, *d_kin_part = nullptr, *d_ke = nullptr;
    int n_epart = 0;
    bool energy_stale = false;  // epart holds the last forces' partials, d_energy not yet their sum
    // trajectory frames recorded during resident steps
    int frame_interval = 0, frame_cap = 0;
    float *d_frame_xyz = nullptr;
    unsigned long long *d_frame_step = nullptr;
    double *d_frame_energy = nullptr, *d_frame_part = nullptr;
    // status
    DevStatus *d_status = nullptr;
    DevStatus *h_status = nullptr;  // pinned
    double *h_energy = nullptr;     // pinned: the energy read back with the results (a copy into
                                    // pageable memory would block the host until it completes)
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    double graph_dt = 0.0;
    int graph_cap = -1;
    long long launches_per_step = 0;
    bool forces_current = false;
    bool use_graph = true;           // GM_GRAPH=0: direct launches (profilers)
    // step form of unconstrained mixed-precision runs: 0 the kernel graph,
    // 1 one persistent cooperative launch per step (gm_step.cu, the default)
    int step_form = GM_STEP_PERSISTENT;
    int persist_blocks = 0;          // its grid: every block resident
    StepSync *d_sync = nullptr;
    bool stall_barrier = false;      // gm_stall_next_barrier: the next persistent call's barrier cannot release
    long long rebuild_base = 0;
    unsigned last_shake_T = 0, last_rattle_T = 0;
};

namespace {

int fail(gm_ctx *c, int code, const char *fmt, ...) {
    if (c) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_status(gm_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GM_OK;
    if (e == cudaErrorMemoryAllocation) return fail(c, GM_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(c, GM_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
    return fail(c, GM_ERR_DEVICE, "%s: %s", what, cudaGetErrorString(e));
}

#define GM_CUDA(ctx, call)                                      \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_status(ctx, e_, #call); \
    } while (0)

template <typename T>
int dalloc(gm_ctx *c, T **ptr, size_t count) {
    *ptr = nullptr;
    size_t bytes = sizeof(T) * (count > 0 ? count : 1);
    cudaError_t e = cudaMalloc((void **)ptr, bytes);
    if (e != cudaSuccess) return cuda_status(c, e, "cudaMalloc");
    c->allocs.push_back(*ptr);
    return GM_OK;
}

template <typename T>
int dupload(gm_ctx *c, T **ptr, const T *host, size_t count) {
    int rc = dalloc(c, ptr, count);
    if (rc) return rc;
    if (count && host) GM_CUDA(c, cudaMemcpy(*ptr, host, sizeof(T) * count, cudaMemcpyHostToDevice));
    return GM_OK;
}

void dfree(gm_ctx *c, void *ptr) {
    if (!ptr) return;
    cudaFree(ptr);
    c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), ptr), c->allocs.end());
}

std::vector<int> to_int(const uint32_t *a, int64_t n) {
    std::vector<int> v((size_t)n);
    for (int64_t i = 0; i < n; i++) v[(size_t)i] = (int)a[i];
    return v;
}

bool finite3(const double *x, const double *y, const double *z, int n) {
    for (int i = 0; i < n; i++)
        if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(z[i])) return false;
    return true;
}

ListArgs list_args(gm_ctx *c) {
    ListArgs a{};
    a.n = c->n;
    a.n_slots = c->n_slots;
    a.n_sys = c->n_sys;
    a.cap = c->cap;
    a.cap_seg = c->cap_seg;
    a.stage = c->d_stage;
    a.pos = c->d_pos;
    a.coord = c->d_coord;
    a.pos64s = c->d_pos64s;
    a.type_sorted = c->d_type_sorted;
    a.perm = c->d_perm;
    a.slot_of = c->d_slot_of;
    a.cell_of = c->d_cell_of;
    a.cell_sorted = c->d_cell_sorted;
    a.cell_count = c->d_cell_count;
    a.cell_start = c->d_cell_start;
    a.cell_cursor = c->d_cell_cursor;
    a.tmp_atom = c->d_tmp_atom;
    a.type = c->d_type;
    a.qw = c->d_qw;
    a.charge64 = c->d_charge64;
    a.excl_start = c->d_excl_start;
    a.excl = c->d_excl;
    a.list = c->d_list;
    a.count = c->d_count;
    a.gmax = c->d_gmax;
    a.ref = c->d_ref;
    a.force = c->d_force;
    a.grid = c->d_grid;
    a.status = c->d_status;
    a.r_list = c->p.r_skin;
    a.r_cut = c->p.r_cutoff;
    a.r_switch = c->p.r_switch;
    for (int d = 0; d < 3; d++) a.box[d] = c->p.box[d];
    a.periodic = c->p.periodic;
    a.bbox_scratch = c->d_bbox;
    a.bbox_blocks = c->bbox_blocks;
    a.max_sys_atoms = c->max_sys_atoms;
    a.sys_atom_off = c->d_sys_atom_off;
    a.sys_slot_off = c->d_sys_slot_off;
    a.sys_cell_off = c->d_sys_cell_off;
    a.atom_sys = c->d_atom_sys;
    a.group_sys = c->d_group_sys;
    a.sys_flag = c->d_sys_flag;
    return a;
}

// periodic && bonded_min_image: bonded, 1-4 and constraint differences at the
// nearest periodic image
bool bonded_min_image(const gm_ctx *c) { return c->p.periodic && c->p.bonded_min_image; }

ForceArgs force_args(gm_ctx *c) {
    ForceArgs a{};
    a.n = c->n;
    a.n_groups = c->n_groups;
    a.n_slots = c->n_slots;
    a.group_sys = c->d_group_sys;
    a.atom_sys = c->d_atom_sys;
    a.e_sys = c->n_sys > 1 ? c->d_e_sys : nullptr;
    a.cap = c->cap;
    a.split = c->split;
    a.pair_warps = c->pair_warps;
    a.pair_grid = c->pair_grid;
    a.coord = c->d_coord;
    a.pos64s = c->d_pos64s;
    a.type_sorted = c->d_type_sorted;
    a.perm = c->d_perm;
    a.list = c->d_list;
    a.count = c->d_count;
    a.gmax = c->d_gmax;
    a.ntypes = c->ntypes;
    a.tab32 = c->d_tab32;
    a.tab64 = c->d_tab64;
    const double rc = c->p.r_cutoff, rsw = c->p.r_switch;
    a.rc2_64 = rc * rc;
    a.rsw_64 = rsw;
    a.rc_64 = rc;
    a.inv_wsw_64 = 1.0 / (rc - rsw);
    {
        // double-float constants of the mixed pair kernel
        auto split = [](double x, float &h, float &l) { h = (float)x; l = (float)(x - (double)h); };
        PairConst &k = a.pc;
        k.rc2 = (float)(rc * rc);
        k.rsw2 = (float)(rsw * rsw);
        split(rsw, k.rsw, k.rsw_lo);
        split(1.0 / (rc - rsw), k.inv_w, k.inv_w_lo);
        split(-30.0 / (rc - rsw), k.mds, k.mds_lo);
        for (int d = 0; d < 3; d++) {
            split(c->p.box[d], k.box[d], k.box_lo[d]);
            k.inv_box[d] = (float)(1.0 / c->p.box[d]);
        }
    }
    a.coulomb = c->p.coulomb;
    for (int d = 0; d < 3; d++) {
        a.box[d] = (float)c->p.box[d];
        a.inv_box[d] = (float)(1.0 / c->p.box[d]);
        a.box64[d] = c->p.box[d];
    }
    a.periodic = c->p.periodic;
    a.bonded_mi = bonded_min_image(c);
    a.force = c->d_force;
    a.epart = c->d_epart;
    a.status = c->d_status;
    a.pos = c->d_pos;
    a.n_bonds = c->n_bonds;
    a.n_angles = c->n_angles;
    a.n_diheds = c->n_diheds;
    a.bond_i = c->d_bi; a.bond_j = c->d_bj; a.bond_k = c->d_bk; a.bond_r0 = c->d_br0;
    a.angle_i = c->d_ai; a.angle_j = c->d_aj; a.angle_k = c->d_ak; a.angle_kth = c->d_akth; a.angle_th0 = c->d_ath0;
    a.dihed_i = c->d_di; a.dihed_j = c->d_dj; a.dihed_k = c->d_dk; a.dihed_l = c->d_dl; a.dihed_kphi = c->d_dkphi;
    a.dihed_n = c->d_dn; a.dihed_delta = c->d_ddelta; a.dihed_cs = c->d_dcs;
    a.bonded_blocks = c->bonded_blocks;
    const int pair_parts = c->n_groups * a.split;
    a.epart_bonded = c->d_epart + pair_parts;
    a.n14 = c->n14; a.p14_i = c->d_p14i; a.p14_j = c->d_p14j;
    a.scale14_lj = c->p.scale14_lj; a.scale14_coul = c->p.scale14_coul;
    a.sigma = c->d_sigma; a.epsilon = c->d_eps; a.charge64 = c->d_charge64;
    a.p14par = c->d_p14par;
    a.blocks14 = c->blocks14;
    a.epart14 = c->d_epart + pair_parts + c->bonded_blocks;
    a.energy = c->d_energy;
    a.n_epart_total = pair_parts + c->bonded_blocks + c->blocks14;
    return a;
}

ClusterArgs cluster_args(gm_ctx *c) {
    ClusterArgs a{};
    a.n_clusters = c->n_clusters;
    a.n_single = c->n_single;
    a.n_star_end = c->n_star_end;
    a.n_warp_end = c->n_warp_end;
    a.cl_cstart = c->d_cl_cstart; a.cl_cons = c->d_cl_cons;
    a.cl_astart = c->d_cl_astart; a.cl_atoms = c->d_cl_atoms;
    a.cl_acstart = c->d_cl_acstart; a.cl_acons = c->d_cl_acons;
    a.constr_i = c->d_ci; a.constr_j = c->d_cj; a.constr_dsq = c->d_cdsq;
    a.inv_mass = c->d_inv_mass;
    a.lam = c->d_lam; a.rvec = c->d_rvec;
    a.cl_iters = c->d_cl_iters; a.cl_worst = c->d_cl_worst; a.cl_worst_idx = c->d_cl_worst_idx;
    a.n_constr = c->n_constr;
    a.max_iter = c->p.max_constr_iter;
    a.tol = c->p.constr_tol;
    a.status = c->d_status;
    a.lam_sum = (c->ws_on || c->ws_rec_stride > 0) ? c->d_lam_sum : nullptr;
    a.lam0 = c->ws_on ? c->d_ws_lam0 : nullptr;
    a.mi = bonded_min_image(c);
    for (int d = 0; d < 3; d++) a.box64[d] = c->p.box[d];
    return a;
}

// SHAKE with the warm start in between the preparation and the iterations
// when a model is enabled, and the training record after it when recording
// (resident steps only).  Returns the number of launches.
long long issue_shake(gm_ctx *c, cudaStream_t s, bool resident) {
    const ClusterArgs a = cluster_args(c);
    long long k = 0;
    gm_launch_shake_prepare(a, c->n, c->d_dref, s); k += 2;
    const bool record = resident && c->ws_rec_stride > 0;
    if (c->ws_on || record) {
        WsFeatureArgs f{};
        f.n_constr = c->n_constr; f.n_atoms = c->n;
        f.constr_i = c->d_ci; f.constr_j = c->d_cj; f.constr_dsq = c->d_cdsq; f.inv_mass = c->d_inv_mass;
        f.atom_cstart = c->d_atom_cstart; f.atom_cref = c->d_atom_cref; f.pos = c->d_pos; f.dref = c->d_dref;
        f.feat = c->d_ws_feat; f.scale = c->d_ws_scale; f.t1 = c->d_ws_t1; f.unit = c->d_ws_unit; f.w = c->d_ws_w;
        gm_launch_ws_predict(f, c->d_ws_packed, c->d_ws_lam0, c->ws_on, s);
        k += 2;
    }
    k += gm_launch_shake_solve(a, c->n, c->d_pos, s);
    if (record) {
        gm_launch_ws_record(c->n_constr, c->d_ws_feat, c->d_lam_sum, c->d_ws_scale, c->d_ws_t1, c->d_rec_feat,
                            c->d_rec_t, c->ws_rec_stride, c->ws_rec_cap, c->d_status, s);
        k += 2;
    }
    return k;
}

// ---- kernel sequences (each counted for gm_counters[3]) -------------------

// The list rebuild of every system (all) or of the systems the rebuild check
// flagged; the flags are cleared at the end.
int seq_rebuild(gm_ctx *c, cudaStream_t s, bool all) {
    ListArgs a = list_args(c);
    if (all) gm_launch_flags(a, true, s);
    gm_launch_wrap(a, c->d_pos, s);
    gm_launch_grid(a, s);
    gm_launch_bin(a, s);
    gm_launch_pack(a, c->fp64, s);
    gm_launch_build(a, s);
    gm_launch_flags(a, false, s);
    // [flags], wrap or bbox, grid (clears the cells), assign, scan, scatter,
    // rank, pack, build, clear flags
    return (all ? 1 : 0) + 9 + (a.periodic || a.n > 0 ? 1 : 0);
}

bool persistent_form(const gm_ctx *c);
int persistent_grid(gm_ctx *c);

// Mixed-precision contexts in the persistent step form (the default)
// evaluate forces with the persistent kernel's force phase, constrained ones
// too: the phase only evaluates forces.
bool force_phase(const gm_ctx *c) { return c->step_form == GM_STEP_PERSISTENT && !c->fp64 && c->n > 0; }

// Force evaluation at the resident positions: the persistent kernel's force
// phase (force_phase), or the pair kernel with the bonded and 1-4 kernels.
// With a branch stream those run on it beside the pair kernel: every force
// and per-system energy sum is an integer sum and every energy partial has its
// own slot, so the order in which the branches add changes no bit.  Without
// `energy` the partials stay unsummed (energy_stale) until refresh_energy.
// `packed`: the step kernel before it already packed the coordinates.
int seq_forces(gm_ctx *c, cudaStream_t s, bool energy = true, cudaStream_t branch = nullptr, bool packed = false) {
    ListArgs la = list_args(c);
    if (c->n_sys > 1) cudaMemsetAsync(c->d_e_sys, 0, sizeof(long long) * (size_t)c->n_sys, s);
    if (!packed) gm_launch_pack(la, c->fp64, s);
    ForceArgs fa = force_args(c);
    if (force_phase(c) && persistent_grid(c) == GM_OK) {
        // the persistent kernel's force phase: the pair items and the bonded
        // / 1-4 blocks from one queue, one launch, the same sums and energy
        // partials as the kernels below; the queue words start cleared (a
        // step launch that gave up at its barrier leaves them set)
        cudaMemsetAsync(c->d_sync, 0, sizeof(StepSync), s);
        gm_launch_forces_persistent(fa, c->d_sync, c->persist_blocks, s);
        if (energy) gm_launch_energy(fa, s);
        c->energy_stale = !energy;
        return (packed ? 0 : 1) + 1 + (energy ? 1 : 0);
    }
    const bool fork = branch && (c->bonded_blocks || c->blocks14);
    const cudaStream_t sb = fork ? branch : s;
    if (fork) {
        cudaEventRecord(c->ev_fork, s);
        cudaStreamWaitEvent(branch, c->ev_fork, 0);
    }
    gm_launch_bonded_pair14(fa, c->fp64, sb);
    gm_launch_pair(fa, c->fp64, s);
    if (fork) {
        cudaEventRecord(c->ev_join, branch);
        cudaStreamWaitEvent(s, c->ev_join, 0);
    }
    if (energy) gm_launch_energy(fa, s);
    c->energy_stale = !energy;
    return (packed ? 0 : 1) + (c->bonded_blocks || c->blocks14 ? 1 : 0) + 1 + (energy ? 1 : 0);
}

PackArgs pack_args(gm_ctx *c) {
    PackArgs p{};
    p.coord = c->d_coord;
    p.pos64s = c->d_pos64s;
    p.type_sorted = c->d_type_sorted;
    p.slot_of = c->d_slot_of;
    p.grid = c->d_grid;
    p.type = c->d_type;
    p.qw = c->d_qw;
    p.charge64 = c->d_charge64;
    p.fp64 = c->fp64 ? 1 : 0;
    return p;
}

// Sum the energy partials of the last force evaluation into d_energy.
void refresh_energy(gm_ctx *c) {
    if (!c->energy_stale) return;
    gm_launch_energy(force_args(c), c->stream);
    c->launches++;
    c->energy_stale = false;
}

int check_status(gm_ctx *c, gm_convergence *conv);

// DevStatus travels through the pinned h_status on the context's own stream
// (the stream is non-blocking, so legacy-stream copies would not be ordered).
int st_read(gm_ctx *c) {
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    GM_CUDA(c, cudaMemcpyAsync(c->h_status, c->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->stream));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

int st_write(gm_ctx *c) {
    GM_CUDA(c, cudaMemcpyAsync(c->d_status, c->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, c->stream));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

// Clears error and per-call fields; keeps the rebuild counter and the step.
int reset_status(gm_ctx *c) {
    int rc = st_read(c);
    if (rc) return rc;
    DevStatus z{};
    z.fail_step = ~0ull;
    z.n_rebuilds = c->h_status->n_rebuilds;
    z.step = c->h_status->step;
    z.c_steps = c->h_status->c_steps;
    z.shake_sum = c->h_status->shake_sum;
    z.rattle_sum = c->h_status->rattle_sum;
    z.rec_n = c->h_status->rec_n;
    z.rebuild_base = c->h_status->rebuild_base;
    z.frame_n = c->h_status->frame_n;
    z.frame_lost = c->h_status->frame_lost;
    *c->h_status = z;
    return st_write(c);
}

int set_step(gm_ctx *c, uint64_t step) {
    int rc = st_read(c);
    if (rc) return rc;
    c->h_status->step = step;
    return st_write(c);
}

int fill_convergence(gm_ctx *c, bool rattle, gm_convergence *conv) {
    // the reference's worst constraint of the last iteration: max |lambda|,
    // smallest constraint index on ties (constraint.rs:123-127, 144-151)
    std::vector<double> w((size_t)c->n_clusters);
    std::vector<int> wi((size_t)c->n_clusters);
    GM_CUDA(c, cudaMemcpy(w.data(), c->d_cl_worst, sizeof(double) * w.size(), cudaMemcpyDeviceToHost));
    GM_CUDA(c, cudaMemcpy(wi.data(), c->d_cl_worst_idx, sizeof(int) * wi.size(), cudaMemcpyDeviceToHost));
    double best = 0.0;
    int bi = -1;
    for (size_t k = 0; k < w.size(); k++) {
        if (bi < 0 || w[k] > best || (w[k] == best && wi[k] < bi)) {
            best = w[k];
            bi = wi[k];
        }
    }
    if (bi < 0) bi = 0;
    if (conv) {
        conv->step = c->h_status->fail_step == ~0ull ? c->h_status->step : c->h_status->fail_step;
        conv->constraint_idx = bi;
        conv->atom_i = c->h_ci.empty() ? 0 : c->h_ci[(size_t)bi];
        conv->atom_j = c->h_cj.empty() ? 0 : c->h_cj[(size_t)bi];
        conv->residual = best;
        conv->max_iter = c->p.max_constr_iter;
    }
    return fail(c, GM_ERR_CONVERGENCE,
                "%s failed to converge for constraint %d (atoms %lld, %lld) at step %llu: residual %g after %u "
                "iterations",
                rattle ? "velocity constraint solver" : "constraint solver", bi,
                (long long)(conv ? conv->atom_i : 0), (long long)(conv ? conv->atom_j : 0),
                (unsigned long long)(conv ? conv->step : 0), best, c->p.max_constr_iter);
}

// The status word as the stream left it, read by the caller into h_status:
// the reference's error for the first device failure it records.
int status_result(gm_ctx *c, gm_convergence *conv) {
    const unsigned e = c->h_status->error;
    c->last_shake_T = c->h_status->shake_T;
    c->last_rattle_T = c->h_status->rattle_T;
    if (!e) return GM_OK;
    if (e & GM_DEV_LIST_OVERFLOW) return fail(c, GM_ERR_LIST_OVERFLOW, "neighbour list capacity %d exceeded", c->cap);
    if (e & GM_DEV_NONFINITE_POS)
        return fail(c, GM_ERR_NONFINITE, "non-finite position at step %llu", (unsigned long long)c->h_status->step);
    if (e & GM_DEV_SHAKE_FAIL) return fill_convergence(c, false, conv);
    if (e & GM_DEV_RATTLE_FAIL) return fill_convergence(c, true, conv);
    if (e & GM_DEV_NONFINITE_FORCE)
        return fail(c, GM_ERR_NONFINITE, "non-finite force at step %llu", (unsigned long long)c->h_status->step);
    if (e & GM_DEV_FIX_OVERFLOW)
        return fail(c, GM_ERR_FIXED_POINT_OVERFLOW, "a force contribution exceeded the fixed-point range (|F| >= 2^22)");
    if (e & GM_DEV_EXTENT)
        return fail(c, GM_ERR_UNSUPPORTED,
                    "non-periodic system extent plus the list radius reaches half the box: the reference's "
                    "min-image would fold pairs; use a larger box");
    if (e & GM_DEV_CELL_OVERFLOW) return fail(c, GM_ERR_UNSUPPORTED, "cell grid overflow");
    if (e & GM_DEV_BARRIER_TIMEOUT)
        return fail(c, GM_ERR_DEVICE, "a grid barrier of the persistent step kernel timed out");
    if (e & GM_DEV_ITER_MISMATCH)
        return fail(c, GM_ERR_UNSUPPORTED, "constraint cluster iteration counts disagree with the global stop rule");
    return fail(c, GM_ERR_DEVICE, "device status 0x%x", e);
}

int check_status(gm_ctx *c, gm_convergence *conv) {
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    GM_CUDA(c, cudaGetLastError());
    int rc0 = st_read(c);
    if (rc0) return rc0;
    return status_result(c, conv);
}

// The list (cap entries per atom) and the list build's staging area (GM_NSEG
// z layers of cap_seg entries per atom).
int ensure_list_buffers(gm_ctx *c, int cap, int cap_seg) {
    if (cap == c->cap && cap_seg == c->cap_seg && c->d_list && c->d_stage) return GM_OK;
    if (cap != c->cap || !c->d_list) {
        dfree(c, c->d_list);
        c->d_list = nullptr;
        c->cap = cap;
        int rc = dalloc(c, &c->d_list, (size_t)c->n_groups * 32 * (size_t)cap);
        if (rc) return rc;
    }
    if (cap_seg != c->cap_seg || !c->d_stage) {
        dfree(c, c->d_stage);
        c->d_stage = nullptr;
        c->cap_seg = cap_seg;
        int rc = dalloc(c, &c->d_stage, (size_t)c->n_groups * GM_NSEG * 32 * (size_t)cap_seg);
        if (rc) return rc;
    }
    // captured graphs hold the old pointer
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
    return GM_OK;
}

int round32(double x) { return std::max(((int)std::ceil(x) + 31) / 32 * 32, 32); }

// List capacity from the densest system's mean density, and the staging
// capacity of one z layer: a layer of cells about half the list radius thick
// through the middle of the sphere holds ~37 % of it.
int ensure_estimated_buffers(gm_ctx *c, const double *px, const double *py, const double *pz) {
    // densest system: its atoms over its bounding box (or the periodic box)
    double est = 32.0;
    const double rl = c->p.r_skin;
    for (int sy = 0; sy < c->n_sys; sy++) {
        const int a0 = c->h_atom_off[(size_t)sy], a1 = c->h_atom_off[(size_t)sy + 1];
        double vol;
        if (c->p.periodic) vol = c->p.box[0] * c->p.box[1] * c->p.box[2];
        else {
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            const double *P[3] = {px, py, pz};
            for (int i = a0; i < a1; i++)
                for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], P[d][i]); hi[d] = std::max(hi[d], P[d][i]); }
            vol = 1.0;
            for (int d = 0; d < 3; d++) vol *= std::max(hi[d] - lo[d], 2.0);
        }
        const double rho = (a1 - a0) / std::max(vol, 1.0);
        double e = 1.35 * (4.0 / 3.0) * M_PI * rl * rl * rl * rho + 48.0;
        e = std::min(e, (double)(a1 - a0) + 32.0);
        est = std::max(est, e);
    }
    return ensure_list_buffers(c, round32(est), round32(0.45 * (est - 48.0) + 48.0));
}

int do_build(gm_ctx *c, bool all = true) {
    // list build on the resident positions (every system, or the flagged
    // ones), growing the capacity on overflow (then rebuilding every system)
    unsigned long long r0 = 0, counted = 0;
    for (int attempt = 0; attempt < 6; attempt++) {
        int rc = reset_status(c);
        if (rc) return rc;
        if (attempt == 0) r0 = c->h_status->n_rebuilds;
        c->launches += seq_rebuild(c, c->stream, all || attempt > 0);
        rc = check_status(c, nullptr);
        if (attempt == 0) counted = c->h_status->n_rebuilds - r0;
        // the build records the longest list and staged layer it met: on an
        // overflow, or (when every system was built) within 20 % of a
        // capacity, since a resident run cannot grow the list, grow that
        // capacity to a third above the need
        const int need = (int)c->h_status->max_count, need_l = (int)c->h_status->max_layer;
        const bool over = rc == GM_ERR_LIST_OVERFLOW;
        const bool room = !rc && (all || attempt > 0);
        const bool grow = need > (over ? c->cap : c->cap - c->cap / 5);
        const bool grow_l = need_l > (over ? c->cap_seg : c->cap_seg - c->cap_seg / 5);
        if ((over || room) && (grow || grow_l)) {
            rc = ensure_list_buffers(c, grow ? round32(std::max(need + need / 3 + 32, c->cap + 32)) : c->cap,
                                     grow_l ? round32(std::max(need_l + need_l / 3 + 32, c->cap_seg + 32)) : c->cap_seg);
            if (rc) return rc;
            continue;
        }
        if (rc) return rc;
        if (attempt > 0) {
            // capacity rebuilds are not list rebuilds: count the first attempt's
            c->h_status->n_rebuilds = r0 + counted;
            rc = st_write(c);
            if (rc) return rc;
        }
        c->built = true;
        c->forces_current = false;
        return GM_OK;
    }
    return fail(c, GM_ERR_LIST_OVERFLOW, "neighbour list capacity could not be sized");
}

// Host rows in one contiguous x|y|z block (the caller's 3 x N array) go in
// one copy; separate rows in three.
int upload3(gm_ctx *c, double *dst, const double *x, const double *y, const double *z, cudaStream_t s = nullptr) {
    const size_t b = sizeof(double) * (size_t)c->n;
    if (!c->n) return GM_OK;
    if (!s) s = c->stream;
    if (y == x + c->n && z == y + c->n) {
        GM_CUDA(c, cudaMemcpyAsync(dst, x, 3 * b, cudaMemcpyHostToDevice, s));
        return GM_OK;
    }
    GM_CUDA(c, cudaMemcpyAsync(dst, x, b, cudaMemcpyHostToDevice, s));
    GM_CUDA(c, cudaMemcpyAsync(dst + c->n, y, b, cudaMemcpyHostToDevice, s));
    GM_CUDA(c, cudaMemcpyAsync(dst + 2 * c->n, z, b, cudaMemcpyHostToDevice, s));
    return GM_OK;
}

int download3(gm_ctx *c, const double *src, double *x, double *y, double *z, cudaStream_t s = nullptr) {
    const size_t b = sizeof(double) * (size_t)c->n;
    if (!c->n) return GM_OK;
    if (!s) s = c->stream;
    if (x && y == x + c->n && z == y + c->n) {
        GM_CUDA(c, cudaMemcpyAsync(x, src, 3 * b, cudaMemcpyDeviceToHost, s));
        return GM_OK;
    }
    if (x) GM_CUDA(c, cudaMemcpyAsync(x, src, b, cudaMemcpyDeviceToHost, s));
    if (y) GM_CUDA(c, cudaMemcpyAsync(y, src + c->n, b, cudaMemcpyDeviceToHost, s));
    if (z) GM_CUDA(c, cudaMemcpyAsync(z, src + 2 * c->n, b, cudaMemcpyDeviceToHost, s));
    return GM_OK;
}

// The persistent form runs unconstrained mixed-precision steps without
// trajectory frames (frames record each step's energy, which its launches do
// not sum).
bool persistent_form(const gm_ctx *c) {
    return c->step_form == GM_STEP_PERSISTENT && !c->fp64 && c->n_clusters == 0 && c->frame_interval == 0 &&
           c->n > 0;
}

// Before the first persistent launch of a call: clear the barrier and queue
// words.  `fresh`: the force sums hold the forces at the resident positions
// (the first launch skips its force phase); otherwise they are zeroed and
// the first launch evaluates them (timed steps each evaluate their forces).
int persistent_grid(gm_ctx *c) {
    if (c->persist_blocks) return GM_OK;
    c->persist_blocks = gm_step_persistent_blocks(force_args(c));
    if (c->persist_blocks > 0) return GM_OK;
    c->persist_blocks = 0;
    return fail(c, GM_ERR_DEVICE, "persistent step kernel: no block fits on an SM");
}

int begin_persistent(gm_ctx *c, bool fresh) {
    int rc = persistent_grid(c);
    if (rc) return rc;
    GM_CUDA(c, cudaMemsetAsync(c->d_sync, 0, sizeof(StepSync), c->stream));
    if (c->stall_barrier) {
        // the arrival count starts far past the grid: no block is the last to
        // arrive, every block waits out the poll limit and reports the timeout
        GM_CUDA(c, cudaMemsetAsync(&c->d_sync->arrive, 0x40, sizeof(unsigned int), c->stream));
        c->stall_barrier = false;
    }
    if (fresh) GM_CUDA(c, cudaMemsetAsync(&c->d_sync->fresh, 1, 1, c->stream));
    else GM_CUDA(c, cudaMemsetAsync(c->d_force, 0, sizeof(long long) * 3 * (size_t)c->n, c->stream));
    return GM_OK;
}

// After the last persistent launch of a call: the forces at the final
// positions, by the force phase alone (the launches left the coordinates
// packed).
int end_persistent(gm_ctx *c) {
    c->launches += seq_forces(c, c->stream, false, c->side, true);
    GM_CUDA(c, cudaGetLastError());
    return GM_OK;
}

// One BAB + RATTLE step (lib.rs:292-323) issued on stream s.  With a graph
// conditional handle the rebuild runs inside an IF node; otherwise the check
// result is read back on the host.
int issue_step(gm_ctx *c, cudaStream_t s, double dt, unsigned long long cond, long long *count) {
    long long k = 0;
    const int n = c->n;
    const bool constrained = c->n_clusters > 0;
    const double half_skin = (c->p.r_skin - c->p.r_cutoff) / 2.0;  // neighbor.rs:61-62
    if (persistent_form(c)) {
        // forces at the resident positions, kick, drift, check and pack in
        // one launch; the rebuild follows in the IF node
        StepArgs sa{};
        sa.n = n;
        sa.pos = c->d_pos;
        sa.vel = c->d_vel;
        sa.dref = c->d_dref;
        sa.inv_mass = c->d_inv_mass;
        sa.ref = c->d_ref;
        sa.dt_half = dt / 2.0;
        sa.dt = dt;
        sa.inv_dt = 1.0 / dt;
        sa.thr_sq = half_skin * half_skin;
        sa.cond = cond;
        sa.atom_sys = c->d_atom_sys;
        sa.sys_flag = c->d_sys_flag;
        sa.sync = c->d_sync;
        gm_launch_step_persistent(force_args(c), sa, pack_args(c), c->persist_blocks, s);
        *count += 1;
        return GM_OK;
    }
    if (!constrained) {
        gm_launch_kick_drift_check(n, c->d_pos, c->d_vel, c->d_dref, c->d_force, c->d_inv_mass, dt / 2.0, dt, c->d_ref,
                                   half_skin * half_skin, c->d_status, cond, c->d_atom_sys, c->d_sys_flag,
                                   pack_args(c), s);
        *count += 1;
        return GM_OK;
    }
    gm_launch_half_kick(n, c->d_vel, c->d_force, c->d_inv_mass, dt / 2.0, c->d_status, s); k++;
    gm_launch_drift(n, c->d_pos, c->d_vel, c->d_dref, dt, false, c->d_status, s); k++;
    k += issue_shake(c, s, true);
    gm_launch_resync(n, c->d_pos, c->d_vel, c->d_dref, dt, c->d_status, s); k++;
    gm_launch_check(n, c->d_pos, c->d_ref, half_skin * half_skin, c->d_status, cond, gm_check_blocks(n), c->d_atom_sys,
                    c->d_sys_flag, s);
    k++;
    *count += k;
    return GM_OK;
}

int issue_step_tail(gm_ctx *c, cudaStream_t s, double dt, long long *count) {
    if (persistent_form(c)) return GM_OK;  // the next launch evaluates the forces
    long long k = seq_forces(c, s, false, c->side, c->n_clusters == 0);
    if (c->n_clusters) {
        gm_launch_half_kick(c->n, c->d_vel, c->d_force, c->d_inv_mass, dt / 2.0, c->d_status, s); k++;
        gm_launch_rattle(cluster_args(c), c->n, c->d_pos, c->d_vel, s); k += 3;
        gm_launch_step(c->d_status, s); k++;
    }
    // (without constraints the closing half-kick is done by the next step's
    // first kernel, or by finish_steps after the last step)
    if (c->frame_interval > 0) {
        // the energy partials of this step's forces, summed by the frame kernel
        ForceArgs fa = force_args(c);
        FrameArgs f{};
        f.interval = c->frame_interval;
        f.cap = c->frame_cap;
        f.xyz = c->d_frame_xyz;
        f.step = c->d_frame_step;
        f.energy = c->d_frame_energy;
        f.partial = c->d_frame_part;
        f.epart = fa.epart;
        f.n_epart = fa.n_epart_total;
        gm_launch_frame(c->n, c->d_pos, c->d_vel, c->d_force, c->d_inv_mass, c->d_mass, dt / 2.0, c->d_status, f, s);
        k++;
    }
    *count += k;
    return GM_OK;
}

int capture_graph(gm_ctx *c, double dt) {
    if (c->graph_exec && c->graph_dt == dt && c->graph_cap == c->cap) return GM_OK;
    if (force_phase(c)) {
        int rc = persistent_grid(c);  // the grid size goes into the captured launches
        if (rc) return rc;
    }
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
    cudaGraph_t g;
    GM_CUDA(c, cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    GM_CUDA(c, cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    GM_CUDA(c, cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    long long count = 0;
    issue_step(c, c->stream, dt, (unsigned long long)h, &count);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t ndeps = 0;
    cudaGraph_t capg = nullptr;
    GM_CUDA(c, cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &capg, &deps, &edges, &ndeps));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    GM_CUDA(c, cudaGraphAddNode(&cnode, capg, deps, edges, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    GM_CUDA(c, cudaStreamBeginCaptureToGraph(c->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    seq_rebuild(c, c->side, false);
    GM_CUDA(c, cudaStreamEndCapture(c->side, &body));
    GM_CUDA(c, cudaStreamUpdateCaptureDependencies(c->stream, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    issue_step_tail(c, c->stream, dt, &count);
    GM_CUDA(c, cudaStreamEndCapture(c->stream, &g));
    GM_CUDA(c, cudaGraphInstantiate(&c->graph_exec, g, 0));
    c->graph = g;
    c->graph_dt = dt;
    c->graph_cap = c->cap;
    c->launches_per_step = count;
    return GM_OK;
}

// After the last resident step of a call: the closing half-kick that the
// unconstrained step leaves to the next step (nothing pending otherwise).
int finish_steps(gm_ctx *c, double dt) {
    if (c->n_clusters) return GM_OK;
    gm_launch_kick_tail(c->n, c->d_vel, c->d_force, c->d_inv_mass, dt / 2.0, c->d_status, c->stream);
    c->launches++;
    GM_CUDA(c, cudaGetLastError());
    return GM_OK;
}

int run_direct(gm_ctx *c, double dt, int64_t n_steps);

// n resident steps (one graph launch each, or direct launches), then the
// closing half-kick; nothing waits for the device.
// The steps themselves: after them the resident positions are final (the
// rest of the call evaluates forces and the closing half-kick).
int launch_loop(gm_ctx *c, double dt, int64_t n_steps) {
    const bool pf = persistent_form(c) && n_steps > 0;
    int rc = pf ? begin_persistent(c, true) : GM_OK;
    if (rc) return rc;
    if (!c->use_graph) {
        rc = run_direct(c, dt, n_steps);
    } else {
        rc = capture_graph(c, dt);
        if (rc) return rc;
        for (int64_t k = 0; k < n_steps; k++) GM_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
        c->launches += c->launches_per_step * n_steps;
    }
    // the steps' force evaluations leave the energy partials unsummed (the
    // flag that seq_forces sets is set only when a graph is captured)
    if (n_steps > 0) c->energy_stale = true;
    return rc;
}

// After launch_loop: the persistent form's forces at the final positions,
// then the pending closing half-kick.
int launch_end(gm_ctx *c, double dt, int64_t n_steps) {
    int rc = persistent_form(c) && n_steps > 0 ? end_persistent(c) : GM_OK;
    return rc ? rc : finish_steps(c, dt);
}

int launch_steps(gm_ctx *c, double dt, int64_t n_steps) {
    int rc = launch_loop(c, dt, n_steps);
    return rc ? rc : launch_end(c, dt, n_steps);
}

// Caller positions into the context.  When the resident forces are current
// and the caller hands back the resident positions (bit for bit), the forces
// stay valid; one read of the device's comparison decides.
// `cleared`: the status word's comparison flag is zero already (the status
// reset kernel ran on the stream).
int stage_positions(gm_ctx *c, const double *px, const double *py, const double *pz, bool cleared = false) {
    if (!c->forces_current) return upload3(c, c->d_pos, px, py, pz);
    int rc = upload3(c, c->d_dref, px, py, pz);
    if (rc) return rc;
    if (!cleared) GM_CUDA(c, cudaMemsetAsync(&c->d_status->differs, 0, sizeof(unsigned int), c->stream));
    gm_launch_differs(c->n, c->d_dref, c->d_pos, &c->d_status->differs, c->stream);
    c->launches++;
    GM_CUDA(c, cudaMemcpyAsync(&c->h_status->differs, &c->d_status->differs, sizeof(unsigned int),
                               cudaMemcpyDeviceToHost, c->stream));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->h_status->differs & 2u) return fail(c, GM_ERR_NONFINITE, "non-finite position");
    if (c->h_status->differs) {
        c->forces_current = false;
        GM_CUDA(c, cudaMemcpyAsync(c->d_pos, c->d_dref, sizeof(double) * 3 * (size_t)c->n, cudaMemcpyDeviceToDevice,
                                   c->stream));
    }
    return GM_OK;
}

// The step without a graph: same kernels on the stream, the rebuild decision
// read back on the host after each check (profilers cannot look inside
// graphs that hold conditional nodes).
int run_direct(gm_ctx *c, double dt, int64_t n_steps) {
    for (int64_t k = 0; k < n_steps; k++) {
        long long count = 0;
        issue_step(c, c->stream, dt, 0ull, &count);
        int rc = st_read(c);
        if (rc) return rc;
        if (c->h_status->rebuild && !c->h_status->error) count += seq_rebuild(c, c->stream, false);
        issue_step_tail(c, c->stream, dt, &count);
        c->launches += count;
    }
    return GM_OK;
}

int ensure_forces(gm_ctx *c) {
    // the first half-kick of a step needs forces at the current positions;
    // an existing list stays valid while no atom moved more than half the
    // skin from its build position (neighbor.rs:60-72)
    if (c->forces_current) return GM_OK;
    if (!c->built) {
        int rc = do_build(c);
        if (rc) return rc;
    } else {
        int rc = reset_status(c);
        if (rc) return rc;
        const double half_skin = (c->p.r_skin - c->p.r_cutoff) / 2.0;
        gm_launch_check(c->n, c->d_pos, c->d_ref, half_skin * half_skin, c->d_status, 0ull, gm_check_blocks(c->n),
                        c->d_atom_sys, c->d_sys_flag,
                        c->stream);
        c->launches++;
        rc = st_read(c);
        if (rc) return rc;
        if (c->h_status->error & GM_DEV_NONFINITE_POS) return fail(c, GM_ERR_NONFINITE, "non-finite position");
        if (c->h_status->rebuild) {
            rc = do_build(c, false);  // the flagged systems
            if (rc) return rc;
        }
    }
    c->launches += seq_forces(c, c->stream);
    c->forces_current = true;
    return GM_OK;
}

void build_clusters(gm_ctx *c, const std::vector<int> &ci, const std::vector<int> &cj, std::vector<int> &cstart,
                    std::vector<int> &cons, std::vector<int> &astart, std::vector<int> &atoms,
                    std::vector<int> &acstart, std::vector<int> &acons) {
    // connected components of the constraint graph (union-find over atoms)
    const int nc = (int)ci.size();
    std::vector<int> parent((size_t)c->n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int x) {
        while (parent[(size_t)x] != x) { parent[(size_t)x] = parent[(size_t)parent[(size_t)x]]; x = parent[(size_t)x]; }
        return x;
    };
    for (int k = 0; k < nc; k++) {
        int a = find(ci[(size_t)k]), b = find(cj[(size_t)k]);
        if (a != b) parent[(size_t)std::max(a, b)] = std::min(a, b);
    }
    std::map<int, int> root_id;
    std::vector<std::vector<int>> ccons, catoms;
    for (int k = 0; k < nc; k++) {
        int r = find(ci[(size_t)k]);
        auto it = root_id.find(r);
        if (it == root_id.end()) { it = root_id.emplace(r, (int)ccons.size()).first; ccons.emplace_back(); catoms.emplace_back(); }
        ccons[(size_t)it->second].push_back(k);  // ascending k
    }
    // clusters in four classes, in this order: one constraint on two atoms
    // (one per thread), stars of 2-8 constraints on one centre atom (one per
    // thread), other clusters of 2-32 constraints on at most 32 atoms with at
    // most 8 constraints per atom (one per warp), the rest; within a class by
    // size (stable), so a warp's threads run loops of the same lengths.  The
    // solution does not depend on the cluster order.
    const size_t ncl = ccons.size();
    std::vector<int> cls(ncl);
    for (size_t q = 0; q < ncl; q++) {
        std::vector<int> at, deg;
        for (int k : ccons[q]) { at.push_back(ci[(size_t)k]); at.push_back(cj[(size_t)k]); }
        std::sort(at.begin(), at.end());
        int maxdeg = 0, run = 0;
        for (size_t t = 0; t < at.size(); t++) {
            run = (t > 0 && at[t] == at[t - 1]) ? run + 1 : 1;
            maxdeg = std::max(maxdeg, run);
        }
        at.erase(std::unique(at.begin(), at.end()), at.end());
        const int nc = (int)ccons[q].size(), na = (int)at.size();
        // a star: every constraint shares one centre atom, the others are distinct
        bool star = nc >= 2 && nc <= 8 && na == nc + 1;
        if (star) {
            const int k0 = ccons[q][0], k1 = ccons[q][1];
            const int cen = (ci[(size_t)k0] == ci[(size_t)k1] || ci[(size_t)k0] == cj[(size_t)k1]) ? ci[(size_t)k0]
                                                                                                   : cj[(size_t)k0];
            for (int k : ccons[q]) star = star && (ci[(size_t)k] == cen || cj[(size_t)k] == cen);
        }
        cls[q] = (nc == 1 && na == 2) ? 0 : star ? 1 : (nc <= 32 && na <= 32 && maxdeg <= 8 ? 2 : 3);
    }
    std::vector<size_t> order(ncl);
    std::iota(order.begin(), order.end(), (size_t)0);
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
        if (cls[x] != cls[y]) return cls[x] < cls[y];
        return ccons[x].size() < ccons[y].size();
    });
    c->n_single = (int)std::count(cls.begin(), cls.end(), 0);
    c->n_star_end = c->n_single + (int)std::count(cls.begin(), cls.end(), 1);
    c->n_warp_end = c->n_star_end + (int)std::count(cls.begin(), cls.end(), 2);
    cstart.assign(1, 0);
    astart.assign(1, 0);
    acstart.assign(1, 0);
    cons.clear(); atoms.clear(); acons.clear();
    for (size_t q : order) {
        std::vector<int> at;
        for (int k : ccons[q]) { at.push_back(ci[(size_t)k]); at.push_back(cj[(size_t)k]); }
        std::sort(at.begin(), at.end());
        at.erase(std::unique(at.begin(), at.end()), at.end());
        for (int k : ccons[q]) cons.push_back(k);
        cstart.push_back((int)cons.size());
        for (int a : at) {
            atoms.push_back(a);
            for (int k : ccons[q]) {
                // per atom, its constraints in ascending order; i side negative
                if (ci[(size_t)k] == a) acons.push_back(-k - 1);
                if (cj[(size_t)k] == a) acons.push_back(k);
            }
            acstart.push_back((int)acons.size());
        }
        astart.push_back((int)atoms.size());
    }
}

}  // namespace

// ===================================================================== C ABI

namespace {

void drop_graph(gm_ctx *c) {
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
}

int ws_alloc_model(gm_ctx *c) {
    if (c->d_ws_params) return GM_OK;
    int rc = dalloc(c, &c->d_ws_params, GM_WS_NPAR);
    if (!rc) rc = dalloc(c, &c->d_ws_norm, GM_WS_NNORM);
    if (!rc) rc = dalloc(c, &c->d_ws_packed, gm_ws_packed_bytes());
    if (!rc) rc = dalloc(c, &c->d_ws_m, GM_WS_NPAR);
    if (!rc) rc = dalloc(c, &c->d_ws_v, GM_WS_NPAR);
    if (!rc) rc = dalloc(c, &c->d_ws_out, GM_WS_NPAR + 1);
    if (!rc) rc = dalloc(c, &c->d_ws_stats, 26 * 256);
    return rc;
}

int ws_partial(gm_ctx *c, int blocks) {
    if (blocks <= c->ws_partial_blocks) return GM_OK;
    dfree(c, c->d_ws_partial);
    c->d_ws_partial = nullptr;
    c->ws_partial_blocks = 0;
    int rc = dalloc(c, &c->d_ws_partial, (size_t)blocks * (GM_WS_NPAR + 1));
    if (!rc) c->ws_partial_blocks = blocks;
    return rc;
}

// Glorot-uniform weights from a splitmix64 stream, zero biases.
void ws_init_params(uint64_t seed, std::vector<float> &P) {
    P.assign(GM_WS_NPAR, 0.0f);
    uint64_t z = seed;
    auto next = [&z]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    };
    auto fill = [&](int off, int fan_in, int fan_out) {
        const double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int k = 0; k < fan_in * fan_out; k++) P[(size_t)(off + k)] = (float)((2.0 * next() - 1.0) * a);
    };
    fill(GM_WS_OFF_W1, GM_WS_IN, GM_WS_H);
    fill(GM_WS_OFF_W2, GM_WS_H, GM_WS_H);
    fill(GM_WS_OFF_W3, GM_WS_H, 1);
}

}  // namespace

namespace {

// Systems of a batch merged into one context: atom arrays concatenated,
// topology indices shifted by each system's first atom.
struct Merged {
    std::vector<int> atom_off;
    std::vector<double> sigma, eps, mass, charge;
    std::vector<uint8_t> element;
    std::vector<uint32_t> bi, bj, ai, aj, ak, di, dj, dk, dl, dn, ci, cj, ei, ej;
    std::vector<double> bk, br0, akth, ath0, dkphi, ddelta, cdsq;
    bool has_element = false;
    gm_atoms A{};
    gm_topology T{};
};

// Returns false when a system's arrays or indices are invalid.
bool merge_systems(int n_sys, const gm_atoms *atoms, const gm_topology *topos, Merged &m) {
    m.atom_off.assign(1, 0);
    for (int s = 0; s < n_sys; s++) {
        const gm_atoms &a = atoms[s];
        if (a.n_atoms < 0 || (a.n_atoms > 0 && (!a.sigma || !a.epsilon || !a.mass))) return false;
        if ((long long)m.atom_off.back() + a.n_atoms > INT32_MAX / 2) return false;
        m.atom_off.push_back(m.atom_off.back() + (int)a.n_atoms);
        if (a.element) m.has_element = true;
    }
    for (int s = 0; s < n_sys; s++) {
        const gm_atoms &a = atoms[s];
        const gm_topology &t = topos[s];
        const uint32_t n = (uint32_t)a.n_atoms, off = (uint32_t)m.atom_off[(size_t)s];
        for (int64_t i = 0; i < a.n_atoms; i++) {
            m.sigma.push_back(a.sigma[i]);
            m.eps.push_back(a.epsilon[i]);
            m.mass.push_back(a.mass[i]);
            m.charge.push_back(a.charge ? a.charge[i] : 0.0);
            m.element.push_back(a.element ? a.element[i] : (uint8_t)1);
        }
        auto idx = [&](const uint32_t *src, int64_t cnt, std::vector<uint32_t> &dst) {
            if (cnt > 0 && !src) return false;
            for (int64_t k = 0; k < cnt; k++) {
                if (src[k] >= n) return false;
                dst.push_back(src[k] + off);
            }
            return true;
        };
        auto val = [](const double *src, int64_t cnt, std::vector<double> &dst) {
            if (cnt > 0 && !src) return false;
            dst.insert(dst.end(), src, src + cnt);
            return true;
        };
        if (t.n_bonds < 0 || t.n_angles < 0 || t.n_diheds < 0 || t.n_constr < 0 || t.n_excl < 0) return false;
        if (!idx(t.bond_i, t.n_bonds, m.bi) || !idx(t.bond_j, t.n_bonds, m.bj) || !val(t.bond_k, t.n_bonds, m.bk) ||
            !val(t.bond_r0, t.n_bonds, m.br0) || !idx(t.angle_i, t.n_angles, m.ai) ||
            !idx(t.angle_j, t.n_angles, m.aj) || !idx(t.angle_k, t.n_angles, m.ak) ||
            !val(t.angle_kth, t.n_angles, m.akth) || !val(t.angle_th0, t.n_angles, m.ath0) ||
            !idx(t.dihed_i, t.n_diheds, m.di) || !idx(t.dihed_j, t.n_diheds, m.dj) ||
            !idx(t.dihed_k, t.n_diheds, m.dk) || !idx(t.dihed_l, t.n_diheds, m.dl) ||
            !val(t.dihed_kphi, t.n_diheds, m.dkphi) || !val(t.dihed_delta, t.n_diheds, m.ddelta) ||
            !idx(t.constr_i, t.n_constr, m.ci) || !idx(t.constr_j, t.n_constr, m.cj) ||
            !val(t.constr_dsq, t.n_constr, m.cdsq) || !idx(t.excl_i, t.n_excl, m.ei) || !idx(t.excl_j, t.n_excl, m.ej))
            return false;
        if (t.n_diheds > 0 && !t.dihed_n) return false;
        m.dn.insert(m.dn.end(), t.dihed_n, t.dihed_n + t.n_diheds);  // a multiplicity, not an index
    }
    const int64_t n = m.atom_off.back();
    m.A = gm_atoms{n, m.sigma.data(), m.eps.data(), m.mass.data(), m.charge.data(),
                   m.has_element ? m.element.data() : nullptr};
    gm_topology &T = m.T;
    T.n_bonds = (int64_t)m.bi.size(); T.bond_i = m.bi.data(); T.bond_j = m.bj.data(); T.bond_k = m.bk.data();
    T.bond_r0 = m.br0.data();
    T.n_angles = (int64_t)m.ai.size(); T.angle_i = m.ai.data(); T.angle_j = m.aj.data(); T.angle_k = m.ak.data();
    T.angle_kth = m.akth.data(); T.angle_th0 = m.ath0.data();
    T.n_diheds = (int64_t)m.di.size(); T.dihed_i = m.di.data(); T.dihed_j = m.dj.data(); T.dihed_k = m.dk.data();
    T.dihed_l = m.dl.data(); T.dihed_kphi = m.dkphi.data(); T.dihed_n = m.dn.data(); T.dihed_delta = m.ddelta.data();
    T.n_constr = (int64_t)m.ci.size(); T.constr_i = m.ci.data(); T.constr_j = m.cj.data(); T.constr_dsq = m.cdsq.data();
    T.n_excl = (int64_t)m.ei.size(); T.excl_i = m.ei.data(); T.excl_j = m.ej.data();
    return true;
}

gm_ctx *create_impl(int n_sys, const gm_atoms *sys_atoms, const gm_topology *sys_topos, const gm_params *params,
                    int32_t *status);

}  // namespace

extern "C" {

gm_ctx *gm_create(const gm_atoms *atoms, const gm_topology *t, const gm_params *params, int32_t *status) {
    return create_impl(1, atoms, t, params, status);
}

gm_ctx *gm_create_ensemble(int32_t n_systems, const gm_atoms *atoms, const gm_topology *topos, const gm_params *params,
                           int32_t *status) {
    return create_impl(n_systems, atoms, topos, params, status);
}

}  // extern "C"

namespace {

gm_ctx *create_impl(int n_sys, const gm_atoms *sys_atoms, const gm_topology *sys_topos, const gm_params *params,
                    int32_t *status) {
    int32_t dummy;
    if (!status) status = &dummy;
    *status = GM_OK;
    Merged mg;
    if (n_sys < 1 || !sys_atoms || !sys_topos || !params || !merge_systems(n_sys, sys_atoms, sys_topos, mg)) {
        *status = GM_ERR_INVALID_ARGUMENT;
        return nullptr;
    }
    const gm_atoms *atoms = &mg.A;
    const gm_topology *t = &mg.T;
    const gm_params &p = *params;
    // config.rs:213-248 validation
    if (!(p.r_switch < p.r_cutoff && p.r_cutoff < p.r_skin) || !(p.box[0] > 0 && p.box[1] > 0 && p.box[2] > 0) ||
        p.max_constr_iter == 0 || !(p.constr_tol > 0) ||
        (p.precision != GM_PRECISION_MIXED && p.precision != GM_PRECISION_FP64)) {
        *status = GM_ERR_INVALID_ARGUMENT;
        return nullptr;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || p.device < 0 || p.device >= ndev) {
        cudaGetLastError();
        *status = GM_ERR_NO_DEVICE;
        return nullptr;
    }
    gm_ctx *c = new gm_ctx();
    c->device = p.device;
    c->p = p;
    c->n = (int)atoms->n_atoms;
    c->fp64 = p.precision == GM_PRECISION_FP64;
    {
        const char *g = getenv("GM_GRAPH");
        c->use_graph = !(g && g[0] == '0');
    }
    const int n = c->n;
    auto bail = [&](int code) -> gm_ctx * {
        // no context survives to carry the message: report it on stderr
        const cudaError_t le = cudaGetLastError();
        fprintf(stderr, "gm_create: status %d (%s; last CUDA error: %s)\n", code,
                c->err.empty() ? "setup failed" : c->err.c_str(), cudaGetErrorString(le));
        *status = code;
        gm_destroy(c);
        return nullptr;
    };
    if (cudaSetDevice(c->device) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (cudaEventCreateWithFlags(&c->ev_xfer_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_xfer_out, cudaEventDisableTiming) != cudaSuccess)
        return bail(GM_ERR_DEVICE);
    if (cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return bail(GM_ERR_DEVICE);
    int rc;
#define TRY(x) do { rc = (x); if (rc) return bail(rc); } while (0)
    // ---- atoms: deduplicate (sigma, epsilon) into types, per system (the
    // systems of a batch never interact, so each has its own type table)
    c->n_sys = n_sys;
    c->h_atom_off = mg.atom_off;
    std::vector<int> type((size_t)n);
    std::vector<std::vector<double>> tsig((size_t)n_sys), teps((size_t)n_sys);
    for (int sy = 0; sy < n_sys; sy++) {
        std::map<std::pair<double, double>, int> types;
        for (int i = mg.atom_off[(size_t)sy]; i < mg.atom_off[(size_t)sy + 1]; i++) {
            auto key = std::make_pair(atoms->sigma[i], atoms->epsilon[i]);
            auto it = types.find(key);
            if (it == types.end()) {
                it = types.emplace(key, (int)tsig[(size_t)sy].size()).first;
                tsig[(size_t)sy].push_back(key.first);
                teps[(size_t)sy].push_back(key.second);
            }
            type[(size_t)i] = it->second;
        }
        c->ntypes = std::max(c->ntypes, std::max((int)tsig[(size_t)sy].size(), 1));
    }
    if (c->ntypes > GM_MAX_TYPES) {
        fail(c, GM_ERR_UNSUPPORTED, "%d distinct (sigma, epsilon) pairs in a system; at most %d are supported",
             c->ntypes, GM_MAX_TYPES);
        return bail(GM_ERR_UNSUPPORTED);
    }
    const size_t T2 = (size_t)c->ntypes * c->ntypes;
    std::vector<float4> tab32(T2 * (size_t)n_sys, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<double2> tab64(T2 * (size_t)n_sys, make_double2(0.0, 0.0));
    for (int sy = 0; sy < n_sys; sy++) {
        const auto &sg_ = tsig[(size_t)sy];
        const auto &ep_ = teps[(size_t)sy];
        for (size_t a = 0; a < sg_.size(); a++)
            for (size_t b = 0; b < sg_.size(); b++) {
                // nonbonded.rs:46-47 Lorentz-Berthelot, evaluated as the reference does
                const double sg = 0.5 * (sg_[a] + sg_[b]);
                const double ep = std::sqrt(ep_[a] * ep_[b]);
                tab64[T2 * (size_t)sy + a * (size_t)c->ntypes + b] = make_double2(sg, ep);
                // the mixed pair kernel's double-float (sigma^2, 24 epsilon)
                const double s2 = sg * sg, e24 = 24.0 * ep;
                const float s2h = (float)s2, e24h = (float)e24;
                tab32[T2 * (size_t)sy + a * (size_t)c->ntypes + b] =
                    make_float4(s2h, (float)(s2 - (double)s2h), e24h, (float)(e24 - (double)e24h));
            }
    }
    std::vector<double> inv_mass((size_t)n), charge64((size_t)n);
    std::vector<float2> qw((size_t)n);
    for (int i = 0; i < n; i++) {
        inv_mass[(size_t)i] = 1.0 / atoms->mass[i];  // integrator.rs:16, constraint.rs:110
        charge64[(size_t)i] = atoms->charge ? atoms->charge[i] : 0.0;
        // Q = sqrt(k_C) q as a double-float, so that Q_i Q_j = k_C q_i q_j
        // (k_C = 332.0522173, the reference's kcal/mol conversion,
        // prmtop.rs:5-9); the low 8 bits of Q_lo carry the atom's type
        const double Q = std::sqrt(332.0522173) * charge64[(size_t)i];
        const float qh = (float)Q, ql = (float)(Q - (double)qh);
        uint32_t bits;
        std::memcpy(&bits, &ql, sizeof bits);
        bits = (bits & ~0xffu) | (uint32_t)type[(size_t)i];
        float qlt;
        std::memcpy(&qlt, &bits, sizeof qlt);
        qw[(size_t)i] = make_float2(qh, qlt);
    }
    TRY(dupload(c, &c->d_mass, atoms->mass, (size_t)n));
    TRY(dupload(c, &c->d_inv_mass, inv_mass.data(), (size_t)n));
    TRY(dupload(c, &c->d_sigma, atoms->sigma, (size_t)n));
    TRY(dupload(c, &c->d_eps, atoms->epsilon, (size_t)n));
    TRY(dupload(c, &c->d_charge64, charge64.data(), (size_t)n));
    TRY(dupload(c, &c->d_qw, qw.data(), (size_t)n));
    TRY(dupload(c, &c->d_type, type.data(), (size_t)n));
    TRY(dupload(c, &c->d_tab32, tab32.data(), tab32.size()));
    TRY(dupload(c, &c->d_tab64, tab64.data(), tab64.size()));
    // ---- exclusions: symmetric CSR, ascending (neighbor.rs:18-23 set semantics)
    std::vector<std::vector<int>> ex((size_t)n);
    for (int64_t e = 0; e < t->n_excl; e++) {
        const uint32_t i = t->excl_i[e], j = t->excl_j[e];
        if ((int64_t)i >= n || (int64_t)j >= n) { fail(c, GM_ERR_INVALID_ARGUMENT, "exclusion %lld out of range", (long long)e); return bail(GM_ERR_INVALID_ARGUMENT); }
        if (i == j) continue;
        ex[i].push_back((int)j);
        ex[j].push_back((int)i);
    }
    std::vector<int> excl_start((size_t)n + 1, 0), excl;
    for (int i = 0; i < n; i++) {
        auto &v = ex[(size_t)i];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        excl.insert(excl.end(), v.begin(), v.end());
        excl_start[(size_t)i + 1] = (int)excl.size();
    }
    TRY(dupload(c, &c->d_excl_start, excl_start.data(), excl_start.size()));
    TRY(dupload(c, &c->d_excl, excl.data(), excl.size()));
    // ---- bonded
    auto check_idx = [&](const uint32_t *a, int64_t cnt) {
        for (int64_t k = 0; k < cnt; k++) if ((int64_t)a[k] >= n) return false;
        return true;
    };
    if (!check_idx(t->bond_i, t->n_bonds) || !check_idx(t->bond_j, t->n_bonds) || !check_idx(t->angle_i, t->n_angles) ||
        !check_idx(t->angle_j, t->n_angles) || !check_idx(t->angle_k, t->n_angles) || !check_idx(t->dihed_i, t->n_diheds) ||
        !check_idx(t->dihed_j, t->n_diheds) || !check_idx(t->dihed_k, t->n_diheds) || !check_idx(t->dihed_l, t->n_diheds) ||
        !check_idx(t->constr_i, t->n_constr) || !check_idx(t->constr_j, t->n_constr)) {
        fail(c, GM_ERR_INVALID_ARGUMENT, "topology index out of range");
        return bail(GM_ERR_INVALID_ARGUMENT);
    }
    c->n_bonds = (int)t->n_bonds;
    c->n_angles = (int)t->n_angles;
    c->n_diheds = (int)t->n_diheds;
    c->bonded_blocks = gm_bonded_blocks(c->n_bonds, c->n_angles, c->n_diheds);
    auto v = [](const uint32_t *a, int64_t cnt) { return to_int(a, cnt); };
    TRY(dupload(c, &c->d_bi, v(t->bond_i, t->n_bonds).data(), (size_t)t->n_bonds));
    TRY(dupload(c, &c->d_bj, v(t->bond_j, t->n_bonds).data(), (size_t)t->n_bonds));
    TRY(dupload(c, &c->d_bk, t->bond_k, (size_t)t->n_bonds));
    TRY(dupload(c, &c->d_br0, t->bond_r0, (size_t)t->n_bonds));
    TRY(dupload(c, &c->d_ai, v(t->angle_i, t->n_angles).data(), (size_t)t->n_angles));
    TRY(dupload(c, &c->d_aj, v(t->angle_j, t->n_angles).data(), (size_t)t->n_angles));
    TRY(dupload(c, &c->d_ak, v(t->angle_k, t->n_angles).data(), (size_t)t->n_angles));
    TRY(dupload(c, &c->d_akth, t->angle_kth, (size_t)t->n_angles));
    TRY(dupload(c, &c->d_ath0, t->angle_th0, (size_t)t->n_angles));
    TRY(dupload(c, &c->d_di, v(t->dihed_i, t->n_diheds).data(), (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_dj, v(t->dihed_j, t->n_diheds).data(), (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_dk, v(t->dihed_k, t->n_diheds).data(), (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_dl, v(t->dihed_l, t->n_diheds).data(), (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_dkphi, t->dihed_kphi, (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_dn, v(t->dihed_n, t->n_diheds).data(), (size_t)t->n_diheds));
    TRY(dupload(c, &c->d_ddelta, t->dihed_delta, (size_t)t->n_diheds));
    {
        std::vector<double2> cs((size_t)t->n_diheds);
        for (int64_t q = 0; q < t->n_diheds; q++)
            cs[(size_t)q] = make_double2(std::cos(t->dihed_delta[q]), std::sin(t->dihed_delta[q]));
        TRY(dupload(c, &c->d_dcs, cs.data(), cs.size()));
    }
    // ---- scaled 1-4 pairs (beyond the reference; off by default)
    if (p.scale14_lj != 0.0 || (p.coulomb && p.scale14_coul != 0.0)) {
        std::vector<std::pair<int, int>> close;
        for (int64_t b = 0; b < t->n_bonds; b++)
            close.emplace_back(std::min(t->bond_i[b], t->bond_j[b]), std::max(t->bond_i[b], t->bond_j[b]));
        for (int64_t a = 0; a < t->n_angles; a++)
            close.emplace_back(std::min(t->angle_i[a], t->angle_k[a]), std::max(t->angle_i[a], t->angle_k[a]));
        std::sort(close.begin(), close.end());
        std::vector<std::pair<int, int>> p14;
        for (int64_t d = 0; d < t->n_diheds; d++) {
            int i = (int)t->dihed_i[d], l = (int)t->dihed_l[d];
            if (i == l) continue;
            auto key = std::make_pair(std::min(i, l), std::max(i, l));
            if (std::binary_search(close.begin(), close.end(), key)) continue;
            p14.push_back(key);
        }
        std::sort(p14.begin(), p14.end());
        p14.erase(std::unique(p14.begin(), p14.end()), p14.end());
        std::vector<int> a((size_t)p14.size()), b((size_t)p14.size());
        for (size_t k = 0; k < p14.size(); k++) { a[k] = p14[k].first; b[k] = p14[k].second; }
        c->n14 = (int)p14.size();
        c->blocks14 = (c->n14 + GM_BONDED_THREADS - 1) / GM_BONDED_THREADS;
        TRY(dupload(c, &c->d_p14i, a.data(), a.size()));
        TRY(dupload(c, &c->d_p14j, b.data(), b.size()));
        // per-pair parameters (force/nonbonded.rs:46-47 mixing; the scales
        // and Coulomb factor applied once)
        std::vector<double4> par(p14.size());
        for (size_t k = 0; k < p14.size(); k++) {
            const int i = a[k], j = b[k];
            const double sg = 0.5 * (atoms->sigma[i] + atoms->sigma[j]);
            const double ep = std::sqrt(atoms->epsilon[i] * atoms->epsilon[j]);
            const double qq = p.coulomb ? 332.0522173 * charge64[(size_t)i] * charge64[(size_t)j] : 0.0;
            par[k] = make_double4(sg, p.scale14_lj * 4.0 * ep, p.scale14_lj * 24.0 * ep, p.scale14_coul * qq);
        }
        TRY(dupload(c, &c->d_p14par, par.data(), par.size()));
    }
    // ---- constraints as independent clusters
    c->n_constr = (int)t->n_constr;
    c->h_ci = v(t->constr_i, t->n_constr);
    c->h_cj = v(t->constr_j, t->n_constr);
    if (c->n_constr) {
        std::vector<int> cstart, cons, astart, cat, acstart, acons;
        build_clusters(c, c->h_ci, c->h_cj, cstart, cons, astart, cat, acstart, acons);
        c->n_clusters = (int)cstart.size() - 1;
        // the kernels index these prefix tables without bounds checks
        if (cstart.empty() || cstart.front() != 0 || cstart.back() != c->n_constr || astart.size() != cstart.size() ||
            astart.front() != 0 || astart.back() != (int)cat.size() || acstart.size() != cat.size() + 1 ||
            acstart.front() != 0 || acstart.back() != (int)acons.size() || c->n_single > c->n_star_end ||
            c->n_star_end > c->n_warp_end || c->n_warp_end > c->n_clusters) {
            fail(c, GM_ERR_DEVICE, "inconsistent constraint cluster tables");
            return bail(GM_ERR_DEVICE);
        }
        TRY(dupload(c, &c->d_ci, c->h_ci.data(), c->h_ci.size()));
        TRY(dupload(c, &c->d_cj, c->h_cj.data(), c->h_cj.size()));
        TRY(dupload(c, &c->d_cdsq, t->constr_dsq, (size_t)c->n_constr));
        TRY(dupload(c, &c->d_cl_cstart, cstart.data(), cstart.size()));
        TRY(dupload(c, &c->d_cl_cons, cons.data(), cons.size()));
        TRY(dupload(c, &c->d_cl_astart, astart.data(), astart.size()));
        TRY(dupload(c, &c->d_cl_atoms, cat.data(), cat.size()));
        TRY(dupload(c, &c->d_cl_acstart, acstart.data(), acstart.size()));
        TRY(dupload(c, &c->d_cl_acons, acons.data(), acons.size()));
        TRY(dalloc(c, &c->d_lam, (size_t)c->n_constr));
        {
            // per-atom constraints, ascending: k where the atom is i, -k-1 where it is j
            std::vector<int> cs((size_t)n + 1, 0), cref(2 * (size_t)c->n_constr);
            for (int k = 0; k < c->n_constr; k++) { cs[(size_t)c->h_ci[(size_t)k] + 1]++; cs[(size_t)c->h_cj[(size_t)k] + 1]++; }
            for (int a = 0; a < n; a++) cs[(size_t)a + 1] += cs[(size_t)a];
            std::vector<int> fill(cs.begin(), cs.end() - 1);
            for (int k = 0; k < c->n_constr; k++) {
                cref[(size_t)fill[(size_t)c->h_ci[(size_t)k]]++] = k;
                cref[(size_t)fill[(size_t)c->h_cj[(size_t)k]]++] = -k - 1;
            }
            TRY(dupload(c, &c->d_atom_cstart, cs.data(), cs.size()));
            TRY(dupload(c, &c->d_atom_cref, cref.data(), cref.size()));
        }
        TRY(dalloc(c, &c->d_lam_sum, (size_t)c->n_constr));
        TRY(dalloc(c, &c->d_ws_lam0, (size_t)c->n_constr));
        TRY(dalloc(c, &c->d_ws_scale, (size_t)c->n_constr));
        TRY(dalloc(c, &c->d_ws_t1, (size_t)c->n_constr));
        TRY(dalloc(c, &c->d_ws_feat, (size_t)GM_WS_IN * c->n_constr));
        TRY(dalloc(c, &c->d_ws_unit, (size_t)c->n_constr));
        {
            // FP32 1/m_i + 1/m_j per constraint, for the warm start's features
            std::vector<float> w((size_t)c->n_constr);
            for (int k = 0; k < c->n_constr; k++)
                w[(size_t)k] = (float)inv_mass[(size_t)c->h_ci[(size_t)k]] + (float)inv_mass[(size_t)c->h_cj[(size_t)k]];
            TRY(dupload(c, &c->d_ws_w, w.data(), w.size()));
        }
        TRY(dalloc(c, &c->d_rvec, 3 * (size_t)c->n_constr));
        TRY(dalloc(c, &c->d_cl_iters, (size_t)c->n_clusters));
        TRY(dalloc(c, &c->d_cl_worst, (size_t)c->n_clusters));
        TRY(dalloc(c, &c->d_cl_worst_idx, (size_t)c->n_clusters));
    }
    // ---- state, sorted copies, cells
    TRY(dalloc(c, &c->d_pos, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_vel, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_ref, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_dref, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_fout, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_host_f, 3 * (size_t)n));
    TRY(dalloc(c, &c->d_force, 3 * (size_t)n));
    // ---- systems: 32-aligned slot ranges, cell budgets, lookup tables
    {
        std::vector<int> slot_off(1, 0), cell_off(1, 0), atom_sys((size_t)n), group_sys;
        long long full_cells = 0;
        for (int sy = 0; sy < n_sys; sy++) {
            const long long ns = mg.atom_off[(size_t)sy + 1] - mg.atom_off[(size_t)sy];
            full_cells += std::min<long long>(std::max<long long>(8LL * ns, 1LL << 20), 1LL << 27) + 1;
        }
        const bool small_budget = full_cells > (1LL << 30);
        for (int sy = 0; sy < n_sys; sy++) {
            const int ns = mg.atom_off[(size_t)sy + 1] - mg.atom_off[(size_t)sy];
            c->max_sys_atoms = std::max(c->max_sys_atoms, ns);
            for (int i = mg.atom_off[(size_t)sy]; i < mg.atom_off[(size_t)sy + 1]; i++) atom_sys[(size_t)i] = sy;
            const int padded = (ns + 31) / 32 * 32;
            for (int g = 0; g < padded / 32; g++) group_sys.push_back(sy);
            slot_off.push_back(slot_off.back() + padded);
            // cell budget: a few cells per atom, at least 2^20 (the grid of a
            // swollen droplet in vacuum stays fine-grained); 12 bytes per cell.
            // A batch gives each system the budget it has alone (so its grid,
            // sorted order and sums are the same) while the total stays below
            // 2^30 cells, else 8 cells per atom.
            const long long cells = small_budget ? std::max<long long>(8LL * ns, 1LL << 15)
                                                 : std::min<long long>(std::max<long long>(8LL * ns, 1LL << 20), 1LL << 27);
            if ((long long)cell_off.back() + cells + 1 > INT32_MAX) {
                fail(c, GM_ERR_UNSUPPORTED, "cell budget of the batch exceeds 2^31");
                return bail(GM_ERR_UNSUPPORTED);
            }
            cell_off.push_back(cell_off.back() + (int)cells + 1);
        }
        c->n_slots = slot_off.back();
        c->total_cells = cell_off.back();
        if (c->n_slots > GM_SLOT_MASK) {
            fail(c, GM_ERR_UNSUPPORTED, "%d padded atom slots; at most %d are supported", c->n_slots, GM_SLOT_MASK);
            return bail(GM_ERR_UNSUPPORTED);
        }
        TRY(dupload(c, &c->d_sys_atom_off, mg.atom_off.data(), mg.atom_off.size()));
        TRY(dupload(c, &c->d_sys_slot_off, slot_off.data(), slot_off.size()));
        TRY(dupload(c, &c->d_sys_cell_off, cell_off.data(), cell_off.size()));
        TRY(dupload(c, &c->d_atom_sys, atom_sys.data(), atom_sys.size()));
        TRY(dupload(c, &c->d_group_sys, group_sys.data(), group_sys.size()));
        TRY(dalloc(c, &c->d_sys_flag, (size_t)n_sys));
        TRY(dalloc(c, &c->d_e_sys, (size_t)n_sys));
        cudaMemset(c->d_sys_flag, 0, sizeof(unsigned int) * (size_t)n_sys);
        cudaMemset(c->d_e_sys, 0, sizeof(long long) * (size_t)n_sys);
    }
    const size_t ns_ = (size_t)c->n_slots;
    TRY(dalloc(c, &c->d_coord, 2 * ns_));
    cudaMemset(c->d_coord, 0, sizeof(float4) * 2 * ns_);
    if (c->fp64) {
        TRY(dalloc(c, &c->d_pos64s, ns_));
        TRY(dalloc(c, &c->d_type_sorted, ns_));
        cudaMemset(c->d_pos64s, 0, sizeof(double4) * ns_);
        cudaMemset(c->d_type_sorted, 0, sizeof(int) * ns_);
    }
    TRY(dalloc(c, &c->d_perm, ns_));
    cudaMemset(c->d_perm, 0xFF, sizeof(int) * ns_);  // -1: padding until a build fills the slot
    TRY(dalloc(c, &c->d_slot_of, (size_t)std::max(n, 1)));
    TRY(dalloc(c, &c->d_cell_of, (size_t)n));
    TRY(dalloc(c, &c->d_cell_sorted, ns_));
    TRY(dalloc(c, &c->d_tmp_atom, ns_));
    TRY(dalloc(c, &c->d_cell_count, (size_t)c->total_cells));
    TRY(dalloc(c, &c->d_cell_cursor, (size_t)c->total_cells));
    TRY(dalloc(c, &c->d_cell_start, (size_t)c->total_cells));
    TRY(dalloc(c, &c->d_grid, (size_t)n_sys));
    cudaMemset(c->d_grid, 0, sizeof(GridInfo) * (size_t)n_sys);
    c->bbox_blocks = std::max(1, std::min(256, (c->max_sys_atoms + 255) / 256));
    TRY(dalloc(c, &c->d_bbox, 9 * (size_t)c->bbox_blocks * n_sys));
    c->n_groups = c->n_slots / 32;
    TRY(dalloc(c, &c->d_count, ns_));
    cudaMemset(c->d_count, 0, sizeof(int) * ns_);  // padding slots keep count 0
    TRY(dalloc(c, &c->d_gmax, (size_t)c->n_groups));
    cudaMemset(c->d_gmax, 0, sizeof(int) * (size_t)c->n_groups);
    c->n_epart = c->n_groups * GM_MAX_SPLIT + c->bonded_blocks + c->blocks14;
    {
        // enough warps in flight to hide the gather latency: about 48 per SM
        int dev_sms = 0;
        cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device);
        const int want = 48 * std::max(dev_sms, 1);
        c->split = std::max(1, std::min(GM_MAX_SPLIT, (want + c->n_groups - 1) / std::max(c->n_groups, 1)));
    }
    TRY(dalloc(c, &c->d_epart, (size_t)c->n_epart));
    TRY(dalloc(c, &c->d_energy, 1));
    TRY(dalloc(c, &c->d_kin_part, 256));
    TRY(dalloc(c, &c->d_ke, 1));
    TRY(dalloc(c, &c->d_status, 1));
    TRY(dalloc(c, &c->d_sync, 1));
    if (cudaMemset(c->d_sync, 0, sizeof(StepSync)) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (cudaMallocHost((void **)&c->h_status, sizeof(DevStatus)) != cudaSuccess) return bail(GM_ERR_OUT_OF_MEMORY);
    if (cudaMallocHost((void **)&c->h_energy, sizeof(double)) != cudaSuccess) return bail(GM_ERR_OUT_OF_MEMORY);
    DevStatus z{};
    z.fail_step = ~0ull;
    if (cudaMemcpy(c->d_status, &z, sizeof z, cudaMemcpyHostToDevice) != cudaSuccess) return bail(GM_ERR_DEVICE);
    if (n) {
        cudaMemset(c->d_force, 0, sizeof(long long) * 3 * (size_t)n);
        cudaMemset(c->d_pos, 0, sizeof(double) * 3 * (size_t)n);
        cudaMemset(c->d_vel, 0, sizeof(double) * 3 * (size_t)n);
        cudaMemset(c->d_ref, 0, sizeof(double) * 3 * (size_t)n);
    }
#undef TRY
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(GM_ERR_DEVICE);
    return c;
}

}  // namespace

extern "C" {

int32_t gm_destroy(gm_ctx *c) {
    if (!c) return GM_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    for (void *ptr : c->allocs) cudaFree(ptr);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_energy) cudaFreeHost(c->h_energy);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->xfer) cudaStreamDestroy(c->xfer);
    if (c->ev_xfer_in) cudaEventDestroy(c->ev_xfer_in);
    if (c->ev_xfer_out) cudaEventDestroy(c->ev_xfer_out);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
    return GM_OK;
}

int32_t gm_n_threads(const gm_ctx *) { return 1; }

int32_t gm_last_error(const gm_ctx *c, char *buf, int64_t len) {
    if (!buf || len <= 0) return GM_ERR_INVALID_ARGUMENT;
    const char *m = c ? c->err.c_str() : "no context";
    snprintf(buf, (size_t)len, "%s", m);
    return GM_OK;
}

int32_t gm_build_list(gm_ctx *c, double *px, double *py, double *pz) {
    if (!c || (!px && c->n)) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!finite3(px, py, pz, c->n)) return fail(c, GM_ERR_NONFINITE, "non-finite position passed to build_neighbor_list");
    if (!c->d_list) {
        int rc = ensure_estimated_buffers(c, px, py, pz);
        if (rc) return rc;
    }
    int rc = upload3(c, c->d_pos, px, py, pz);
    if (rc) return rc;
    rc = do_build(c);
    if (rc) return rc;
    if (c->p.periodic) {
        rc = download3(c, c->d_pos, px, py, pz);  // neighbor.rs:13-15 wraps the caller's state
        if (rc) return rc;
        GM_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return GM_OK;
}

int32_t gm_compute_forces(gm_ctx *c, const double *px, const double *py, const double *pz, double *fx, double *fy,
                          double *fz, double *energy) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    auto poison = [&](int code) {
        // compute_forces is infallible in the trait: NaN forces make the run
        // loop's check_forces_finite (lib.rs:307) stop the run
        const double nan = std::nan("");
        for (int i = 0; i < c->n; i++) { if (fx) fx[i] = nan; if (fy) fy[i] = nan; if (fz) fz[i] = nan; }
        if (energy) *energy = nan;
        return code;
    };
    if (cudaSetDevice(c->device) != cudaSuccess) return poison(GM_ERR_DEVICE);
    if (!c->built) return poison(fail(c, GM_ERR_NOT_BUILT, "compute_forces before build_neighbor_list"));
    int rc = upload3(c, c->d_pos, px, py, pz);
    if (rc) return poison(rc);
    rc = reset_status(c);
    if (rc) return poison(rc);
    c->launches += seq_forces(c, c->stream);
    gm_launch_forces_out(c->n, c->d_force, c->d_fout, c->stream);
    c->launches++;
    rc = download3(c, c->d_fout, fx, fy, fz);
    if (rc) return poison(rc);
    if (energy)
        GM_CUDA(c, cudaMemcpyAsync(c->h_energy, c->d_energy, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    rc = check_status(c, nullptr);
    if (rc) return poison(rc);
    if (energy) *energy = *c->h_energy;
    c->forces_current = true;
    return GM_OK;
}

int32_t gm_needs_rebuild(gm_ctx *c, const double *px, const double *py, const double *pz, int32_t *result) {
    if (!c || !result) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!c->built) { *result = 1; return GM_OK; }
    int rc = upload3(c, c->d_pos, px, py, pz);
    if (rc) return rc;
    rc = reset_status(c);
    if (rc) return rc;
    const double half_skin = (c->p.r_skin - c->p.r_cutoff) / 2.0;
    gm_launch_check(c->n, c->d_pos, c->d_ref, half_skin * half_skin, c->d_status, 0ull, gm_check_blocks(c->n),
                    c->d_atom_sys, c->d_sys_flag, c->stream);
    rc = st_read(c);
    if (rc) return rc;
    *result = c->h_status->rebuild ? 1 : 0;
    gm_launch_flags(list_args(c), false, c->stream);  // a query: leave no system marked
    c->launches += 2;
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

int32_t gm_geodesic_drift(gm_ctx *c, double *px, double *py, double *pz, double *vx, double *vy, double *vz,
                          double dt, uint64_t step, gm_convergence *err) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = upload3(c, c->d_pos, px, py, pz);
    if (!rc) rc = upload3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    rc = reset_status(c);
    if (!rc) rc = set_step(c, step);
    if (rc) return rc;
    const bool constrained = c->n_clusters > 0;
    gm_launch_drift(c->n, c->d_pos, c->d_vel, c->d_dref, dt, !constrained, c->d_status, c->stream);
    c->launches++;
    if (constrained) {
        c->launches += issue_shake(c, c->stream, false);
        gm_launch_resync(c->n, c->d_pos, c->d_vel, c->d_dref, dt, c->d_status, c->stream);
        c->launches += 1;
    }
    rc = download3(c, c->d_pos, px, py, pz);
    if (!rc) rc = download3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    c->forces_current = false;
    return check_status(c, err);
}

int32_t gm_half_kick(gm_ctx *c, double *vx, double *vy, double *vz, const double *fx, const double *fy,
                     const double *fz, double dt_half) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = upload3(c, c->d_vel, vx, vy, vz);
    if (!rc) rc = upload3(c, c->d_host_f, fx, fy, fz);
    if (rc) return rc;
    gm_launch_half_kick_f64(c->n, c->d_vel, c->d_host_f, c->d_inv_mass, dt_half, c->stream);
    c->launches++;
    rc = download3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

int32_t gm_constrain_velocities(gm_ctx *c, const double *px, const double *py, const double *pz, double *vx,
                                double *vy, double *vz, uint64_t step, gm_convergence *err) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!c->n_clusters) return GM_OK;  // constraint.rs:183-186
    int rc = upload3(c, c->d_pos, px, py, pz);
    if (!rc) rc = upload3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    rc = reset_status(c);
    if (!rc) rc = set_step(c, step);
    if (rc) return rc;
    gm_launch_rattle(cluster_args(c), c->n, c->d_pos, c->d_vel, c->stream);
    c->launches += 3;
    rc = download3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    return check_status(c, err);
}

int32_t gm_kinetic_energy(gm_ctx *c, const double *vx, const double *vy, const double *vz, double *ke) {
    if (!c || !ke) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = upload3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    gm_launch_kinetic(c->n, c->d_vel, c->d_mass, c->d_kin_part, 64, c->d_ke, c->stream);
    c->launches += 2;
    GM_CUDA(c, cudaMemcpyAsync(ke, c->d_ke, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

int32_t gm_get_pairs(gm_ctx *c, int64_t cap, uint32_t *pair_i, uint32_t *pair_j, int64_t *n_pairs) {
    if (!c || !n_pairs) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!c->built) return fail(c, GM_ERR_NOT_BUILT, "no neighbour list");
    const int ns = c->n_slots;
    std::vector<int> perm((size_t)ns), count((size_t)ns), list((size_t)ns * c->cap);
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (ns) {
        GM_CUDA(c, cudaMemcpy(perm.data(), c->d_perm, sizeof(int) * (size_t)ns, cudaMemcpyDeviceToHost));
        GM_CUDA(c, cudaMemcpy(count.data(), c->d_count, sizeof(int) * (size_t)ns, cudaMemcpyDeviceToHost));
        GM_CUDA(c, cudaMemcpy(list.data(), c->d_list, sizeof(int) * list.size(), cudaMemcpyDeviceToHost));
    }
    std::vector<uint64_t> keys;
    for (int s = 0; s < ns; s++) {
        if (perm[(size_t)s] < 0) continue;  // padding slot
        const int g = s / 32, l = s % 32;
        for (int e = 0; e < count[(size_t)s]; e++) {
            const int j = list[(size_t)g * 32 * c->cap + (size_t)e * 32 + l];
            const uint32_t a = (uint32_t)perm[(size_t)s], b = (uint32_t)perm[(size_t)j];
            if (a < b) keys.push_back(((uint64_t)a << 32) | b);
        }
    }
    std::sort(keys.begin(), keys.end());
    *n_pairs = (int64_t)keys.size();
    if (pair_i && pair_j) {
        const int64_t m = std::min<int64_t>(cap, (int64_t)keys.size());
        for (int64_t k = 0; k < m; k++) { pair_i[k] = (uint32_t)(keys[(size_t)k] >> 32); pair_j[k] = (uint32_t)keys[(size_t)k]; }
    }
    return GM_OK;
}

int32_t gm_upload_state(gm_ctx *c, const double *px, const double *py, const double *pz, const double *vx,
                        const double *vy, const double *vz) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!finite3(px, py, pz, c->n)) return fail(c, GM_ERR_NONFINITE, "non-finite position");
    if (!c->d_list) {
        int rc = ensure_estimated_buffers(c, px, py, pz);
        if (rc) return rc;
    }
    int rc;
    if (c->forces_current) {
        // forces stay valid when the caller hands back the resident positions
        rc = upload3(c, c->d_dref, px, py, pz);
        if (rc) return rc;
        rc = reset_status(c);
        if (rc) return rc;
        gm_launch_differs(c->n, c->d_dref, c->d_pos, &c->d_status->differs, c->stream);
        c->launches++;
        rc = st_read(c);
        if (rc) return rc;
        if (c->h_status->differs) {
            c->forces_current = false;
            GM_CUDA(c, cudaMemcpyAsync(c->d_pos, c->d_dref, sizeof(double) * 3 * (size_t)c->n,
                                       cudaMemcpyDeviceToDevice, c->stream));
        }
    } else {
        rc = upload3(c, c->d_pos, px, py, pz);
        if (rc) return rc;
    }
    rc = upload3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

// Average duration of one kernel (or sequence) measured with CUDA events on
// the context's stream: which = 0 pair kernel, 1 bonded kernel, 2 list
// rebuild sequence, 3 one captured BAB step (graph launch), 4 pack kernel.
int32_t gm_profile(gm_ctx *c, int32_t which, int32_t n_iter, double dt, double *avg_ms) {
    if (!c || !avg_ms || n_iter <= 0) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = ensure_forces(c);
    if (rc) return rc;
    if (which == 3 && c->use_graph) {
        rc = capture_graph(c, dt);
        if (rc) return rc;
    }
    cudaEvent_t e0, e1;
    GM_CUDA(c, cudaEventCreate(&e0));
    GM_CUDA(c, cudaEventCreate(&e1));
    double total = 0.0;
    ForceArgs fa = force_args(c);
    ListArgs la = list_args(c);
    const bool pf = which == 3 && persistent_form(c);
    for (int k = 0; k < n_iter; k++) {
        if (pf) {
            rc = begin_persistent(c, false);  // the timed launch evaluates its forces
            if (rc) return rc;
        }
        cudaEventRecord(e0, c->stream);
        switch (which) {
            case 0: gm_launch_pair(fa, c->fp64, c->stream); break;
            case 1: gm_launch_bonded(fa, c->fp64, c->stream); break;
            case 2: seq_rebuild(c, c->stream, true); break;
            case 3:
                if (c->use_graph) cudaGraphLaunch(c->graph_exec, c->stream);
                else run_direct(c, dt, 1);
                break;
            case 5: seq_forces(c, c->stream, false, c->side); break;
            case 6: gm_launch_pair14(fa, c->fp64, c->stream); break;
            case 7:  // the list build kernel alone, every system
                gm_launch_flags(la, true, c->stream);
                gm_launch_build(la, c->stream);
                gm_launch_flags(la, false, c->stream);
                break;
            default: gm_launch_pack(la, c->fp64, c->stream); break;
        }
        cudaEventRecord(e1, c->stream);
        GM_CUDA(c, cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        if (which == 3) {
            // outside the timed span, as after a run
            rc = pf ? end_persistent(c) : GM_OK;
            if (!rc) rc = finish_steps(c, dt);
            if (rc) return rc;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *avg_ms = total / n_iter;
    // the pair/bonded kernels add into the force buffer: recompute it
    c->forces_current = false;
    rc = ensure_forces(c);
    if (rc) return rc;
    return check_status(c, nullptr);
}

int32_t gm_download_state(gm_ctx *c, double *px, double *py, double *pz, double *vx, double *vy, double *vz) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = download3(c, c->d_pos, px, py, pz);
    if (!rc) rc = download3(c, c->d_vel, vx, vy, vz);
    if (rc) return rc;
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    return GM_OK;
}

int32_t gm_forces_resident(gm_ctx *c) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    // the list is rebuilt first when the resident positions moved more than
    // half the skin from its build (neighbor.rs:60-72), as in a step
    c->forces_current = false;
    return ensure_forces(c);
}

int32_t gm_run_resident(gm_ctx *c, double dt, uint64_t first_step, int64_t n_steps) {
    if (!c || !(dt > 0) || n_steps < 0) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = reset_status(c);
    if (!rc) rc = set_step(c, first_step);
    if (rc) return rc;
    rc = ensure_forces(c);
    if (rc) return rc;
    return launch_steps(c, dt, n_steps);
}

int32_t gm_time_steps(gm_ctx *c, double dt, uint64_t first_step, int64_t n_steps, void *flush_buf,
                      int64_t flush_bytes, double *total_ms) {
    if (!c || !(dt > 0) || n_steps <= 0 || !total_ms) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = reset_status(c);
    if (!rc) rc = set_step(c, first_step);
    if (!rc) rc = ensure_forces(c);
    if (!rc && c->use_graph) rc = capture_graph(c, dt);
    // every timed persistent launch evaluates its forces
    const bool pf = persistent_form(c);
    if (!rc && pf) rc = begin_persistent(c, false);
    if (rc) return rc;
    std::vector<cudaEvent_t> ev((size_t)(2 * n_steps));
    for (auto &e : ev) GM_CUDA(c, cudaEventCreate(&e));
    if (flush_buf && flush_bytes > 0)
        GM_CUDA(c, cudaMemsetAsync(flush_buf, 0, (size_t)flush_bytes, c->stream));
    for (int64_t k = 0; k < n_steps; k++) {
        GM_CUDA(c, cudaEventRecord(ev[(size_t)(2 * k)], c->stream));
        if (c->use_graph) {
            GM_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
        } else {
            rc = run_direct(c, dt, 1);
            if (rc) return rc;
        }
        GM_CUDA(c, cudaEventRecord(ev[(size_t)(2 * k + 1)], c->stream));
        // evict the step's working set so every timed step starts from HBM
        if (flush_buf && flush_bytes > 0)
            GM_CUDA(c, cudaMemsetAsync(flush_buf, (int)((k + 1) & 0xff), (size_t)flush_bytes, c->stream));
    }
    if (c->use_graph) c->launches += c->launches_per_step * n_steps;
    c->energy_stale = true;  // the steps leave their energy partials unsummed
    if (pf) rc = end_persistent(c);
    if (!rc) rc = finish_steps(c, dt);
    if (rc) return rc;
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    double total = 0.0;
    for (int64_t k = 0; k < n_steps; k++) {
        float ms = 0.f;
        GM_CUDA(c, cudaEventElapsedTime(&ms, ev[(size_t)(2 * k)], ev[(size_t)(2 * k + 1)]));
        total += ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *total_ms = total;
    return check_status(c, nullptr);
}

int32_t gm_synchronize(gm_ctx *c, gm_convergence *err) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    return check_status(c, err);
}

void *gm_stream(gm_ctx *c) { return c ? (void *)c->stream : nullptr; }

int32_t gm_steps(gm_ctx *c, double *px, double *py, double *pz, double *vx, double *vy, double *vz, double dt,
                 uint64_t first_step, int64_t n_steps, double *fx, double *fy, double *fz, double *energy,
                 int64_t *n_rebuilds, gm_convergence *err) {
    // Two host synchronisations per call: the check whether the caller's
    // positions are the resident ones (forces stay valid), and the results
    // with the status word at the end.  The status reset, the step number and
    // the call's rebuild base are set on the device.  The velocity upload
    // runs on a copy stream beside the position check, the position download
    // beside the forces at the final positions.
    if (!c || !(dt > 0) || n_steps < 0) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    // positions are checked for finiteness on the device when the resident
    // forces are current (the comparison kernel reads them anyway), on the
    // host otherwise
    if (!c->forces_current && !finite3(px, py, pz, c->n)) return fail(c, GM_ERR_NONFINITE, "non-finite position");
    if (!c->d_list) {
        int rc = ensure_estimated_buffers(c, px, py, pz);
        if (rc) return rc;
    }
    gm_launch_status_reset(c->d_status, 1, first_step, c->stream);
    c->launches++;
    // the velocities travel on the copy stream, after the work already on
    // the context's stream and beside the position check
    GM_CUDA(c, cudaEventRecord(c->ev_xfer_in, c->stream));
    GM_CUDA(c, cudaStreamWaitEvent(c->xfer, c->ev_xfer_in, 0));
    int rc = upload3(c, c->d_vel, vx, vy, vz, c->xfer);
    if (rc) return rc;
    GM_CUDA(c, cudaEventRecord(c->ev_xfer_out, c->xfer));
    rc = stage_positions(c, px, py, pz, true);
    if (!rc) rc = cudaStreamWaitEvent(c->stream, c->ev_xfer_out, 0) == cudaSuccess ? GM_OK
                  : fail(c, GM_ERR_DEVICE, "cudaStreamWaitEvent");
    if (!rc) rc = ensure_forces(c);
    if (!rc) rc = launch_loop(c, dt, n_steps);
    if (rc) {
        cudaStreamSynchronize(c->xfer);
        return rc;
    }
    // the final positions go out on the copy stream while the forces at
    // them and the closing half-kick run
    GM_CUDA(c, cudaEventRecord(c->ev_xfer_in, c->stream));
    GM_CUDA(c, cudaStreamWaitEvent(c->xfer, c->ev_xfer_in, 0));
    rc = download3(c, c->d_pos, px, py, pz, c->xfer);
    if (!rc) GM_CUDA(c, cudaEventRecord(c->ev_xfer_out, c->xfer));
    if (!rc) rc = launch_end(c, dt, n_steps);
    if (!rc) GM_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_xfer_out, 0));
    if (rc) {
        cudaStreamSynchronize(c->xfer);
        return rc;
    }
    rc = download3(c, c->d_vel, vx, vy, vz);
    if (!rc && (fx || fy || fz)) {
        gm_launch_forces_out(c->n, c->d_force, c->d_fout, c->stream);
        c->launches++;
        rc = download3(c, c->d_fout, fx, fy, fz);
    }
    if (!rc && energy) {
        refresh_energy(c);
        GM_CUDA(c, cudaMemcpyAsync(c->h_energy, c->d_energy, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    GM_CUDA(c, cudaMemcpyAsync(c->h_status, c->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->stream));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    GM_CUDA(c, cudaGetLastError());
    if (!rc && energy) *energy = *c->h_energy;
    if (n_rebuilds) *n_rebuilds = (int64_t)(c->h_status->n_rebuilds - c->h_status->rebuild_base);
    const int rs = status_result(c, err);
    // after a failed step the force sums may not be the forces at the
    // resident positions: the next call evaluates them afresh
    if (rs) c->forces_current = false;
    return rs ? rs : rc;
}

int32_t gm_counters(const gm_ctx *cc, int64_t *out, int64_t n) {
    if (!cc || !out) return GM_ERR_INVALID_ARGUMENT;
    gm_ctx *c = const_cast<gm_ctx *>(cc);
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = st_read(c);
    if (rc) return rc;
    const DevStatus st = *c->h_status;
    int64_t v[12] = {0, (int64_t)st.n_rebuilds, c->cap, c->launches, (int64_t)st.shake_T, (int64_t)st.rattle_T,
                     c->launches_per_step, c->split, (int64_t)st.c_steps, (int64_t)st.shake_sum,
                     (int64_t)st.rattle_sum, (int64_t)st.rec_n};
    if (c->built && n > 0) {
        // pairs in the current list (half of the symmetric entries)
        std::vector<int> count((size_t)c->n_slots);
        if (c->n_slots)
            GM_CUDA(c, cudaMemcpy(count.data(), c->d_count, sizeof(int) * (size_t)c->n_slots, cudaMemcpyDeviceToHost));
        long long s = 0;
        for (int x : count) s += x;
        v[0] = s / 2;
    }
    for (int64_t k = 0; k < n && k < 12; k++) out[k] = v[k];
    return GM_OK;
}

/* ---- constraint warm start ------------------------------------------- */

int32_t gm_ws_record(gm_ctx *c, int64_t cap_steps, int32_t stride) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    if (!c->n_constr) return fail(c, GM_ERR_UNSUPPORTED, "the system has no constraints");
    if (bonded_min_image(c) && cap_steps > 0 && stride > 0)
        return fail(c, GM_ERR_UNSUPPORTED, "the warm start's features take raw position differences: not with bonded_min_image");
    drop_graph(c);
    if (cap_steps <= 0 || stride <= 0) {  // stop; the samples stay for training
        c->ws_rec_stride = 0;
        return GM_OK;
    }
    if ((double)cap_steps * c->n_constr * GM_WS_IN > 4e9) return fail(c, GM_ERR_INVALID_ARGUMENT, "record too large");
    dfree(c, c->d_rec_feat);
    dfree(c, c->d_rec_t);
    c->d_rec_feat = c->d_rec_t = nullptr;
    int rc = dalloc(c, &c->d_rec_feat, (size_t)cap_steps * c->n_constr * GM_WS_IN);
    if (!rc) rc = dalloc(c, &c->d_rec_t, (size_t)cap_steps * c->n_constr);
    if (rc) return rc;
    rc = st_read(c);
    if (rc) return rc;
    c->h_status->rec_n = 0;
    rc = st_write(c);
    if (rc) return rc;
    c->ws_rec_cap = (int)cap_steps;
    c->ws_rec_stride = stride;
    return GM_OK;
}

int32_t gm_ws_samples(gm_ctx *c, int64_t cap, float *feat, float *target, int64_t *n_samples) {
    if (!c || !n_samples) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = st_read(c);
    if (rc) return rc;
    const int64_t n = c->d_rec_t ? (int64_t)c->h_status->rec_n * c->n_constr : 0;
    *n_samples = n;
    const int64_t m = std::min<int64_t>(n, cap);
    if (m > 0 && feat) GM_CUDA(c, cudaMemcpy(feat, c->d_rec_feat, sizeof(float) * GM_WS_IN * m, cudaMemcpyDeviceToHost));
    if (m > 0 && target) GM_CUDA(c, cudaMemcpy(target, c->d_rec_t, sizeof(float) * m, cudaMemcpyDeviceToHost));
    return GM_OK;
}

int32_t gm_ws_train(gm_ctx *c, int64_t iters, int32_t blocks, double lr, uint64_t seed, double *final_loss) {
    if (!c || iters < 0 || blocks <= 0) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = st_read(c);
    if (rc) return rc;
    const long long n = c->d_rec_t ? (long long)c->h_status->rec_n * c->n_constr : 0;
    if (n <= 0) return fail(c, GM_ERR_NOT_BUILT, "no recorded warm-start samples");
    if ((rc = ws_alloc_model(c)) || (rc = ws_partial(c, blocks))) return rc;
    cudaStream_t s = c->stream;
    gm_launch_ws_stats(n, c->d_rec_feat, c->d_rec_t, c->d_ws_stats, 256, c->d_ws_norm, s);
    std::vector<float> P;
    ws_init_params(seed, P);
    GM_CUDA(c, cudaMemcpyAsync(c->d_ws_params, P.data(), sizeof(float) * P.size(), cudaMemcpyHostToDevice, s));
    GM_CUDA(c, cudaMemsetAsync(c->d_ws_m, 0, sizeof(float) * GM_WS_NPAR, s));
    GM_CUDA(c, cudaMemsetAsync(c->d_ws_v, 0, sizeof(float) * GM_WS_NPAR, s));
    GM_CUDA(c, cudaMemsetAsync(c->d_ws_out, 0, sizeof(float) * (GM_WS_NPAR + 1), s));
    for (int64_t it = 0; it < iters; it++) {
        const double lr_t = lr * 0.5 * (1.0 + std::cos(M_PI * (double)it / (double)iters));  // cosine decay
        gm_launch_ws_grad(n, c->d_rec_feat, c->d_rec_t, c->d_ws_norm, false, c->d_ws_params, blocks, seed,
                          (long long)it, (long long)blocks * GM_WS_TILE, c->d_ws_partial, s);
        gm_launch_ws_update(blocks, c->d_ws_partial, c->d_ws_params, c->d_ws_m, c->d_ws_v, (float)lr_t, 0.9f, 0.999f,
                            1e-8f, (int)(it + 1), c->d_ws_out, s);
    }
    gm_launch_ws_pack(c->d_ws_params, c->d_ws_norm, c->d_ws_packed, s);  // the inference's layout
    c->launches += 3 + 2 * iters;
    GM_CUDA(c, cudaGetLastError());
    float loss = 0.0f;
    GM_CUDA(c, cudaMemcpyAsync(&loss, c->d_ws_out, sizeof(float), cudaMemcpyDeviceToHost, s));
    GM_CUDA(c, cudaStreamSynchronize(s));
    if (final_loss) *final_loss = (double)loss / ((double)blocks * GM_WS_TILE);
    c->ws_model = true;
    drop_graph(c);
    return GM_OK;
}

int32_t gm_ws_enable(gm_ctx *c, int32_t on) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    if (on && !c->ws_model) return fail(c, GM_ERR_NOT_BUILT, "no warm-start model (train or set one first)");
    if (on && !c->n_constr) return fail(c, GM_ERR_UNSUPPORTED, "the system has no constraints");
    if (on && bonded_min_image(c))
        return fail(c, GM_ERR_UNSUPPORTED, "the warm start's features take raw position differences: not with bonded_min_image");
    c->ws_on = on != 0;
    drop_graph(c);
    return GM_OK;
}

int32_t gm_ws_params(gm_ctx *c, float *get_params, float *get_norm, const float *set_params, const float *set_norm) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = ws_alloc_model(c);
    if (rc) return rc;
    if (set_params) GM_CUDA(c, cudaMemcpy(c->d_ws_params, set_params, sizeof(float) * GM_WS_NPAR, cudaMemcpyHostToDevice));
    if (set_norm) GM_CUDA(c, cudaMemcpy(c->d_ws_norm, set_norm, sizeof(float) * GM_WS_NNORM, cudaMemcpyHostToDevice));
    if (set_params && set_norm) c->ws_model = true;
    if ((get_params || get_norm) && !c->ws_model) return fail(c, GM_ERR_NOT_BUILT, "no warm-start model");
    if (get_params) GM_CUDA(c, cudaMemcpy(get_params, c->d_ws_params, sizeof(float) * GM_WS_NPAR, cudaMemcpyDeviceToHost));
    if (get_norm) GM_CUDA(c, cudaMemcpy(get_norm, c->d_ws_norm, sizeof(float) * GM_WS_NNORM, cudaMemcpyDeviceToHost));
    if (set_params || set_norm) {
        gm_launch_ws_pack(c->d_ws_params, c->d_ws_norm, c->d_ws_packed, c->stream);  // the inference's layout
        c->launches++;
        GM_CUDA(c, cudaStreamSynchronize(c->stream));
        drop_graph(c);
    }
    return GM_OK;
}

int32_t gm_ws_forward(gm_ctx *c, const float *x, int64_t m, float *y) {
    if (!c || m < 0 || (m && (!x || !y))) return GM_ERR_INVALID_ARGUMENT;
    if (!c->ws_model) return fail(c, GM_ERR_NOT_BUILT, "no warm-start model");
    if (!m) return GM_OK;
    GM_CUDA(c, cudaSetDevice(c->device));
    float *dx = nullptr, *dy = nullptr;
    int rc = dupload(c, &dx, x, (size_t)m * GM_WS_IN);
    if (!rc) rc = dalloc(c, &dy, (size_t)m);
    if (!rc) {
        gm_launch_ws_forward((int)m, dx, c->d_ws_params, dy, c->stream);
        c->launches++;
        cudaError_t e = cudaMemcpyAsync(y, dy, sizeof(float) * m, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        rc = cuda_status(c, e, "gm_ws_forward");
    }
    dfree(c, dx);
    dfree(c, dy);
    return rc;
}

int32_t gm_ws_gradient(gm_ctx *c, const float *x, const float *t, int64_t m, float *grad, double *loss) {
    if (!c || m <= 0 || !x || !t) return GM_ERR_INVALID_ARGUMENT;
    if (!c->ws_model) return fail(c, GM_ERR_NOT_BUILT, "no warm-start model");
    GM_CUDA(c, cudaSetDevice(c->device));
    const int blocks = (int)((m + GM_WS_TILE - 1) / GM_WS_TILE);
    float *dx = nullptr, *dt = nullptr, *dp = nullptr, *dg = nullptr;
    int rc = dupload(c, &dx, x, (size_t)m * GM_WS_IN);
    if (!rc) rc = dupload(c, &dt, t, (size_t)m);
    if (!rc) rc = dalloc(c, &dp, (size_t)blocks * (GM_WS_NPAR + 1));
    if (!rc) rc = dalloc(c, &dg, (size_t)GM_WS_NPAR + 1);
    if (!rc) {
        gm_launch_ws_grad(m, dx, dt, nullptr, true, c->d_ws_params, blocks, 0, -1, m, dp, c->stream);
        gm_launch_ws_update(blocks, dp, nullptr, nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 0, dg, c->stream);
        c->launches += 2;
        std::vector<float> h((size_t)GM_WS_NPAR + 1);
        cudaError_t e = cudaMemcpyAsync(h.data(), dg, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        rc = cuda_status(c, e, "gm_ws_gradient");
        if (!rc) {
            if (grad) std::copy(h.begin(), h.begin() + GM_WS_NPAR, grad);
            if (loss) *loss = (double)h[GM_WS_NPAR] / (double)m;
        }
    }
    dfree(c, dx);
    dfree(c, dt);
    dfree(c, dp);
    dfree(c, dg);
    return rc;
}

int32_t gm_ws_last(gm_ctx *c, float *feat, double *lam0, double *lam_sum) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    if (!c->n_constr) return GM_OK;
    GM_CUDA(c, cudaSetDevice(c->device));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    const size_t nc = (size_t)c->n_constr;
    if (feat) GM_CUDA(c, cudaMemcpy(feat, c->d_ws_feat, sizeof(float) * GM_WS_IN * nc, cudaMemcpyDeviceToHost));
    if (lam0) GM_CUDA(c, cudaMemcpy(lam0, c->d_ws_lam0, sizeof(double) * nc, cudaMemcpyDeviceToHost));
    if (lam_sum) GM_CUDA(c, cudaMemcpy(lam_sum, c->d_lam_sum, sizeof(double) * nc, cudaMemcpyDeviceToHost));
    return GM_OK;
}

/* ---- batches of independent systems ----------------------------------- */

/* ---- trajectory frames ------------------------------------------------- */

int32_t gm_frames_enable(gm_ctx *c, int32_t frame_interval, int32_t capacity) {
    if (!c || frame_interval < 0 || (frame_interval > 0 && capacity < 1)) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    dfree(c, c->d_frame_xyz);
    dfree(c, c->d_frame_step);
    dfree(c, c->d_frame_energy);
    dfree(c, c->d_frame_part);
    c->d_frame_xyz = nullptr;
    c->d_frame_step = nullptr;
    c->d_frame_energy = nullptr;
    c->d_frame_part = nullptr;
    c->frame_interval = 0;
    c->frame_cap = 0;
    if (frame_interval > 0) {
        int rc = dalloc(c, &c->d_frame_xyz, (size_t)capacity * 3 * (size_t)std::max(c->n, 1));
        if (!rc) rc = dalloc(c, &c->d_frame_step, (size_t)capacity);
        if (!rc) rc = dalloc(c, &c->d_frame_energy, 2 * (size_t)capacity);
        if (!rc) rc = dalloc(c, &c->d_frame_part, (size_t)GM_FRAME_BLOCKS);
        if (rc) return rc;
        c->frame_interval = frame_interval;
        c->frame_cap = capacity;
    }
    // the step graph is captured with or without the frame kernel
    drop_graph(c);
    int rc = st_read(c);
    if (rc) return rc;
    c->h_status->frame_n = 0;
    c->h_status->frame_lost = 0;
    return st_write(c);
}

int32_t gm_frames_take(gm_ctx *c, int64_t max_frames, float *xyz, uint64_t *steps, double *e_pot, double *e_kin,
                       int64_t *n_frames, int64_t *n_lost) {
    if (!c || !n_frames) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = st_read(c);
    if (rc) return rc;
    const int64_t n = c->h_status->frame_n;
    *n_frames = n;
    if (n_lost) *n_lost = c->h_status->frame_lost;
    if (n > max_frames) return fail(c, GM_ERR_INVALID_ARGUMENT, "%lld frames recorded, room for %lld",
                                    (long long)n, (long long)max_frames);
    if (n > 0) {
        if (xyz)
            GM_CUDA(c, cudaMemcpyAsync(xyz, c->d_frame_xyz, sizeof(float) * 3 * (size_t)c->n * (size_t)n,
                                       cudaMemcpyDeviceToHost, c->stream));
        if (steps)
            GM_CUDA(c, cudaMemcpyAsync(steps, c->d_frame_step, sizeof(unsigned long long) * (size_t)n,
                                       cudaMemcpyDeviceToHost, c->stream));
        if (e_pot || e_kin) {
            std::vector<double> e(2 * (size_t)n);
            GM_CUDA(c, cudaMemcpyAsync(e.data(), c->d_frame_energy, sizeof(double) * e.size(),
                                       cudaMemcpyDeviceToHost, c->stream));
            GM_CUDA(c, cudaStreamSynchronize(c->stream));
            for (int64_t k = 0; k < n; k++) {
                if (e_pot) e_pot[k] = e[2 * (size_t)k];
                if (e_kin) e_kin[k] = e[2 * (size_t)k + 1];
            }
        }
    }
    c->h_status->frame_n = 0;
    c->h_status->frame_lost = 0;
    return st_write(c);
}

int32_t gm_ensemble_info(const gm_ctx *c, int64_t *atom_offsets) {
    if (!c || !atom_offsets) return GM_ERR_INVALID_ARGUMENT;
    for (int sy = 0; sy <= c->n_sys; sy++) atom_offsets[sy] = c->h_atom_off[(size_t)sy];
    return GM_OK;
}

int32_t gm_ensemble_energies(gm_ctx *c, double *e_pot, double *e_kin) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    GM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (e_pot) {
        if (!c->forces_current) return fail(c, GM_ERR_NOT_BUILT, "no forces evaluated at the current positions");
        if (c->n_sys == 1) {
            refresh_energy(c);
            GM_CUDA(c, cudaStreamSynchronize(c->stream));
            GM_CUDA(c, cudaMemcpy(e_pot, c->d_energy, sizeof(double), cudaMemcpyDeviceToHost));
        } else {
            std::vector<long long> q((size_t)c->n_sys);
            GM_CUDA(c, cudaMemcpy(q.data(), c->d_e_sys, sizeof(long long) * q.size(), cudaMemcpyDeviceToHost));
            for (int sy = 0; sy < c->n_sys; sy++) e_pot[sy] = (double)q[(size_t)sy] / GM_EFIX_SCALE;
        }
    }
    if (e_kin) {
        // lib.rs:68-77 per system, in atom order
        const size_t n = (size_t)c->n;
        std::vector<double> v(3 * n), m(n);
        if (n) {
            GM_CUDA(c, cudaMemcpy(v.data(), c->d_vel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost));
            GM_CUDA(c, cudaMemcpy(m.data(), c->d_mass, sizeof(double) * n, cudaMemcpyDeviceToHost));
        }
        for (int sy = 0; sy < c->n_sys; sy++) {
            double sum = 0.0;
            for (int i = c->h_atom_off[(size_t)sy]; i < c->h_atom_off[(size_t)sy + 1]; i++) {
                const double vx = v[(size_t)i], vy = v[n + (size_t)i], vz = v[2 * n + (size_t)i];
                sum += m[(size_t)i] * (vx * vx + vy * vy + vz * vz);
            }
            e_kin[sy] = 0.5 * sum * (1.0 / (20.455 * 20.455));
        }
    }
    return GM_OK;
}

/* ---- autotuner ---------------------------------------------------------- */

int32_t gm_pair_shape(gm_ctx *c, int32_t split, int32_t warps_per_block, int32_t grid) {
    if (!c || split < 1 || split > GM_MAX_SPLIT || grid < 0 ||
        (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8))
        return GM_ERR_INVALID_ARGUMENT;
    c->split = split;
    c->pair_warps = warps_per_block;
    c->pair_grid = grid;
    drop_graph(c);  // the captured step holds the old launch shape
    return GM_OK;
}

int32_t gm_stall_next_barrier(gm_ctx *c) {
    if (!c) return GM_ERR_INVALID_ARGUMENT;
    if (!persistent_form(c)) return fail(c, GM_ERR_UNSUPPORTED, "the context does not step in the persistent form");
    c->stall_barrier = true;
    return GM_OK;
}

int32_t gm_step_form(gm_ctx *c, int32_t form) {
    if (!c || (form != GM_STEP_GRAPH && form != GM_STEP_PERSISTENT)) return GM_ERR_INVALID_ARGUMENT;
    if (form == GM_STEP_PERSISTENT && (c->fp64 || c->n_clusters > 0))
        return fail(c, GM_ERR_UNSUPPORTED, "the persistent step form runs unconstrained mixed-precision contexts");
    if (form != c->step_form) {
        c->step_form = form;
        drop_graph(c);  // the captured step is the other form's
    }
    return GM_OK;
}

int32_t gm_autotune(gm_ctx *c, int32_t reps, int64_t *choice) {
    if (!c || reps < 1) return GM_ERR_INVALID_ARGUMENT;
    GM_CUDA(c, cudaSetDevice(c->device));
    int rc = ensure_forces(c);
    if (rc) return rc;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    cudaEvent_t e0, e1;
    GM_CUDA(c, cudaEventCreate(&e0));
    GM_CUDA(c, cudaEventCreate(&e1));
    const int splits[] = {1, 2, 3, 4, 6, 8, 12, 16};
    const int warps[] = {2, 4, 8};
    const int grids[] = {0, 2, 4, 8, 16};  // 0: one work item per warp, else blocks per SM (persistent)
    double best = 1e300;
    int bs = c->split, bw = c->pair_warps, bg = c->pair_grid;
    for (int sp : splits)
        for (int w : warps)
            for (int gk : grids) {
                c->split = sp;
                c->pair_warps = w;
                c->pair_grid = gk ? gk * std::max(sms, 1) : 0;
                ForceArgs fa = force_args(c);
                gm_launch_pair(fa, c->fp64, c->stream);  // warm-up
                cudaEventRecord(e0, c->stream);
                for (int r = 0; r < reps; r++) gm_launch_pair(fa, c->fp64, c->stream);
                cudaEventRecord(e1, c->stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                c->launches += reps + 1;
                if (ms < best) { best = ms; bs = sp; bw = w; bg = c->pair_grid; }
            }
    c->pair_warps = bw;
    c->pair_grid = bg;
    if (force_phase(c) && persistent_grid(c) == GM_OK) {
        // with the persistent kernel's force phase (pair items and bonded
        // blocks from one queue) the split is the one that phase runs
        // fastest with
        double bestp = 1e300;
        GM_CUDA(c, cudaMemsetAsync(c->d_sync, 0, sizeof(StepSync), c->stream));
        for (int sp : splits) {
            c->split = sp;
            ForceArgs fa = force_args(c);
            gm_launch_forces_persistent(fa, c->d_sync, c->persist_blocks, c->stream);  // warm-up
            cudaEventRecord(e0, c->stream);
            for (int r = 0; r < reps; r++) gm_launch_forces_persistent(fa, c->d_sync, c->persist_blocks, c->stream);
            cudaEventRecord(e1, c->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            c->launches += reps + 1;
            if (ms < bestp) { bestp = ms; bs = sp; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->split = bs;
    GM_CUDA(c, cudaGetLastError());
    // the timing runs added forces many times over: evaluate them once more
    c->launches += seq_forces(c, c->stream);
    drop_graph(c);
    if (choice) { choice[0] = bs; choice[1] = bw; choice[2] = bg; }
    return check_status(c, nullptr);
}

}  // extern "C"
