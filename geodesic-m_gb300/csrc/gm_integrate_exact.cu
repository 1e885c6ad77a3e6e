// gm_integrate_exact.cu — FP64 integrator and constraint kernels.
//
// Built with --fmad=false: every expression below rounds after each
// operation in the order written, like the reference's Rust (which never
// contracts a*b+c).  Given the same forces, half-kick, drift and the
// SHAKE/RATTLE projections therefore return the reference's exact bits.
//
// Constraint solver (constraint.rs:62-152, :170-259).  The reference sweeps
// every constraint per Jacobi iteration and stops when max|lambda| < tol
// over all of them.  Constraints only couple through shared atoms, so the
// work splits into independent clusters (connected components of the
// constraint graph, found once on the host); one thread owns one cluster.
// Phase 1 iterates each cluster until its own max|lambda| < tol and records
// its count t_c; the global count is T = max t_c (the first iteration where
// every cluster is below tol, given that a converged cluster stays below
// tol).  Phase 2 advances every cluster to exactly T iterations and checks
// that assumption at iteration T (flagging GM_DEV_ITER_MISMATCH otherwise).
// Within a cluster, per-atom deltas are summed over the atom's constraints in
// ascending constraint index, starting from 0.0, as the reference's
// delta_x/y/z arrays are; positions after T iterations are bit-identical.
#include "gm_internal.cuh"

namespace {

constexpr double kForceToAccel = 20.455 * 20.455;  // integrator.rs:9

__global__ void half_kick_kernel(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                                 const DevStatus *st) {
    // integrator.rs:14-21: v += dt_half * F * inv_m * 20.455^2
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st->error) return;
    const double inv_m = inv_mass[i];
    for (int d = 0; d < 3; d++) {
        const double f = (double)force[d * n + i] * GM_FIX_INV;
        vel[d * n + i] += dt_half * f * inv_m * kForceToAccel;
    }
}

__global__ void half_kick_f64_kernel(int n, double *vel, const double *force, const double *inv_mass, double dt_half) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inv_m = inv_mass[i];
    for (int d = 0; d < 3; d++) vel[d * n + i] += dt_half * force[d * n + i] * inv_m * kForceToAccel;
}

__global__ void drift_kernel(int n, double *pos, double *vel, double *dref, double dt, int resync,
                             const DevStatus *st) {
    // integrator.rs:32-48 (and :64-68 when no constraint can move the atom)
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st->error) return;
    for (int d = 0; d < 3; d++) {
        const double p = pos[d * n + i];
        const double v = vel[d * n + i];
        dref[d * n + i] = p;
        const double np = p + dt * v;
        pos[d * n + i] = np;
        if (resync) vel[d * n + i] = (np - p) / dt;
    }
}

__global__ void resync_kernel(int n, const double *pos, double *vel, const double *dref, double dt,
                              const DevStatus *st) {
    // integrator.rs:64-68 (skipped after a failed projection, like the `?` at integrator.rs:256)
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st->error) return;
    for (int d = 0; d < 3; d++) vel[d * n + i] = (pos[d * n + i] - dref[d * n + i]) / dt;
}

__global__ void check_kernel(int n, const double *pos, const double *ref, double thr_sq, DevStatus *st,
                             unsigned long long cond, const int *atom_sys, unsigned int *sys_flag) {
    // neighbor.rs:60-72 plus the run loop's finite-position guard (lib.rs:94-107);
    // the atom's system is marked for the rebuild
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int need = 0, bad = 0;
    if (i < n) {
        const double x = pos[i], y = pos[n + i], z = pos[2 * n + i];
        bad = !(isfinite(x) && isfinite(y) && isfinite(z));
        const double dx = x - ref[i], dy = y - ref[n + i], dz = z - ref[2 * n + i];
        need = dx * dx + dy * dy + dz * dz > thr_sq;
        if (need) sys_flag[atom_sys[i]] = 1u;
    }
    need = __syncthreads_or(need);
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        if (need) atomicOr(&st->rebuild, 1u);
        if (bad) atomicOr(&st->error, (unsigned)GM_DEV_NONFINITE_POS);
        __threadfence();
        const unsigned done = atomicAdd(&st->blocks_done, 1u);
        if (done == gridDim.x - 1) {
            // last block: every block's flag is visible now
            __threadfence();
            const unsigned r = atomicOr(&st->rebuild, 0u);
            st->blocks_done = 0;
            // never rebuild from a failed state (NaN positions would pile into one cell)
            const unsigned e = atomicOr(&st->error, 0u);
            if (cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, (r && !e) ? 1u : 0u);
        }
    }
}

// One Jacobi iteration over a cluster.  Returns max|lambda| and its
// constraint (first in ascending order, as the reference's strict '>').
__device__ void shake_iteration(const ClusterArgs &c, int cl, const double *rvec, double *pos, int n_atoms,
                                double &max_out, int &worst_out) {
    const int c0 = c.cl_cstart[cl], c1 = c.cl_cstart[cl + 1];
    double max_lambda = 0.0;
    int worst = c0 < c1 ? c.cl_cons[c0] : 0;
    const int nc = c.n_constr;
    for (int q = c0; q < c1; q++) {
        const int k = c.cl_cons[q];
        const int i = c.constr_i[k], j = c.constr_j[k];
        const double dx = pos[i] - pos[j];
        const double dy = pos[n_atoms + i] - pos[n_atoms + j];
        const double dz = pos[2 * n_atoms + i] - pos[2 * n_atoms + j];
        const double diff = dx * dx + dy * dy + dz * dz - c.constr_dsq[k];
        const double rx = rvec[k], ry = rvec[nc + k], rz = rvec[2 * nc + k];
        const double inv_mi = c.inv_mass[i], inv_mj = c.inv_mass[j];
        const double dot_new_old = dx * rx + dy * ry + dz * rz;
        const double denom = 2.0 * (inv_mi + inv_mj) * dot_new_old;
        const double lambda = denom == 0.0 ? 0.0 : diff / denom;
        c.lam[k] = lambda;
        if (c.lam_sum) c.lam_sum[k] += lambda;  // the multiplier total, lam0 + sum of iterations
        const double la = fabs(lambda);
        if (la > max_lambda) { max_lambda = la; worst = k; }
    }
    const int a0 = c.cl_astart[cl], a1 = c.cl_astart[cl + 1];
    for (int q = a0; q < a1; q++) {
        const int a = c.cl_atoms[q];
        const double inv_m = c.inv_mass[a];
        double ddx = 0.0, ddy = 0.0, ddz = 0.0;
        for (int r = c.cl_acstart[q]; r < c.cl_acstart[q + 1]; r++) {
            const int ref = c.cl_acons[r];
            const int k = ref >= 0 ? ref : -ref - 1;   // negative: atom is constraint's i
            const double w = c.lam[k] * inv_m;
            const double tx = w * rvec[k], ty = w * rvec[nc + k], tz = w * rvec[2 * nc + k];
            if (ref < 0) { ddx -= tx; ddy -= ty; ddz -= tz; }
            else { ddx += tx; ddy += ty; ddz += tz; }
        }
        pos[a] += ddx;
        pos[n_atoms + a] += ddy;
        pos[2 * n_atoms + a] += ddz;
    }
    max_out = max_lambda;
    worst_out = worst;
}

__device__ void rattle_iteration(const ClusterArgs &c, int cl, const double *pos, double *vel, int n_atoms,
                                 double &max_out, int &worst_out) {
    const int c0 = c.cl_cstart[cl], c1 = c.cl_cstart[cl + 1];
    double max_mu = 0.0;
    int worst = c0 < c1 ? c.cl_cons[c0] : 0;
    const int nc = c.n_constr;
    for (int q = c0; q < c1; q++) {
        const int k = c.cl_cons[q];
        const int i = c.constr_i[k], j = c.constr_j[k];
        const double rx = pos[i] - pos[j];
        const double ry = pos[n_atoms + i] - pos[n_atoms + j];
        const double rz = pos[2 * n_atoms + i] - pos[2 * n_atoms + j];
        const double rsq = rx * rx + ry * ry + rz * rz;
        const double dvx = vel[i] - vel[j];
        const double dvy = vel[n_atoms + i] - vel[n_atoms + j];
        const double dvz = vel[2 * n_atoms + i] - vel[2 * n_atoms + j];
        const double rel_vel = dvx * rx + dvy * ry + dvz * rz;
        const double inv_mi = c.inv_mass[i], inv_mj = c.inv_mass[j];
        const double denom = (inv_mi + inv_mj) * rsq;
        const double mu = denom == 0.0 ? 0.0 : rel_vel / denom;
        c.lam[k] = mu;
        c.rvec[k] = rx;
        c.rvec[nc + k] = ry;
        c.rvec[2 * nc + k] = rz;
        const double ma = fabs(mu);
        if (ma > max_mu) { max_mu = ma; worst = k; }
    }
    const int a0 = c.cl_astart[cl], a1 = c.cl_astart[cl + 1];
    for (int q = a0; q < a1; q++) {
        const int a = c.cl_atoms[q];
        const double inv_m = c.inv_mass[a];
        double ddx = 0.0, ddy = 0.0, ddz = 0.0;
        for (int r = c.cl_acstart[q]; r < c.cl_acstart[q + 1]; r++) {
            const int ref = c.cl_acons[r];
            const int k = ref >= 0 ? ref : -ref - 1;
            const double w = c.lam[k] * inv_m;
            const double tx = w * c.rvec[k], ty = w * c.rvec[nc + k], tz = w * c.rvec[2 * nc + k];
            if (ref < 0) { ddx -= tx; ddy -= ty; ddz -= tz; }
            else { ddx += tx; ddy += ty; ddz += tz; }
        }
        vel[a] += ddx;
        vel[n_atoms + a] += ddy;
        vel[2 * n_atoms + a] += ddz;
    }
    max_out = max_mu;
    worst_out = worst;
}

// Reference vectors r_ref = ref_i - ref_j (constraint.rs:106-108), fixed for the call.
__global__ void shake_prepare(ClusterArgs c, const double *dref, int n_atoms) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n_constr) return;
    const int i = c.constr_i[k], j = c.constr_j[k];
    c.rvec[k] = dref[i] - dref[j];
    c.rvec[c.n_constr + k] = dref[n_atoms + i] - dref[n_atoms + j];
    c.rvec[2 * c.n_constr + k] = dref[2 * n_atoms + i] - dref[2 * n_atoms + j];
    if (c.lam_sum) c.lam_sum[k] = 0.0;
}

// Warm start: one displacement with the predicted multipliers lam0, by the
// update of a Jacobi sweep (per-atom deltas over the atom's constraints in
// ascending order from 0.0, then added), before the unchanged iterations.
// The multiplier totals start from lam0.
__global__ void warm_start_apply(ClusterArgs c, double *pos, int n_atoms) {
    int cl = blockIdx.x * blockDim.x + threadIdx.x;
    if (cl >= c.n_clusters || c.status->error) return;
    const int nc = c.n_constr;
    if (c.lam_sum)
        for (int q = c.cl_cstart[cl]; q < c.cl_cstart[cl + 1]; q++) c.lam_sum[c.cl_cons[q]] = c.lam0[c.cl_cons[q]];
    for (int q = c.cl_astart[cl]; q < c.cl_astart[cl + 1]; q++) {
        const int a = c.cl_atoms[q];
        const double inv_m = c.inv_mass[a];
        double ddx = 0.0, ddy = 0.0, ddz = 0.0;
        for (int r = c.cl_acstart[q]; r < c.cl_acstart[q + 1]; r++) {
            const int ref = c.cl_acons[r];
            const int k = ref >= 0 ? ref : -ref - 1;
            const double w = c.lam0[k] * inv_m;
            const double tx = w * c.rvec[k], ty = w * c.rvec[nc + k], tz = w * c.rvec[2 * nc + k];
            if (ref < 0) { ddx -= tx; ddy -= ty; ddz -= tz; }
            else { ddx += tx; ddy += ty; ddz += tz; }
        }
        pos[a] += ddx;
        pos[n_atoms + a] += ddy;
        pos[2 * n_atoms + a] += ddz;
    }
}

template <bool RATTLE>
__global__ void cluster_phase1(ClusterArgs c, double *pos, double *vel, int n_atoms) {
    int cl = blockIdx.x * blockDim.x + threadIdx.x;
    if (cl >= c.n_clusters || c.status->error) return;
    double mx = 0.0;
    int worst = 0;
    unsigned it = 0;
    bool ok = false;
    while (it < c.max_iter) {
        if (RATTLE) rattle_iteration(c, cl, pos, vel, n_atoms, mx, worst);
        else shake_iteration(c, cl, c.rvec, pos, n_atoms, mx, worst);
        it++;
        if (mx < c.tol) { ok = true; break; }
    }
    c.cl_iters[cl] = (int)it;
    c.cl_worst[cl] = mx;
    c.cl_worst_idx[cl] = worst;
    if (!ok) {
        atomicOr(&c.status->error, RATTLE ? (unsigned)GM_DEV_RATTLE_FAIL : (unsigned)GM_DEV_SHAKE_FAIL);
        atomicMin(&c.status->fail_step, c.status->step);
    }
    atomicMax(RATTLE ? &c.status->rattle_T : &c.status->shake_T, it);
}

template <bool RATTLE>
__global__ void cluster_phase2(ClusterArgs c, double *pos, double *vel, int n_atoms) {
    int cl = blockIdx.x * blockDim.x + threadIdx.x;
    if (cl >= c.n_clusters) return;
    const unsigned T = RATTLE ? c.status->rattle_T : c.status->shake_T;
    if ((c.status->error & ~(unsigned)(GM_DEV_SHAKE_FAIL | GM_DEV_RATTLE_FAIL)) != 0) return;
    unsigned it = (unsigned)c.cl_iters[cl];
    if (it >= T) return;
    double mx = c.cl_worst[cl];
    int worst = c.cl_worst_idx[cl];
    while (it < T) {
        if (RATTLE) rattle_iteration(c, cl, pos, vel, n_atoms, mx, worst);
        else shake_iteration(c, cl, c.rvec, pos, n_atoms, mx, worst);
        it++;
    }
    c.cl_iters[cl] = (int)it;
    c.cl_worst[cl] = mx;
    c.cl_worst_idx[cl] = worst;
    // the global stop at T needs every cluster below tol at iteration T
    if (!(mx < c.tol) && T < c.max_iter) atomicOr(&c.status->error, (unsigned)GM_DEV_ITER_MISMATCH);
}

__global__ void reset_T(DevStatus *st, int rattle) {
    if (rattle) st->rattle_T = 0; else st->shake_T = 0;
}

__global__ void step_kernel(DevStatus *st) {
    if (st->error) return;
    st->step += 1;
    if (st->shake_T || st->rattle_T) {
        st->c_steps += 1;
        st->shake_sum += st->shake_T;
        st->rattle_sum += st->rattle_T;
    }
}

__global__ void kinetic_partial(int n, const double *vel, const double *mass, double *partial) {
    __shared__ double s[256];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double vx = vel[i], vy = vel[n + i], vz = vel[2 * n + i];
        acc += mass[i] * (vx * vx + vy * vy + vz * vz);
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void kinetic_final(const double *partial, int blocks, double *out) {
    if (threadIdx.x != 0) return;
    double sum = 0.0;
    for (int b = 0; b < blocks; b++) sum += partial[b];
    *out = 0.5 * sum * (1.0 / (20.455 * 20.455));  // lib.rs:25,76
}

__global__ void differs_kernel(int n3, const double *a, const double *b, unsigned int *flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int d = 0;
    if (i < n3) d = __double_as_longlong(a[i]) != __double_as_longlong(b[i]);
    if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(flag, 1u);
}

__global__ void forces_out_kernel(int n3, const long long *force, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) out[i] = (double)force[i] * GM_FIX_INV;
}

}  // namespace

int gm_check_blocks(int n) { return n > 0 ? (n + 255) / 256 : 1; }

void gm_launch_half_kick(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                         const DevStatus *st, cudaStream_t s) {
    if (n) half_kick_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, vel, force, inv_mass, dt_half, st);
}

void gm_launch_half_kick_f64(int n, double *vel, const double *force, const double *inv_mass, double dt_half,
                             cudaStream_t s) {
    if (n) half_kick_f64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, vel, force, inv_mass, dt_half);
}

void gm_launch_drift(int n, double *pos, double *vel, double *dref, double dt, bool resync, const DevStatus *st,
                     cudaStream_t s) {
    if (n) drift_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, vel, dref, dt, resync ? 1 : 0, st);
}

void gm_launch_resync(int n, const double *pos, double *vel, const double *dref, double dt, const DevStatus *st,
                      cudaStream_t s) {
    if (n) resync_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, vel, dref, dt, st);
}

void gm_launch_step(DevStatus *st, cudaStream_t s) { step_kernel<<<1, 1, 0, s>>>(st); }

void gm_launch_check(int n, const double *pos, const double *ref, double thr_sq, DevStatus *st,
                     unsigned long long cond, int blocks, const int *atom_sys, unsigned int *sys_flag, cudaStream_t s) {
    check_kernel<<<blocks, 256, 0, s>>>(n, pos, ref, thr_sq, st, cond, atom_sys, sys_flag);
}

void gm_launch_shake_prepare(const ClusterArgs &c, int n_atoms, const double *dref, cudaStream_t s) {
    if (c.n_clusters == 0) return;
    reset_T<<<1, 1, 0, s>>>(c.status, 0);
    shake_prepare<<<(c.n_constr + 255) / 256, 256, 0, s>>>(c, dref, n_atoms);
}

int gm_launch_shake_solve(const ClusterArgs &c, int n_atoms, double *pos, cudaStream_t s) {
    if (c.n_clusters == 0) return 0;
    const int b = (c.n_clusters + 127) / 128;
    int k = 0;
    if (c.lam0) { warm_start_apply<<<b, 128, 0, s>>>(c, pos, n_atoms); k++; }
    cluster_phase1<false><<<b, 128, 0, s>>>(c, pos, nullptr, n_atoms);
    cluster_phase2<false><<<b, 128, 0, s>>>(c, pos, nullptr, n_atoms);
    return k + 2;
}

void gm_launch_shake(const ClusterArgs &c, int n_atoms, const double *dref, double *pos, cudaStream_t s) {
    gm_launch_shake_prepare(c, n_atoms, dref, s);
    gm_launch_shake_solve(c, n_atoms, pos, s);
}

void gm_launch_rattle(const ClusterArgs &c, int n_atoms, const double *pos, double *vel, cudaStream_t s) {
    if (c.n_clusters == 0) return;
    reset_T<<<1, 1, 0, s>>>(c.status, 1);
    const int b = (c.n_clusters + 127) / 128;
    cluster_phase1<true><<<b, 128, 0, s>>>(c, const_cast<double *>(pos), vel, n_atoms);
    cluster_phase2<true><<<b, 128, 0, s>>>(c, const_cast<double *>(pos), vel, n_atoms);
}

void gm_launch_kinetic(int n, const double *vel, const double *mass, double *partials, int blocks, double *out,
                       cudaStream_t s) {
    kinetic_partial<<<blocks, 256, 0, s>>>(n, vel, mass, partials);
    kinetic_final<<<1, 32, 0, s>>>(partials, blocks, out);
}

void gm_launch_differs(int n, const double *a, const double *b, unsigned int *flag, cudaStream_t s) {
    if (n) differs_kernel<<<(3 * n + 255) / 256, 256, 0, s>>>(3 * n, a, b, flag);
}

void gm_launch_forces_out(int n, const long long *force, double *out, cudaStream_t s) {
    if (n) forces_out_kernel<<<(3 * n + 255) / 256, 256, 0, s>>>(3 * n, force, out);
}
