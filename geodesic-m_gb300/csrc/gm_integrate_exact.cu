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

constexpr double kForceToAccel = GM_FORCE_TO_ACCEL;  // integrator.rs:9

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

__global__ void resync_kernel(int n, const double *pos, double *vel, const double *dref, double dt, double inv_dt,
                              const DevStatus *st) {
    // integrator.rs:64-68 (skipped after a failed projection, like the `?` at integrator.rs:256)
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st->error) return;
    for (int d = 0; d < 3; d++) vel[d * n + i] = gm_div_by_dt(pos[d * n + i] - dref[d * n + i], dt, inv_dt);
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

// The position difference a - b along axis d of a constraint: raw (the
// reference), or at the nearest periodic image when c.mi (bonded_min_image).
// Exact arithmetic (this file builds without FMA contraction), so the raw
// difference is the same bits as before the option existed and the image
// form those of the restated min_image.
__device__ __forceinline__ double cdiff(const ClusterArgs &c, double a, double b, int d) {
    const double v = a - b;
    return c.mi ? gm_min_image(v, c.box64[d]) : v;
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
        const double dx = cdiff(c, pos[i], pos[j], 0);
        const double dy = cdiff(c, pos[n_atoms + i], pos[n_atoms + j], 1);
        const double dz = cdiff(c, pos[2 * n_atoms + i], pos[2 * n_atoms + j], 2);
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
        const double rx = cdiff(c, pos[i], pos[j], 0);
        const double ry = cdiff(c, pos[n_atoms + i], pos[n_atoms + j], 1);
        const double rz = cdiff(c, pos[2 * n_atoms + i], pos[2 * n_atoms + j], 2);
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
    c.rvec[k] = cdiff(c, dref[i], dref[j], 0);
    c.rvec[c.n_constr + k] = cdiff(c, dref[n_atoms + i], dref[n_atoms + j], 1);
    c.rvec[2 * c.n_constr + k] = cdiff(c, dref[2 * n_atoms + i], dref[2 * n_atoms + j], 2);
    if (c.lam_sum) c.lam_sum[k] = 0.0;
}

// A star cluster: NC constraints that all share one centre atom (a heavy
// atom and its NC hydrogens), one cluster per thread with every value in a
// register.  The operations are those of the general sweep in the same
// order: each constraint's multiplier, then each atom's sum over its
// constraints (the centre's in ascending constraint order, from 0.0).
template <bool RATTLE, int NC>
__device__ void cluster_star(const ClusterArgs &c, int cl, double *pos, double *vel, int n, bool phase2) {
    const DevStatus *st = c.status;
    unsigned T = 0;
    if (!phase2) {
        if (st->error) return;
    } else {
        T = RATTLE ? st->rattle_T : st->shake_T;
        if ((st->error & ~(unsigned)(GM_DEV_SHAKE_FAIL | GM_DEV_RATTLE_FAIL)) != 0) return;
        if ((unsigned)c.cl_iters[cl] >= T) return;
    }
    const int c0 = c.cl_cstart[cl];
    int kk[NC], hq[NC];
    bool cen_i[NC];  // the centre is the constraint's i (it subtracts)
    {
        const int k0 = c.cl_cons[c0], k1 = c.cl_cons[c0 + 1];
        const int i0 = c.constr_i[k0], j0 = c.constr_j[k0];
        const int cen_ = (i0 == c.constr_i[k1] || i0 == c.constr_j[k1]) ? i0 : j0;
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const int k = c.cl_cons[c0 + q];
            kk[q] = k;
            const int i = c.constr_i[k];
            cen_i[q] = i == cen_;
            hq[q] = cen_i[q] ? c.constr_j[k] : i;
        }
        // centre
        const int cen = cen_;
        const double inv_c = c.inv_mass[cen];
        double *v = RATTLE ? vel : pos;
        double cx = v[cen], cy = v[n + cen], cz = v[2 * n + cen];
        double hx[NC], hy[NC], hz[NC], inv_h[NC], rx[NC], ry[NC], rz[NC], wq[NC], dsq[NC], acc[NC];
        const int ncst = c.n_constr;
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const int h = hq[q];
            hx[q] = v[h]; hy[q] = v[n + h]; hz[q] = v[2 * n + h];
            inv_h[q] = c.inv_mass[h];
            const int k = kk[q];
            const double inv_mi = cen_i[q] ? inv_c : inv_h[q], inv_mj = cen_i[q] ? inv_h[q] : inv_c;
            if (!RATTLE) {
                dsq[q] = c.constr_dsq[k];
                rx[q] = c.rvec[k]; ry[q] = c.rvec[ncst + k]; rz[q] = c.rvec[2 * ncst + k];
                wq[q] = 2.0 * (inv_mi + inv_mj);
            } else {
                const int i = cen_i[q] ? cen : h, j = cen_i[q] ? h : cen;
                rx[q] = cdiff(c, pos[i], pos[j], 0);
                ry[q] = cdiff(c, pos[n + i], pos[n + j], 1);
                rz[q] = cdiff(c, pos[2 * n + i], pos[2 * n + j], 2);
                const double rsq = rx[q] * rx[q] + ry[q] * ry[q] + rz[q] * rz[q];
                wq[q] = (inv_mi + inv_mj) * rsq;
                dsq[q] = 0.0;
            }
            acc[q] = 0.0;
        }
        const bool keep_sum = !RATTLE && c.lam_sum;
        double lam[NC];
        unsigned it;
        double mx;
        int worst;
        bool apply_first = false;
        if (!phase2) {
            it = 0;
            mx = 0.0;
            worst = 0;
            if (!RATTLE && c.lam0) {
#pragma unroll
                for (int q = 0; q < NC; q++) { acc[q] = c.lam0[kk[q]]; lam[q] = acc[q]; }
                apply_first = true;
            }
        } else {
            it = (unsigned)c.cl_iters[cl];
            mx = c.cl_worst[cl];
            worst = c.cl_worst_idx[cl];
            if (keep_sum)
#pragma unroll
                for (int q = 0; q < NC; q++) acc[q] = c.lam_sum[kk[q]];
        }
        bool ok = false;
        const unsigned stop = phase2 ? T : c.max_iter;
        while (true) {
            if (!apply_first) {
                if (it >= stop) break;
                double m_ = 0.0;
                int w_ = kk[0];
#pragma unroll
                for (int q = 0; q < NC; q++) {
                    // the constraint's i minus its j
                    const double xi = cen_i[q] ? cx : hx[q], yi = cen_i[q] ? cy : hy[q], zi = cen_i[q] ? cz : hz[q];
                    const double xj = cen_i[q] ? hx[q] : cx, yj = cen_i[q] ? hy[q] : cy, zj = cen_i[q] ? hz[q] : cz;
                    double l_;
                    if (RATTLE) {
                        const double dvx = xi - xj;
                        const double dvy = yi - yj;
                        const double dvz = zi - zj;
                        const double rel_vel = dvx * rx[q] + dvy * ry[q] + dvz * rz[q];
                        l_ = wq[q] == 0.0 ? 0.0 : rel_vel / wq[q];
                    } else {
                        const double dx = cdiff(c, xi, xj, 0);
                        const double dy = cdiff(c, yi, yj, 1);
                        const double dz = cdiff(c, zi, zj, 2);
                        const double diff = dx * dx + dy * dy + dz * dz - dsq[q];
                        const double dot_new_old = dx * rx[q] + dy * ry[q] + dz * rz[q];
                        const double denom = wq[q] * dot_new_old;
                        l_ = denom == 0.0 ? 0.0 : diff / denom;
                        if (keep_sum) acc[q] += l_;
                    }
                    lam[q] = l_;
                    const double la = fabs(l_);
                    if (la > m_) { m_ = la; w_ = kk[q]; }
                }
                mx = m_;
                worst = w_;
            }
            // atoms: the centre over its constraints in ascending order, then each H
            double ddx = 0.0, ddy = 0.0, ddz = 0.0;
#pragma unroll
            for (int q = 0; q < NC; q++) {
                const double w = lam[q] * inv_c;
                const double tx = w * rx[q], ty = w * ry[q], tz = w * rz[q];
                if (cen_i[q]) { ddx -= tx; ddy -= ty; ddz -= tz; }
                else { ddx += tx; ddy += ty; ddz += tz; }
            }
            cx += ddx; cy += ddy; cz += ddz;
#pragma unroll
            for (int q = 0; q < NC; q++) {
                const double w = lam[q] * inv_h[q];
                const double tx = w * rx[q], ty = w * ry[q], tz = w * rz[q];
                double ex = 0.0, ey = 0.0, ez = 0.0;
                if (cen_i[q]) { ex += tx; ey += ty; ez += tz; }
                else { ex -= tx; ey -= ty; ez -= tz; }
                hx[q] += ex; hy[q] += ey; hz[q] += ez;
            }
            if (apply_first) { apply_first = false; continue; }
            it++;
            if (!phase2 && mx < c.tol) { ok = true; break; }
        }
        v[cen] = cx; v[n + cen] = cy; v[2 * n + cen] = cz;
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const int h = hq[q];
            v[h] = hx[q]; v[n + h] = hy[q]; v[2 * n + h] = hz[q];
            if (keep_sum) c.lam_sum[kk[q]] = acc[q];
        }
        c.cl_iters[cl] = (int)it;
        c.cl_worst[cl] = mx;
        c.cl_worst_idx[cl] = worst;
        if (!phase2) {
            if (!ok) {
                atomicOr(&c.status->error, RATTLE ? (unsigned)GM_DEV_RATTLE_FAIL : (unsigned)GM_DEV_SHAKE_FAIL);
                atomicMin(&c.status->fail_step, c.status->step);
            }
            atomicMax(RATTLE ? &c.status->rattle_T : &c.status->shake_T, it);
        } else if (!(mx < c.tol) && T < c.max_iter) {
            atomicOr(&c.status->error, (unsigned)GM_DEV_ITER_MISMATCH);
        }
    }
}

template <bool RATTLE>
__device__ void cluster_star_any(const ClusterArgs &c, int cl, double *pos, double *vel, int n, bool phase2) {
    switch (c.cl_cstart[cl + 1] - c.cl_cstart[cl]) {
        case 2: cluster_star<RATTLE, 2>(c, cl, pos, vel, n, phase2); break;
        case 3: cluster_star<RATTLE, 3>(c, cl, pos, vel, n, phase2); break;
        case 4: cluster_star<RATTLE, 4>(c, cl, pos, vel, n, phase2); break;
        case 5: cluster_star<RATTLE, 5>(c, cl, pos, vel, n, phase2); break;
        case 6: cluster_star<RATTLE, 6>(c, cl, pos, vel, n, phase2); break;
        case 7: cluster_star<RATTLE, 7>(c, cl, pos, vel, n, phase2); break;
        default: cluster_star<RATTLE, 8>(c, cl, pos, vel, n, phase2); break;
    }
}

// Clusters of 2-32 constraints on at most 32 atoms (a heavy atom with its H
// atoms): one warp per cluster.  Lane a keeps atom a's coordinates and its
// constraint list in registers, lane q keeps constraint q's bond vector and
// multiplier; values move between lanes by shuffles.  Each lane's arithmetic
// is that of shake_iteration / rattle_iteration in the same order, and the
// largest |lambda| and its constraint (the first in ascending order on ties)
// come from a warp reduction, so the bits are those of the sequential sweep.
constexpr int kWarpRefs = 8;  // constraints per atom handled by the warp path

// Lane a < na adds its atom's displacement over its constraints (ascending,
// from 0.0): every lane runs the loop to the warp's longest list so that
// every shuffle has all 32 lanes.
__device__ __forceinline__ void warp_atom_update(int lane, int na, int nref, int maxref, const int *ref_l,
                                                 const int *ref_s, double im_a, double lam, double rx, double ry,
                                                 double rz, double &X, double &Y, double &Z) {
    double ddx = 0.0, ddy = 0.0, ddz = 0.0;
    for (int r = 0; r < maxref; r++) {
        const bool mine = lane < na && r < nref;
        const int l = mine ? ref_l[r] : 0;
        const double lam_l = __shfl_sync(0xffffffffu, lam, l);
        const double rx_l = __shfl_sync(0xffffffffu, rx, l);
        const double ry_l = __shfl_sync(0xffffffffu, ry, l);
        const double rz_l = __shfl_sync(0xffffffffu, rz, l);
        if (mine) {
            const double w = lam_l * im_a;
            const double tx = w * rx_l, ty = w * ry_l, tz = w * rz_l;
            if (ref_s[r] < 0) { ddx -= tx; ddy -= ty; ddz -= tz; }
            else { ddx += tx; ddy += ty; ddz += tz; }
        }
    }
    if (lane < na) {
        X += ddx;
        Y += ddy;
        Z += ddz;
    }
}

template <bool RATTLE>
__device__ void cluster_warp(const ClusterArgs &c, int cl, double *pos, double *vel, int n, bool phase2) {
    const int lane = threadIdx.x & 31;
    const DevStatus *st = c.status;
    unsigned T = 0;
    if (!phase2) {
        if (st->error) return;
    } else {
        T = RATTLE ? st->rattle_T : st->shake_T;
        if ((st->error & ~(unsigned)(GM_DEV_SHAKE_FAIL | GM_DEV_RATTLE_FAIL)) != 0) return;
        if ((unsigned)c.cl_iters[cl] >= T) return;
    }
    const int c0 = c.cl_cstart[cl], nc = c.cl_cstart[cl + 1] - c0;
    const int a0 = c.cl_astart[cl], na = c.cl_astart[cl + 1] - a0;
    const int ncst = c.n_constr;
    double *v = RATTLE ? vel : pos;
    // atoms: lane a holds atom a and its constraint list (local indices)
    int ag = 0;
    double im_a = 0.0, X = 0.0, Y = 0.0, Z = 0.0;
    int nref = 0, ref_l[kWarpRefs], ref_s[kWarpRefs];
    if (lane < na) {
        ag = c.cl_atoms[a0 + lane];
        im_a = c.inv_mass[ag];
        X = v[ag]; Y = v[n + ag]; Z = v[2 * n + ag];
        const int r0 = c.cl_acstart[a0 + lane], r1 = c.cl_acstart[a0 + lane + 1];
        for (int r = r0; r < r1 && nref < kWarpRefs; r++) {
            const int ref = c.cl_acons[r];
            const int kk = ref >= 0 ? ref : -ref - 1;
            int l = 0;
            for (int t = 0; t < nc; t++) if (c.cl_cons[c0 + t] == kk) l = t;
            ref_l[nref] = l;
            ref_s[nref] = ref >= 0 ? 1 : -1;
            nref++;
        }
    }
    int maxref = nref;
    for (int o = 16; o > 0; o >>= 1) maxref = max(maxref, __shfl_xor_sync(0xffffffffu, maxref, o));
    // constraints: lane q holds constraint q
    int k = 0, il = 0, jl = 0;
    double wq = 0.0, dsq = 0.0, acc = 0.0, rx = 0.0, ry = 0.0, rz = 0.0, lam = 0.0;
    if (lane < nc) {
        k = c.cl_cons[c0 + lane];
        const int i = c.constr_i[k], j = c.constr_j[k];
        for (int t = 0; t < na; t++) {
            const int a = c.cl_atoms[a0 + t];
            if (a == i) il = t;
            if (a == j) jl = t;
        }
        const double inv_mi = c.inv_mass[i], inv_mj = c.inv_mass[j];
        if (!RATTLE) {
            dsq = c.constr_dsq[k];
            rx = c.rvec[k]; ry = c.rvec[ncst + k]; rz = c.rvec[2 * ncst + k];
            wq = 2.0 * (inv_mi + inv_mj);
        } else {
            // constraint.rs:205-215: the bond vector of the fixed positions
            rx = cdiff(c, pos[i], pos[j], 0);
            ry = cdiff(c, pos[n + i], pos[n + j], 1);
            rz = cdiff(c, pos[2 * n + i], pos[2 * n + j], 2);
            const double rsq = rx * rx + ry * ry + rz * rz;
            wq = (inv_mi + inv_mj) * rsq;
        }
    }
    const int k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool keep_sum = !RATTLE && c.lam_sum;
    unsigned it;
    double mx;
    int worst;
    if (!phase2) {
        it = 0;
        mx = 0.0;
        worst = 0;
        if (!RATTLE && c.lam0) {
            if (lane < nc) { acc = c.lam0[k]; lam = acc; }
            warp_atom_update(lane, na, nref, maxref, ref_l, ref_s, im_a, lam, rx, ry, rz, X, Y, Z);
        }
    } else {
        it = (unsigned)c.cl_iters[cl];
        mx = c.cl_worst[cl];
        worst = c.cl_worst_idx[cl];
        if (keep_sum && lane < nc) acc = c.lam_sum[k];
    }
    bool ok = false;
    const unsigned stop = phase2 ? T : c.max_iter;
    while (it < stop) {
        // constraint lanes fetch their two atoms
        const double xi = __shfl_sync(0xffffffffu, X, il), yi = __shfl_sync(0xffffffffu, Y, il),
                     zi = __shfl_sync(0xffffffffu, Z, il);
        const double xj = __shfl_sync(0xffffffffu, X, jl), yj = __shfl_sync(0xffffffffu, Y, jl),
                     zj = __shfl_sync(0xffffffffu, Z, jl);
        double la = 0.0;
        lam = 0.0;
        if (lane < nc) {
            double l_;
            if (RATTLE) {
                const double dvx = xi - xj;
                const double dvy = yi - yj;
                const double dvz = zi - zj;
                const double rel_vel = dvx * rx + dvy * ry + dvz * rz;
                l_ = wq == 0.0 ? 0.0 : rel_vel / wq;
            } else {
                const double dx = cdiff(c, xi, xj, 0);
                const double dy = cdiff(c, yi, yj, 1);
                const double dz = cdiff(c, zi, zj, 2);
                const double diff = dx * dx + dy * dy + dz * dz - dsq;
                const double dot_new_old = dx * rx + dy * ry + dz * rz;
                const double denom = wq * dot_new_old;
                l_ = denom == 0.0 ? 0.0 : diff / denom;
                if (keep_sum) acc += l_;
            }
            la = fabs(l_);
            lam = l_;
        }
        // the largest |lambda| (a NaN never wins, as with the sequential '>')
        // and the first constraint that reaches it
        double m = la > 0.0 ? la : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        const unsigned hit = __ballot_sync(0xffffffffu, lane < nc && la == m && m > 0.0);
        worst = __shfl_sync(0xffffffffu, k, hit ? __ffs(hit) - 1 : 0);
        if (!hit) worst = k0;
        mx = m;
        warp_atom_update(lane, na, nref, maxref, ref_l, ref_s, im_a, lam, rx, ry, rz, X, Y, Z);
        it++;
        if (!phase2 && mx < c.tol) { ok = true; break; }
    }
    if (lane < na) { v[ag] = X; v[n + ag] = Y; v[2 * n + ag] = Z; }
    if (keep_sum && lane < nc) c.lam_sum[k] = acc;
    if (lane == 0) {
        c.cl_iters[cl] = (int)it;
        c.cl_worst[cl] = mx;
        c.cl_worst_idx[cl] = worst;
        if (!phase2) {
            if (!ok) {
                atomicOr(&c.status->error, RATTLE ? (unsigned)GM_DEV_RATTLE_FAIL : (unsigned)GM_DEV_SHAKE_FAIL);
                atomicMin(&c.status->fail_step, c.status->step);
            }
            atomicMax(RATTLE ? &c.status->rattle_T : &c.status->shake_T, it);
        } else if (!(mx < c.tol) && T < c.max_iter) {
            atomicOr(&c.status->error, (unsigned)GM_DEV_ITER_MISMATCH);
        }
    }
}

// The per-atom update of a one-constraint cluster for multiplier l: atom i
// subtracts, atom j adds, each sum starting from 0.0.
__device__ __forceinline__ void single_apply(double l, double inv_mi, double inv_mj, double rx, double ry, double rz,
                                             double &xi, double &yi, double &zi, double &xj, double &yj, double &zj) {
    const double wi = l * inv_mi;
    double ddx = 0.0, ddy = 0.0, ddz = 0.0;
    ddx -= wi * rx; ddy -= wi * ry; ddz -= wi * rz;
    const double wj = l * inv_mj;
    double edx = 0.0, edy = 0.0, edz = 0.0;
    edx += wj * rx; edy += wj * ry; edz += wj * rz;
    xi += ddx; yi += ddy; zi += ddz;
    xj += edx; yj += edy; zj += edz;
}

// A cluster of one constraint (one heavy atom and one H: most H-bond
// clusters) entirely in scalar registers.  The operations are those of the
// general path in the same order, including the per-atom sums that start
// from 0.0, so the bits are the same.
template <bool RATTLE>
__device__ void cluster_single(const ClusterArgs &c, int cl, double *pos, double *vel, int n, bool phase2) {
    const DevStatus *st = c.status;
    unsigned T = 0;
    if (!phase2) {
        if (st->error) return;
    } else {
        T = RATTLE ? st->rattle_T : st->shake_T;
        if ((st->error & ~(unsigned)(GM_DEV_SHAKE_FAIL | GM_DEV_RATTLE_FAIL)) != 0) return;
        if ((unsigned)c.cl_iters[cl] >= T) return;
    }
    const int k = c.cl_cons[c.cl_cstart[cl]];
    const int i = c.constr_i[k], j = c.constr_j[k];
    const double inv_mi = c.inv_mass[i], inv_mj = c.inv_mass[j];
    double *v = RATTLE ? vel : pos;
    double xi = v[i], yi = v[n + i], zi = v[2 * n + i];
    double xj = v[j], yj = v[n + j], zj = v[2 * n + j];
    const int ncst = c.n_constr;
    double rx, ry, rz, wq, dsq = 0.0;
    if (!RATTLE) {
        dsq = c.constr_dsq[k];
        rx = c.rvec[k]; ry = c.rvec[ncst + k]; rz = c.rvec[2 * ncst + k];
        wq = 2.0 * (inv_mi + inv_mj);
    } else {
        rx = cdiff(c, pos[i], pos[j], 0);
        ry = cdiff(c, pos[n + i], pos[n + j], 1);
        rz = cdiff(c, pos[2 * n + i], pos[2 * n + j], 2);
        const double rsq = rx * rx + ry * ry + rz * rz;
        wq = (inv_mi + inv_mj) * rsq;
    }
    const bool keep_sum = !RATTLE && c.lam_sum;
    double acc = 0.0;
    unsigned it;
    double mx;
    int worst;
    if (!phase2) {
        it = 0;
        mx = 0.0;
        worst = 0;
        if (!RATTLE && c.lam0) {
            acc = c.lam0[k];
            single_apply(acc, inv_mi, inv_mj, rx, ry, rz, xi, yi, zi, xj, yj, zj);
        }
    } else {
        it = (unsigned)c.cl_iters[cl];
        mx = c.cl_worst[cl];
        worst = c.cl_worst_idx[cl];
        if (keep_sum) acc = c.lam_sum[k];
    }
    bool ok = false;
    const unsigned stop = phase2 ? T : c.max_iter;
    while (it < stop) {
        double l_;
        if (RATTLE) {
            const double dvx = xi - xj;
            const double dvy = yi - yj;
            const double dvz = zi - zj;
            const double rel_vel = dvx * rx + dvy * ry + dvz * rz;
            l_ = wq == 0.0 ? 0.0 : rel_vel / wq;
        } else {
            const double dx = cdiff(c, xi, xj, 0);
            const double dy = cdiff(c, yi, yj, 1);
            const double dz = cdiff(c, zi, zj, 2);
            const double diff = dx * dx + dy * dy + dz * dz - dsq;
            const double dot_new_old = dx * rx + dy * ry + dz * rz;
            const double denom = wq * dot_new_old;
            l_ = denom == 0.0 ? 0.0 : diff / denom;
            if (keep_sum) acc += l_;
        }
        const double la = fabs(l_);
        mx = 0.0;
        worst = k;
        if (la > mx) mx = la;
        single_apply(l_, inv_mi, inv_mj, rx, ry, rz, xi, yi, zi, xj, yj, zj);
        it++;
        if (!phase2 && mx < c.tol) { ok = true; break; }
    }
    v[i] = xi; v[n + i] = yi; v[2 * n + i] = zi;
    v[j] = xj; v[n + j] = yj; v[2 * n + j] = zj;
    if (keep_sum) c.lam_sum[k] = acc;
    c.cl_iters[cl] = (int)it;
    c.cl_worst[cl] = mx;
    c.cl_worst_idx[cl] = worst;
    if (!phase2) {
        if (!ok) {
            atomicOr(&c.status->error, RATTLE ? (unsigned)GM_DEV_RATTLE_FAIL : (unsigned)GM_DEV_SHAKE_FAIL);
            atomicMin(&c.status->fail_step, c.status->step);
        }
        atomicMax(RATTLE ? &c.status->rattle_T : &c.status->shake_T, it);
    } else if (!(mx < c.tol) && T < c.max_iter) {
        atomicOr(&c.status->error, (unsigned)GM_DEV_ITER_MISMATCH);
    }
}

// Warm start: one displacement with the predicted multipliers lam0, by the
// update of a Jacobi sweep (per-atom deltas over the atom's constraints in
// ascending order from 0.0, then added), before the unchanged iterations.
// The multiplier totals start from lam0.
// Clusters come in four ranges, launched with 32-thread blocks:
// [0, n_single) one constraint, one per thread; [n_single, n_star_end)
// stars of 2-8 constraints, one per thread; [n_star_end, n_warp_end) other
// clusters of 2-32 constraints, one per warp; the rest one per thread
// through global memory.
struct ClusterBlocks {
    int single, star, warp, big;
};

__host__ __device__ __forceinline__ ClusterBlocks cluster_block_ranges(const ClusterArgs &c) {
    ClusterBlocks b;
    b.single = (c.n_single + 31) / 32;
    b.star = (c.n_star_end - c.n_single + 31) / 32;
    b.warp = c.n_warp_end - c.n_star_end;
    b.big = (c.n_clusters - c.n_warp_end + 31) / 32;
    return b;
}

int cluster_blocks(const ClusterArgs &c) {
    const ClusterBlocks b = cluster_block_ranges(c);
    return b.single + b.star + b.warp + b.big;
}

// Runs the cluster of this thread (or warp) by its class; false for the
// global-memory class, which the caller handles, with *cl set.
template <bool RATTLE>
__device__ __forceinline__ bool cluster_dispatch(const ClusterArgs &c, double *pos, double *vel, int n, bool phase2,
                                                 int *cl) {
    const ClusterBlocks b = cluster_block_ranges(c);
    int blk = blockIdx.x;
    if (blk < b.single) {
        const int q = blk * 32 + threadIdx.x;
        if (q < c.n_single) cluster_single<RATTLE>(c, q, pos, vel, n, phase2);
        return true;
    }
    blk -= b.single;
    if (blk < b.star) {
        const int q = c.n_single + blk * 32 + threadIdx.x;
        if (q < c.n_star_end) cluster_star_any<RATTLE>(c, q, pos, vel, n, phase2);
        return true;
    }
    blk -= b.star;
    if (blk < b.warp) {
        cluster_warp<RATTLE>(c, c.n_star_end + blk, pos, vel, n, phase2);
        return true;
    }
    blk -= b.warp;
    *cl = c.n_warp_end + blk * 32 + threadIdx.x;
    return false;
}

__global__ void warm_start_apply(ClusterArgs c, double *pos, int n_atoms) {
    // big clusters only: the other paths apply the warm start themselves
    const ClusterBlocks b = cluster_block_ranges(c);
    const int blk = (int)blockIdx.x - b.single - b.star - b.warp;
    if (blk < 0) return;
    const int cl = c.n_warp_end + blk * 32 + threadIdx.x;
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
    int cl = 0;
    if (cluster_dispatch<RATTLE>(c, pos, vel, n_atoms, false, &cl)) return;
    if (cl >= c.n_clusters) return;
    if (c.status->error) return;
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
    int cl = 0;
    if (cluster_dispatch<RATTLE>(c, pos, vel, n_atoms, true, &cl)) return;
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

// Trajectory frame (see gm_launch_frame).  The completed step count is the
// counter plus one while the unconstrained step's closing half-kick is still
// pending; every block takes the same early exit.
__global__ void __launch_bounds__(256) frame_kernel(int n, const double *pos, const double *vel,
                                                    const long long *force, const double *inv_mass,
                                                    const double *mass, double dt_half, DevStatus *st, FrameArgs f) {
    const bool tail = st->tail_pending != 0;
    const unsigned long long step = st->step + (tail ? 1ull : 0ull);
    if (st->error || f.interval <= 0 || step % (unsigned long long)f.interval != 0) return;
    const unsigned slot = st->frame_n;  // every block reads it before the last block advances it
    const bool store = slot < (unsigned)f.cap;
    float *fx = f.xyz + (size_t)(store ? slot : 0) * 3 * (size_t)n;
    __shared__ double s[256];
    __shared__ bool last;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double v[3];
        for (int d = 0; d < 3; d++) {
            if (store) fx[(size_t)d * n + i] = (float)pos[d * n + i];
            v[d] = vel[d * n + i];
            if (tail) {
                const double fd = (double)force[d * n + i] * GM_FIX_INV;
                v[d] += dt_half * fd * inv_mass[i] * kForceToAccel;
            }
        }
        acc += mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);  // kinetic_partial's order
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        f.partial[blockIdx.x] = s[0];
        __threadfence();
        last = atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double e_pot = gm_block_sum256(f.epart, f.n_epart, s);
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int b = 0; b < (int)gridDim.x; b++) sum += ((volatile double *)f.partial)[b];
        const double e_kin = 0.5 * sum * (1.0 / (20.455 * 20.455));  // kinetic_final
        st->blocks_done = 0;
        if (store) {
            f.step[slot] = step;
            f.energy[2 * slot] = e_pot;
            f.energy[2 * slot + 1] = e_kin;
            st->frame_n = slot + 1;
        } else {
            st->frame_lost += 1;
        }
    }
}

__global__ void kinetic_final(const double *partial, int blocks, double *out) {
    if (threadIdx.x != 0) return;
    double sum = 0.0;
    for (int b = 0; b < blocks; b++) sum += partial[b];
    *out = 0.5 * sum * (1.0 / (20.455 * 20.455));  // lib.rs:25,76
}

// flag |= 1 when a differs from b anywhere (bit for bit), |= 2 when a holds
// a non-finite value
__global__ void differs_kernel(int n3, const double *a, const double *b, unsigned int *flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int d = 0, bad = 0;
    if (i < n3) {
        d = __double_as_longlong(a[i]) != __double_as_longlong(b[i]);
        bad = !isfinite(a[i]);
    }
    d = __syncthreads_or(d);
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0 && (d || bad)) atomicOr(flag, (d ? 1u : 0u) | (bad ? 2u : 0u));
}

__global__ void status_reset_kernel(DevStatus *st, int set_step, unsigned long long step) {
    DevStatus z{};
    z.fail_step = ~0ull;
    z.n_rebuilds = st->n_rebuilds;
    z.step = set_step ? step : st->step;
    z.c_steps = st->c_steps;
    z.shake_sum = st->shake_sum;
    z.rattle_sum = st->rattle_sum;
    z.rec_n = st->rec_n;
    z.frame_n = st->frame_n;
    z.frame_lost = st->frame_lost;
    z.rebuild_base = st->n_rebuilds;
    *st = z;
}

__global__ void forces_out_kernel(int n3, const long long *force, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) out[i] = (double)force[i] * GM_FIX_INV;
}

}  // namespace

// half_kick_kernel, drift_kernel (resync), check_kernel and pack_kernel's
// per-atom work fused for systems without constraints: one atom per thread,
// the same operations in the same order (a rebuild that the check triggers
// packs again with the new grid).  A block that finds a non-finite position marks bad_pending instead of
// error, and the last block moves it to error, so every block of the launch
// reads the error word as it stood before the launch (as the separate kick and
// drift kernels do).
__global__ void kick_drift_check_kernel(int n, double *pos, double *vel, double *dref, long long *force,
                                        const double *inv_mass, double dt_half, double dt, double inv_dt,
                                        const double *ref, double thr_sq, DevStatus *st, unsigned long long cond,
                                        const int *atom_sys, unsigned int *sys_flag, PackArgs pk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int need = 0, bad = 0;
    // read by every block before the last block updates them
    const bool err0 = st->error != 0, tail0 = st->tail_pending != 0;
    if (i < n) {
        double np[3];
        if (!err0) {
            const double inv_m = inv_mass[i];
            for (int d = 0; d < 3; d++) {
                const double f = (double)force[d * n + i] * GM_FIX_INV;
                // the previous step's closing half-kick (same forces) when it
                // is pending, then this step's opening one: two additions in
                // the order of the separate kernels
                const double kick = dt_half * f * inv_m * kForceToAccel;
                double v = vel[d * n + i];
                if (tail0) v = v + kick;
                v = v + kick;
                const double p = pos[d * n + i];
                dref[d * n + i] = p;
                np[d] = p + dt * v;
                pos[d * n + i] = np[d];
                vel[d * n + i] = gm_div_by_dt(np[d] - p, dt, inv_dt);
            }
        } else {
            for (int d = 0; d < 3; d++) np[d] = pos[d * n + i];
        }
        // pack_kernel's work for this atom, from the same FP64 position
        const int sl = pk.slot_of[i];
        const GridInfo *g = pk.grid + atom_sys[i];
        gm_pack_record(pk.coord + 2 * sl, np[0] - g->origin[0], np[1] - g->origin[1], np[2] - g->origin[2], pk.qw[i]);
        if (pk.fp64) {
            pk.pos64s[sl] = make_double4(np[0], np[1], np[2], pk.charge64[i]);
            pk.type_sorted[sl] = pk.type[i];
        }
        for (int d = 0; d < 3; d++) force[d * n + i] = 0;
        bad = !(isfinite(np[0]) && isfinite(np[1]) && isfinite(np[2]));
        const double dx = np[0] - ref[i], dy = np[1] - ref[n + i], dz = np[2] - ref[2 * n + i];
        need = dx * dx + dy * dy + dz * dz > thr_sq;
        if (need) sys_flag[atom_sys[i]] = 1u;
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
            if (cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, (r && !e) ? 1u : 0u);
            // the previous step is complete; this one's closing half-kick is
            // left to the next step's kernel or the finalizer
            if (!err0) {
                if (tail0) st->step += 1;
                st->tail_pending = 1u;
            }
        }
    }
}
// The closing half-kick of the last unconstrained resident step and its step
// count, when pending; the last block clears the flag after every block has
// read it.
__global__ void kick_tail_kernel(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                                 DevStatus *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool go = st->tail_pending != 0 && st->error == 0;
    if (i < n && go) {
        const double inv_m = inv_mass[i];
        for (int d = 0; d < 3; d++) {
            const double f = (double)force[d * n + i] * GM_FIX_INV;
            vel[d * n + i] += dt_half * f * inv_m * kForceToAccel;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned done = atomicAdd(&st->blocks_done, 1u);
        if (done == gridDim.x - 1) {
            st->blocks_done = 0;
            if (go) st->step += 1;
            st->tail_pending = 0u;
        }
    }
}
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
    if (n) resync_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, vel, dref, dt, 1.0 / dt, st);
}

void gm_launch_step(DevStatus *st, cudaStream_t s) { step_kernel<<<1, 1, 0, s>>>(st); }
void gm_launch_kick_drift_check(int n, double *pos, double *vel, double *dref, long long *force,
                                const double *inv_mass, double dt_half, double dt, const double *ref, double thr_sq,
                                DevStatus *st, unsigned long long cond, const int *atom_sys, unsigned int *sys_flag,
                                const PackArgs &pk, cudaStream_t s) {
    kick_drift_check_kernel<<<gm_check_blocks(n), 256, 0, s>>>(n, pos, vel, dref, force, inv_mass, dt_half, dt,
                                                              1.0 / dt, ref, thr_sq, st, cond, atom_sys, sys_flag,
                                                              pk);
}
void gm_launch_kick_tail(int n, double *vel, const long long *force, const double *inv_mass, double dt_half,
                         DevStatus *st, cudaStream_t s) {
    kick_tail_kernel<<<gm_check_blocks(n), 256, 0, s>>>(n, vel, force, inv_mass, dt_half, st);
}

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
    // 32-thread blocks over the three cluster ranges: the FP64 pipe of
    // every SM gets a share of the (few) clusters
    const int b = cluster_blocks(c);
    int k = 0;
    if (c.lam0) { warm_start_apply<<<b, 32, 0, s>>>(c, pos, n_atoms); k++; }
    cluster_phase1<false><<<b, 32, 0, s>>>(c, pos, nullptr, n_atoms);
    cluster_phase2<false><<<b, 32, 0, s>>>(c, pos, nullptr, n_atoms);
    return k + 2;
}

void gm_launch_shake(const ClusterArgs &c, int n_atoms, const double *dref, double *pos, cudaStream_t s) {
    gm_launch_shake_prepare(c, n_atoms, dref, s);
    gm_launch_shake_solve(c, n_atoms, pos, s);
}

void gm_launch_rattle(const ClusterArgs &c, int n_atoms, const double *pos, double *vel, cudaStream_t s) {
    if (c.n_clusters == 0) return;
    reset_T<<<1, 1, 0, s>>>(c.status, 1);
    const int b = cluster_blocks(c);
    cluster_phase1<true><<<b, 32, 0, s>>>(c, const_cast<double *>(pos), vel, n_atoms);
    cluster_phase2<true><<<b, 32, 0, s>>>(c, const_cast<double *>(pos), vel, n_atoms);
}

void gm_launch_kinetic(int n, const double *vel, const double *mass, double *partials, int blocks, double *out,
                       cudaStream_t s) {
    kinetic_partial<<<blocks, 256, 0, s>>>(n, vel, mass, partials);
    kinetic_final<<<1, 32, 0, s>>>(partials, blocks, out);
}

void gm_launch_frame(int n, const double *pos, const double *vel, const long long *force, const double *inv_mass,
                     const double *mass, double dt_half, DevStatus *st, const FrameArgs &f, cudaStream_t s) {
    frame_kernel<<<GM_FRAME_BLOCKS, 256, 0, s>>>(n, pos, vel, force, inv_mass, mass, dt_half, st, f);
}
void gm_launch_status_reset(DevStatus *st, int set_step, unsigned long long step, cudaStream_t s) {
    status_reset_kernel<<<1, 1, 0, s>>>(st, set_step, step);
}
void gm_launch_differs(int n, const double *a, const double *b, unsigned int *flag, cudaStream_t s) {
    if (n) differs_kernel<<<(3 * n + 255) / 256, 256, 0, s>>>(3 * n, a, b, flag);
}

void gm_launch_forces_out(int n, const long long *force, double *out, cudaStream_t s) {
    if (n) forces_out_kernel<<<(3 * n + 255) / 256, 256, 0, s>>>(3 * n, force, out);
}
