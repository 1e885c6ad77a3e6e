// gm_force_terms.cuh — the per-item force arithmetic shared by the force
// kernels (gm_force.cu) and the persistent step kernel (gm_step.cu).  Both
// translation units compile these functions with the same flags (FMA
// contraction on), so a force evaluated by either form has the same bits.
//   pair_item_mixed  one warp's share of a 32-atom group's list columns
//   bonded_term      one bond, angle or dihedral (FP64)
//   pair14_term      one scaled 1-4 pair (FP64)
#pragma once
#include "gm_internal.cuh"

namespace {

constexpr int kChunk = 32;
constexpr int kBatch = 4;  // list entries gathered together in the mixed pair kernel

// MUFU approximations of 1/x and 1/sqrt(x); the double-float corrections
// that follow them absorb their few-ulp error.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Minimum image of a pair difference held as dh (a multiple of 2^-8) plus
// dl: the image shift n L is taken with L as a double-float, dh - n L_hi is
// exact (Sterbenz), and the result is put back on the 2^-8 grid so that its
// square stays exact.
__device__ __forceinline__ void image_df(float &dh, float &dl, float L, float Llo, float iL) {
    const float k = rintf(dh * iL);
    dh = fmaf(-k, L, dh);
    dl = fmaf(-k, Llo, dl);
    const float q = rintf(dh * 256.f) * (1.f / 256.f);
    dl += dh - q;
    dh = q;
}

// One work item of the mixed-precision nonbonded kernel (force/nonbonded.rs:20-82
// physics plus the switched Coulomb term): FP32 operations throughout, arranged as
// double-float arithmetic so that each pair's force carries ~1e-10 relative
// error (an FP64 pipe is 1/64 of the FP32 one on this part).
//   * Coordinates: each slot holds hi = (x, y, z) rounded to a multiple of
//     2^-8 A and lo = the FP32 remainder.  dh = hj - hi is exact, each dh^2
//     is exact (|dh| < 16 A) and so is their sum S; r^2 = S + c with
//     c = dl (2 dh + dl), renormalised to (Rh, Rl).
//   * 1/r^2 and 1/r: MUFU approximations corrected by one residual each.
//   * LJ below the switch radius and the Coulomb term in double-float; the
//     switch polynomial S(u) and dS/du in double-float; LJ inside the switch
//     band (under 1e-2 kcal/mol/A there) in plain FP32.
//   * F_i -= G d accumulated per lane with TwoSum over chunks of 32 entries;
//     each chunk's (hi, lo) sum is folded into int64 fixed point, so the
//     result is independent of how the columns are split over warps.
// The list columns are ordered by build distance (inside the switch radius,
// the switch band, then the shell beyond the cutoff), so a warp's 32 lanes
// usually take the same branch and skip whole regions together.
// Warp w works on group w / split and on the part w % split of the group's
// list columns: entries [part * per, (part + 1) * per), per a multiple of the
// 32-entry chunk.  The split raises the number of warps in flight (a
// 50k-atom system has only 1,563 groups).
// BATCH: systems of a batch have their own type tables ([system][type][type],
// read through L1); a single system keeps its table in shared memory.
// ENERGY false: the item adds its forces only (no energy partial, no
// per-system energy); the force bits are the same.
template <bool PERIODIC, bool COULOMB, bool BATCH, bool ENERGY = true>
__device__ __forceinline__ void
pair_item_mixed(int wid, int lane, int n, int cap, int split, const float4 *__restrict__ coord,
                const int *__restrict__ perm, const int *__restrict__ list, const int *__restrict__ count,
                const int *__restrict__ gmax, int ntypes, const float4 *__restrict__ tab, const float4 *s_tab,
                const PairConst &k, long long *__restrict__ force, double *__restrict__ epart, DevStatus *st,
                const int *__restrict__ group_sys, long long *e_sys) {
    const unsigned full = 0xffffffffu;
    const int group = wid / split, part = wid - group * split;
    const int s = group * 32 + lane;
    const int atom = perm[s];  // -1 on a padding slot
    const bool valid = atom >= 0;
    float4 mh = make_float4(0.f, 0.f, 0.f, 0.f), ml = mh;
    int cnt = 0;
    if (valid) { gm_ld_coord(coord + 2 * s, mh, ml); cnt = count[s]; }
    const float4 *trow = (BATCH ? tab + (size_t)group_sys[group] * ntypes * ntypes : s_tab) +
                         (valid ? gm_slot_type(ml.w) : 0) * ntypes;
    const gm_df qi = gm_df_make(mh.w, ml.w);
    const int gm = gmax[group];
    const int per = ((gm + split - 1) / split + kChunk - 1) / kChunk * kChunk;
    const int e_begin = part * per, e_end = min(gm, e_begin + per);
    const int *L = list + (size_t)group * 32 * cap + lane;
    const int self = valid ? s : 0;
    long long ax = 0, ay = 0, az = 0;
    double eacc = 0.0;
    unsigned int bad = 0;
    for (int e0 = e_begin; e0 < e_end; e0 += kChunk) {
        gm_df acc[3] = {gm_df_make(0.f, 0.f), gm_df_make(0.f, 0.f), gm_df_make(0.f, 0.f)};
        float ev = 0.f;
        const int e1 = min(e0 + kChunk, e_end);
        for (int e = e0; e < e1; e += kBatch) {
            // lanes past their own count (or the chunk) gather their own
            // atom: r2 == 0 drops it
            int jj[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++)
                jj[u] = (e + u < cnt && e + u < e1) ? __ldg(L + (size_t)(e + u) * 32) : self;
            float4 jhv[kBatch], jlv[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) gm_ld_coord(coord + 2 * jj[u], jhv[u], jlv[u]);
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
            const float4 jh = jhv[u], jl = jlv[u];
            float d_h[3] = {jh.x - mh.x, jh.y - mh.y, jh.z - mh.z};
            float d_l[3] = {jl.x - ml.x, jl.y - ml.y, jl.z - ml.z};
            if (PERIODIC) {
#pragma unroll
                for (int d = 0; d < 3; d++) image_df(d_h[d], d_l[d], k.box[d], k.box_lo[d], k.inv_box[d]);
            }
            const float S = fmaf(d_h[2], d_h[2], fmaf(d_h[1], d_h[1], d_h[0] * d_h[0]));  // exact
            const float c = fmaf(d_l[2], fmaf(2.f, d_h[2], d_l[2]),
                                 fmaf(d_l[1], fmaf(2.f, d_h[1], d_l[1]), d_l[0] * fmaf(2.f, d_h[0], d_l[0])));
            const gm_df R = gm_fast_sum(S, c);  // r^2
            const bool in = R.h <= k.rc2 && R.h > 0.f;
            if (!__any_sync(full, in)) continue;  // warp-uniform: the shell beyond the cutoff
            const float Rh = in ? R.h : 1.f, Rl = in ? R.l : 0.f;
            // 1/r^2 = y (1 + rho - Rl y), rho = 1 - Rh y
            const float y = rcp_approx(Rh);
            const float rho = fmaf(-Rh, y, 1.f);
            const gm_df inv = gm_df_make(y, y * fmaf(-Rl, y, rho));
            // 1/r = z (1 - tau / 2), tau = (Rh + Rl) z^2 - 1 from exact products
            const float z = rsqrt_approx(Rh);
            const float a = __fmul_rn(Rh, z), ea = fmaf(Rh, z, -a);
            const float tau = fmaf(Rl, y, fmaf(ea, z, fmaf(a, z, -1.f)));
            const gm_df rinv = gm_df_make(z, -0.5f * z * tau);
            const float4 p = BATCH ? __ldg(trow + gm_slot_type(jl.w)) : trow[gm_slot_type(jl.w)];
            gm_df Vc = gm_df_make(0.f, 0.f), Gc = Vc;
            if (COULOMB) {
                Vc = gm_dmul(gm_dmul(qi, gm_df_make(jh.w, jl.w)), rinv);  // k q_i q_j / r
                Gc = gm_dmul(Vc, inv);                                     // (k q_i q_j / r^2) / r
            }
            gm_df G = Gc;  // F_r / r
            float v = 0.f;
            const bool near = in && R.h <= k.rsw2;
            const bool band = in && !near;
            if (__any_sync(full, near) && near) {
                const gm_df x = gm_dmul(gm_df_make(p.x, p.y), inv);  // (sigma / r)^2
                const gm_df x3 = gm_dmul(gm_dsqr(x), x);
                gm_df w2 = gm_two_sum(x3.h + x3.h, -1.f);  // 2 x3 - 1
                w2.l += x3.l + x3.l;
                const gm_df g = gm_dmul(gm_dmul(gm_dmul(gm_df_make(p.z, p.w), x3), w2), inv);
                G = gm_dadd(g, Gc);
                v = p.z * (1.f / 6.f) * x3.h * (x3.h - 1.f) + (Vc.h + Vc.l);
            }
            if (__any_sync(full, band) && band) {
                // LJ in FP32 (tiny here), then V S and F_r S - V dS/dr
                // (products rounded where the compiler could otherwise fuse them
                // into the sums that follow)
                const float xs = p.x * y, x3 = __fmul_rn(__fmul_rn(xs, xs), xs);
                const float vlj = p.z * (1.f / 6.f) * x3 * (x3 - 1.f);
                const float glj = p.z * x3 * fmaf(2.f, x3, -1.f) * y;
                const gm_df V = gm_dadd(Vc, gm_df_make(vlj, 0.f));
                const gm_df G0 = gm_dadd(Gc, gm_df_make(glj, 0.f));
                const gm_df r = gm_dmul(gm_df_make(Rh, Rl), rinv);
                gm_df u0 = gm_two_sum(r.h, -k.rsw);
                u0.l += r.l - k.rsw_lo;
                const gm_df uu = gm_dmul(u0, gm_df_make(k.inv_w, k.inv_w_lo));
                const gm_df u2 = gm_dsqr(uu), u3 = gm_dmul(u2, uu);
                // S = 1 + u^3 (-10 + u (15 - 6 u))
                const float p6 = __fmul_rn(6.f, uu.h), e6 = fmaf(6.f, uu.h, -p6);
                gm_df t = gm_two_sum(15.f, -p6);
                t.l -= fmaf(6.f, uu.l, e6);
                t = gm_dmul(uu, t);
                gm_df t3 = gm_two_sum(-10.f, t.h);
                t3.l += t.l;
                t = gm_dmul(u3, t3);
                gm_df sw = gm_two_sum(1.f, t.h);
                sw.l += t.l;
                // dS/dr = -30 u^2 (1 - u)^2 / w
                gm_df om = gm_two_sum(1.f, -uu.h);
                om.l -= uu.l;
                const gm_df ds = gm_dmul(gm_dmul(u2, gm_dsqr(om)), gm_df_make(k.mds, k.mds_lo));
                G = gm_dadd(gm_dmul(G0, sw), gm_dneg(gm_dmul(gm_dmul(V, ds), rinv)));
                v = (V.h + V.l) * (sw.h + sw.l);
            }
            if (in) {
                // F_i -= G d, each product with its exact error
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float pr = __fmul_rn(G.h, d_h[d]);
                    const float er = fmaf(G.h, d_l[d], fmaf(G.l, d_h[d], fmaf(G.h, d_h[d], -pr)));
                    gm_df sum = gm_two_sum(acc[d].h, -pr);
                    sum.l += acc[d].l - er;
                    acc[d] = sum;
                }
                if (ENERGY) ev += v;
            }
            }
        }
        ax += gm_to_fix_checked(acc[0].h, bad) + gm_f2fix(acc[0].l);
        ay += gm_to_fix_checked(acc[1].h, bad) + gm_f2fix(acc[1].l);
        az += gm_to_fix_checked(acc[2].h, bad) + gm_f2fix(acc[2].l);
        if (ENERGY) eacc += (double)ev;
    }
    if (valid && e_begin < e_end) {
        gm_atomic_fix_add(force + atom, ax);
        gm_atomic_fix_add(force + n + atom, ay);
        gm_atomic_fix_add(force + 2 * n + atom, az);
    }
    if (ENERGY) {
        for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(full, eacc, o);
        if (lane == 0) epart[wid] = 0.5 * eacc;
        if (e_sys && lane == 0)
            gm_atomic_fix_add(e_sys + group_sys[group], __double2ll_rn(0.5 * eacc * GM_EFIX_SCALE));
    }
    bad = __reduce_or_sync(full, bad);
    if (bad && lane == 0) atomicOr(&st->error, bad);
}

// ----------------------------------------------------------------- bonded
//
// Bond, angle and dihedral terms and the scaled 1-4 pairs run in FP64 in both
// precisions: they are ~3N terms against ~400N pair evaluations, and their
// forces (k = 300 bonds balancing the LJ repulsion of a dense lattice) are
// large enough that FP32 rounding alone would exceed 1e-5 of a small net
// force.

struct V3 { double x, y, z; };

// pos[ia] - pos[ib] in FP64; with MI at the nearest periodic image (the
// reference's min_image on each component)
template <bool MI>
__device__ __forceinline__ V3 pdiff(const ForceArgs &a, int ia, int ib) {
    const int n = a.n;
    V3 d = {a.pos[ia] - a.pos[ib], a.pos[n + ia] - a.pos[n + ib], a.pos[2 * n + ia] - a.pos[2 * n + ib]};
    if constexpr (MI) {
        d.x = gm_min_image(d.x, a.box64[0]);
        d.y = gm_min_image(d.y, a.box64[1]);
        d.z = gm_min_image(d.z, a.box64[2]);
    }
    return d;
}
// The FP64 term arithmetic below fixes every fused multiply-add itself
// (fma where a product feeds a sum, __dmul_rn where a product must stay
// rounded): the compiler's own contraction choices may differ between the
// kernels that inline these functions, and both step forms must round alike.
__device__ __forceinline__ double pmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {fma(a.y, b.z, -pmul(a.z, b.y)), fma(a.z, b.x, -pmul(a.x, b.z)), fma(a.x, b.y, -pmul(a.y, b.x))};
}
__device__ __forceinline__ double dot(V3 a, V3 b) { return fma(a.z, b.z, fma(a.y, b.y, pmul(a.x, b.x))); }

__device__ __forceinline__ void add_force(long long *f, int n, int a, double x, double y, double z, unsigned &bad) {
    gm_atomic_fix_add(f + a, gm_to_fix_checked(x, bad));
    gm_atomic_fix_add(f + n + a, gm_to_fix_checked(y, bad));
    gm_atomic_fix_add(f + 2 * n + a, gm_to_fix_checked(z, bad));
}

// Term t of the bonded list (bonds, then angles, then dihedrals; t past the
// end is no term): adds its forces and returns its energy; `first` is an atom
// of the term (its system owns the energy).
template <bool MI>
__device__ __forceinline__ double bonded_term(const ForceArgs &a, int t, unsigned &bad, int &first) {
    const int n = a.n;
    double e = 0.0;
    if (t < a.n_bonds) {
        // force/bonded.rs:5-40, V = k (r - r0)^2
        const int i = a.bond_i[t], j = a.bond_j[t];
        first = i;
        const V3 d = pdiff<MI>(a, j, i);
        const double k = a.bond_k[t], r0 = a.bond_r0[t];
        const double r2 = dot(d, d);
        if (r2 > 0.0) {
            const double ir = rsqrt(r2);
            const double dr = fma(r2, ir, -r0);
            e = pmul(pmul(k, dr), dr);
            const double g = pmul(pmul(pmul(2.0, k), dr), ir);
            const double gx = pmul(g, d.x), gy = pmul(g, d.y), gz = pmul(g, d.z);
            add_force(a.force, n, i, gx, gy, gz, bad);
            add_force(a.force, n, j, -gx, -gy, -gz, bad);
        }
    } else if (t < a.n_bonds + a.n_angles) {
        // force/bonded.rs:44-102, V = k (theta - theta0)^2
        const int q = t - a.n_bonds;
        const int i = a.angle_i[q], j = a.angle_j[q], kk = a.angle_k[q];
        first = i;
        const V3 b1 = pdiff<MI>(a, i, j), b2 = pdiff<MI>(a, kk, j);
        const double q1 = dot(b1, b1), q2 = dot(b2, b2);
        if (q1 != 0.0 && q2 != 0.0) {
            const double i1 = rsqrt(q1), i2 = rsqrt(q2);
            double c = pmul(pmul(dot(b1, b2), i1), i2);
            c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
            double sn = sqrt(fma(-c, c, 1.0));
            sn = sn > 1e-8 ? sn : 1e-8;
            const double dth = acos(c) - a.angle_th0[q];
            const double k = a.angle_kth[q];
            e = pmul(pmul(k, dth), dth);
            const double aa = pmul(pmul(2.0, k), dth) / sn;
            const double ir12 = pmul(i1, i2), ir11 = pmul(i1, i1), ir22 = pmul(i2, i2);
            // aa (b2 / (|b1| |b2|) - c b1 / |b1|^2), and the same for k
            const V3 fi = {pmul(aa, fma(b2.x, ir12, -pmul(pmul(c, b1.x), ir11))),
                           pmul(aa, fma(b2.y, ir12, -pmul(pmul(c, b1.y), ir11))),
                           pmul(aa, fma(b2.z, ir12, -pmul(pmul(c, b1.z), ir11)))};
            const V3 fk = {pmul(aa, fma(b1.x, ir12, -pmul(pmul(c, b2.x), ir22))),
                           pmul(aa, fma(b1.y, ir12, -pmul(pmul(c, b2.y), ir22))),
                           pmul(aa, fma(b1.z, ir12, -pmul(pmul(c, b2.z), ir22)))};
            add_force(a.force, n, i, fi.x, fi.y, fi.z, bad);
            add_force(a.force, n, kk, fk.x, fk.y, fk.z, bad);
            add_force(a.force, n, j, -(fi.x + fk.x), -(fi.y + fk.y), -(fi.z + fk.z), bad);
        }
    } else if (t < a.n_bonds + a.n_angles + a.n_diheds) {
        // force/bonded.rs:112-164, V = k [1 + cos(n phi - delta)]
        const int q = t - a.n_bonds - a.n_angles;
        const int i = a.dihed_i[q], j = a.dihed_j[q], k = a.dihed_k[q], l = a.dihed_l[q];
        first = i;
        const V3 b1 = pdiff<MI>(a, j, i), b2 = pdiff<MI>(a, k, j), b3 = pdiff<MI>(a, l, k);
        const V3 m = cross(b1, b2), nv = cross(b2, b3);
        const double m2 = dot(m, m), n2 = dot(nv, nv), b22 = dot(b2, b2);
        if (m2 != 0.0 && n2 != 0.0 && b22 != 0.0) {
            const double ib2 = rsqrt(b22), b2l = pmul(b22, ib2);
            // phi = atan2(y, x) as in the reference; cos(n phi - delta) and
            // sin(n phi - delta) are taken without the transcendentals:
            // (cos phi, sin phi) = (x, y) / |(x, y)|, raised to the n-th
            // power as a complex number, then rotated by delta (the FP64
            // pipe of this part is 1/64 of its FP32 one)
            const double x = dot(m, nv);
            const double y = pmul(dot(cross(m, nv), b2), ib2);
            const double ir = rsqrt(fma(x, x, pmul(y, y)));
            const double c1 = pmul(x, ir), s1 = pmul(y, ir);
            const unsigned mult = a.dihed_n[q];
            double cn = 1.0, sn = 0.0;
            for (unsigned it = 0; it < mult; it++) {
                const double c2 = fma(cn, c1, -pmul(sn, s1));
                sn = fma(sn, c1, pmul(cn, s1));
                cn = c2;
            }
            const double2 cs = a.dihed_cs[q];  // (cos delta, sin delta)
            const double kphi = a.dihed_kphi[q];
            e = pmul(kphi, 1.0 + fma(cn, cs.x, pmul(sn, cs.y)));
            const double dv = pmul(pmul(kphi, (double)mult), fma(sn, cs.x, -pmul(cn, cs.y)));  // -dV/dphi
            const double imn = pmul(dv, b2l) / pmul(m2, n2);
            const double si = pmul(-imn, n2), sl = pmul(imn, m2);
            const V3 fi = {pmul(m.x, si), pmul(m.y, si), pmul(m.z, si)};
            const V3 fl = {pmul(nv.x, sl), pmul(nv.y, sl), pmul(nv.z, sl)};
            const double ib = pmul(ib2, ib2);
            const double p = pmul(dot(b1, b2), ib), qq = pmul(dot(b3, b2), ib);
            const double p1 = -(p + 1.0), q1 = qq + 1.0;
            const V3 fj = {fma(qq, fl.x, pmul(p1, fi.x)), fma(qq, fl.y, pmul(p1, fi.y)), fma(qq, fl.z, pmul(p1, fi.z))};
            const V3 fk = {fma(p, fi.x, -pmul(q1, fl.x)), fma(p, fi.y, -pmul(q1, fl.y)), fma(p, fi.z, -pmul(q1, fl.z))};
            add_force(a.force, n, i, fi.x, fi.y, fi.z, bad);
            add_force(a.force, n, j, fj.x, fj.y, fj.z, bad);
            add_force(a.force, n, k, fk.x, fk.y, fk.z, bad);
            add_force(a.force, n, l, fl.x, fl.y, fl.z, bad);
        }
    }
    return e;
}

// Scaled 1-4 pair t (beyond the reference): unswitched, no cutoff; LJ scaled
// by scale14_lj, Coulomb by scale14_coul.
template <bool MI>
__device__ __forceinline__ double pair14_term(const ForceArgs &a, int t, unsigned &bad, int &first) {
    const int n = a.n;
    double e = 0.0;
    if (t < a.n14) {
        const int i = a.p14_i[t], j = a.p14_j[t];
        first = i;
        const V3 d = pdiff<MI>(a, j, i);
        const double r2 = dot(d, d);
        if (r2 > 0.0) {
            // (sigma_ij, 4 eps_ij s_lj, 24 eps_ij s_lj, k_C q_i q_j s_coul)
            const double4 p = a.p14par[t];
            const double rinv = rsqrt(r2);
            const double sr = pmul(p.x, rinv), s2 = pmul(sr, sr), s4 = pmul(s2, s2), s6 = pmul(s2, s4);
            const double s12 = pmul(s6, s6);
            const double vc = pmul(p.w, rinv);
            e = fma(p.y, s12 - s6, vc);
            const double g = pmul(pmul(fma(p.z, fma(2.0, s12, -s6), vc), rinv), rinv);
            const double gx = pmul(g, d.x), gy = pmul(g, d.y), gz = pmul(g, d.z);
            add_force(a.force, n, i, -gx, -gy, -gz, bad);
            add_force(a.force, n, j, gx, gy, gz, bad);
        }
    }
    return e;
}

}  // namespace
