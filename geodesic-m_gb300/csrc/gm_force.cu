// gm_force.cu — force and energy kernels.
//
// Nonbonded (force/nonbonded.rs:20-82 physics): one lane per cell-sorted atom
// i walks its own column of the symmetric neighbour list, gathers each j's
// float4 pair (hi, lo), one 32-byte sector, with one 256-bit load through the
// read-only path (four entries' gathers in flight before their arithmetic) and
// accumulates the force
// on i only, so no atomics are needed and every atom's sum has a fixed order.
// In mixed precision the pair arithmetic is FP32; per-lane partial sums over
// chunks of 32 entries are folded into int64 fixed point (2^-40 kcal/mol/A),
// and the energy into FP64.  Each pair is evaluated by both of its atoms
// (the list is symmetric), the energy total is halved.
// Bonded terms (force/bonded.rs) use one thread per term and int64 atomics;
// integer addition is associative, so the result is run-to-run identical.
#include "gm_internal.cuh"

namespace {

constexpr int kPairWarps = 4;
constexpr int kChunk = 32;
constexpr int kBatch = 4;  // list entries gathered together in the FP32 pair kernel
constexpr float kCoulomb = 332.0522173f;
constexpr double kCoulomb64 = 332.0522173;

// Warp w works on group w / split and on the part w % split of the group's
// list columns: entries [part * per, (part + 1) * per), per a multiple of the
// 32-entry summation chunk.  The split raises the number of warps in flight
// (a 50k-atom system has only 1,563 groups), and integer partial sums keep the
// result independent of the order in which the parts land.
// BATCH: systems of a batch have their own type tables ([system][type][type],
// read through L1); a single system keeps its table in shared memory.
template <bool PERIODIC, bool COULOMB, bool BATCH, int W>
__global__ void __launch_bounds__(W * 32)
pair_kernel_f32(int n, int n_slots, int cap, int split, const float4 *__restrict__ coord,
                const int *__restrict__ perm, const int *__restrict__ list, const int *__restrict__ count,
                const int *__restrict__ gmax, int ntypes, const float2 *__restrict__ tab, float rc2, float rsw,
                float inv_wsw, float bx, float by, float bz, float ibx, float iby, float ibz,
                long long *__restrict__ force, double *__restrict__ epart, DevStatus *st,
                const int *__restrict__ group_sys, long long *e_sys) {
    extern __shared__ float2 s_tab[];
    if (!BATCH) {
        for (int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x) s_tab[t] = tab[t];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    // work items (group, part of its columns); a grid smaller than the work
    // makes the kernel persistent, every item is computed the same either way
    const int n_work = (n_slots / 32) * split;
    for (int wid = blockIdx.x * W + (threadIdx.x >> 5); wid < n_work; wid += gridDim.x * W) {
    const int group = wid / split, part = wid - group * split;
    const int s = group * 32 + lane;
    const int atom = perm[s];  // -1 on a padding slot
    const bool valid = atom >= 0;
    float4 mh = make_float4(0.f, 0.f, 0.f, 0.f), ml = mh;
    int cnt = 0;
    if (valid) { mh = coord[2 * s]; ml = coord[2 * s + 1]; cnt = count[s]; }
    const float2 *trow = (BATCH ? tab + (size_t)group_sys[group] * ntypes * ntypes : s_tab) +
                         (valid ? __float_as_int(mh.w) : 0) * ntypes;
    const float qi = ml.w * kCoulomb;
    const int gm = gmax[group];
    const int per = ((gm + split - 1) / split + kChunk - 1) / kChunk * kChunk;
    const int e_begin = part * per, e_end = min(gm, e_begin + per);
    const int *L = list + (size_t)group * 32 * cap + lane;
    const int self = valid ? s : 0;
    long long ax = 0, ay = 0, az = 0;
    double eacc = 0.0;
    unsigned int bad = 0;
    for (int e0 = e_begin; e0 < e_end; e0 += kChunk) {
        float fx = 0.f, fy = 0.f, fz = 0.f, ev = 0.f;
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
            for (int u = 0; u < kBatch; u++) {
                gm_ld_coord(coord + 2 * jj[u], jhv[u], jlv[u]);
            }
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
            const float4 jh = jhv[u], jl = jlv[u];
            float dx = (jh.x - mh.x) + (jl.x - ml.x);
            float dy = (jh.y - mh.y) + (jl.y - ml.y);
            float dz = (jh.z - mh.z) + (jl.z - ml.z);
            if (PERIODIC) {
                dx -= bx * rintf(dx * ibx);
                dy -= by * rintf(dy * iby);
                dz -= bz * rintf(dz * ibz);
            }
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 <= rc2 && r2 > 0.f) {
                const float2 p = BATCH ? __ldg(trow + __float_as_int(jh.w)) : trow[__float_as_int(jh.w)];
                // rsqrtf plus one Newton step: the pair sums cancel to
                // small net forces, so the last ulps of 1/r matter
                float rinv = rsqrtf(r2);
                rinv = fmaf(0.5f * rinv, fmaf(-r2 * rinv, rinv, 1.0f), rinv);
                const float rinv2 = rinv * rinv;
                const float s2 = p.x * rinv2;
                const float s6 = s2 * s2 * s2;
                const float s12 = s6 * s6;
                float v = 4.f * p.y * (s12 - s6);
                float fr = 24.f * p.y * (2.f * s12 - s6) * rinv2;  // F_r / r
                if (COULOMB) {
                    const float vc = qi * jl.w * rinv;
                    v += vc;
                    fr += vc * rinv2;
                }
                const float r = r2 * rinv;
                if (r > rsw) {
                    const float u_ = (r - rsw) * inv_wsw;
                    const float u2 = u_ * u_;
                    const float sw = 1.f + u2 * u_ * (-10.f + u_ * (15.f - 6.f * u_));
                    const float dsw = -30.f * u2 * (1.f - u_) * (1.f - u_) * inv_wsw;
                    fr = fr * sw - v * dsw * rinv;
                    v *= sw;
                }
                fx -= fr * dx;
                fy -= fr * dy;
                fz -= fr * dz;
                ev += v;
            }
            }
        }
        ax += gm_to_fix_checked(fx, bad);
        ay += gm_to_fix_checked(fy, bad);
        az += gm_to_fix_checked(fz, bad);
        eacc += (double)ev;
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

template <bool PERIODIC, bool COULOMB, bool BATCH>
__global__ void __launch_bounds__(kPairWarps * 32)
pair_kernel_f64(int n, int n_slots, int cap, const double4 *__restrict__ p64, const int *__restrict__ type_s,
                const int *__restrict__ perm, const int *__restrict__ list, const int *__restrict__ count,
                const int *__restrict__ gmax, int ntypes, const double2 *__restrict__ tab, double rc2, double rsw,
                double rc, double bx, double by, double bz, long long *__restrict__ force,
                double *__restrict__ epart, DevStatus *st, const int *__restrict__ group_sys, long long *e_sys) {
    extern __shared__ double2 s_tab64[];
    if (!BATCH) {
        for (int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x) s_tab64[t] = tab[t];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int group = blockIdx.x * kPairWarps + (threadIdx.x >> 5);
    if (group * 32 >= n_slots) return;
    const int s = group * 32 + lane;
    const int atom = perm[s];  // -1 on a padding slot
    const bool valid = atom >= 0;
    double4 mi = make_double4(0, 0, 0, 0);
    int cnt = 0, ti = 0;
    if (valid) { mi = p64[s]; cnt = count[s]; ti = type_s[s]; }
    const double2 *trow = (BATCH ? tab + (size_t)group_sys[group] * ntypes * ntypes : s_tab64) + ti * ntypes;
    const double qi = mi.w * kCoulomb64;
    const int gm = gmax[group];
    const int *L = list + (size_t)group * 32 * cap + lane;
    double fx = 0, fy = 0, fz = 0, eacc = 0;
    const double wsw = rc - rsw;
    for (int e = 0; e < gm; e++) {
        if (e >= cnt) continue;
        const int j = __ldg(L + (size_t)e * 32);
        const double4 pj = p64[j];
        double dx = pj.x - mi.x, dy = pj.y - mi.y, dz = pj.z - mi.z;
        if (PERIODIC) {
            dx -= bx * round(dx / bx);
            dy -= by * round(dy / by);
            dz -= bz * round(dz / bz);
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
    unsigned int bad = 0;
    if (valid) {
        gm_atomic_fix_add(force + atom, gm_to_fix_checked(fx, bad));
        gm_atomic_fix_add(force + n + atom, gm_to_fix_checked(fy, bad));
        gm_atomic_fix_add(force + 2 * n + atom, gm_to_fix_checked(fz, bad));
    }
    for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
    if (lane == 0) epart[group] = 0.5 * eacc;
    if (e_sys && lane == 0) gm_atomic_fix_add(e_sys + group_sys[group], __double2ll_rn(0.5 * eacc * GM_EFIX_SCALE));
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && lane == 0) atomicOr(&st->error, bad);
}

// ----------------------------------------------------------------- bonded

template <typename T>
struct V3 { T x, y, z; };

template <typename T>
__device__ __forceinline__ V3<T> diff(const double *pos, int n, int a, int b) {
    // pos[a] - pos[b], differenced in FP64 before any narrowing
    return {(T)(pos[a] - pos[b]), (T)(pos[n + a] - pos[n + b]), (T)(pos[2 * n + a] - pos[2 * n + b])};
}
// FP32 difference of two atoms of one system from their (hi, lo) slot copies
// (relative to the same grid origin): the rounded FP64 difference within an ulp
__device__ __forceinline__ V3<float> fdiff(const ForceArgs &a, int ia, int ib) {
    float4 ha, la, hb, lb;
    gm_ld_coord(a.coord + 2 * a.slot_of[ia], ha, la);
    gm_ld_coord(a.coord + 2 * a.slot_of[ib], hb, lb);
    return {(ha.x - hb.x) + (la.x - lb.x), (ha.y - hb.y) + (la.y - lb.y), (ha.z - hb.z) + (la.z - lb.z)};
}
// pos[ia] - pos[ib] in FP64; with MI at the nearest periodic image (the
// reference's min_image on each component)
template <bool MI>
__device__ __forceinline__ V3<double> pdiff(const ForceArgs &a, int ia, int ib) {
    const int n = a.n;
    V3<double> d = {a.pos[ia] - a.pos[ib], a.pos[n + ia] - a.pos[n + ib], a.pos[2 * n + ia] - a.pos[2 * n + ib]};
    if constexpr (MI) {
        d.x = gm_min_image(d.x, a.box64[0]);
        d.y = gm_min_image(d.y, a.box64[1]);
        d.z = gm_min_image(d.z, a.box64[2]);
    }
    return d;
}
// The T-typed difference a bonded term works in: fdiff (mixed) or the FP64
// difference, or with MI the nearest-image FP64 difference narrowed to T (the
// slot copies of two atoms on opposite faces of the box are not close, so
// fdiff would lose the difference's low bits there)
template <typename T, bool MI>
__device__ __forceinline__ V3<T> term_diff(const ForceArgs &a, int ia, int ib) {
    if constexpr (MI) {
        const V3<double> d = pdiff<true>(a, ia, ib);
        return {(T)d.x, (T)d.y, (T)d.z};
    } else if constexpr (sizeof(T) == sizeof(float)) {
        return fdiff(a, ia, ib);
    } else {
        return diff<T>(a.pos, a.n, ia, ib);
    }
}
template <typename T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

template <typename T>
__device__ __forceinline__ void add_force(long long *f, int n, int a, T x, T y, T z, unsigned &bad) {
    gm_atomic_fix_add(f + a, gm_to_fix_checked(x, bad));
    gm_atomic_fix_add(f + n + a, gm_to_fix_checked(y, bad));
    gm_atomic_fix_add(f + 2 * n + a, gm_to_fix_checked(z, bad));
}

__device__ __forceinline__ float gm_acos(float x) { return acosf(x); }
__device__ __forceinline__ double gm_acos(double x) { return acos(x); }
__device__ __forceinline__ float gm_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double gm_atan2(double y, double x) { return atan2(y, x); }

template <typename T, bool MI>
__device__ __forceinline__ void bonded_block(const ForceArgs &a, int blk) {
    constexpr bool kMixed = sizeof(T) == sizeof(float);
    const int t = blk * blockDim.x + threadIdx.x;
    const int n = a.n;
    double e = 0.0;
    unsigned bad = 0;
    int first = -1;  // an atom of the term: its system owns the energy
    if (t < a.n_bonds) {
        // force/bonded.rs:5-40, V = k (r - r0)^2.  FP64 in both paths: a bond
        // stretched across a wrapped periodic boundary carries forces ~1e5
        // kcal/mol/A whose FP32 rounding would swamp small net forces (the
        // reference's GPU backend also keeps bonded terms in FP64).
        const int i = a.bond_i[t], j = a.bond_j[t];
        first = i;
        const V3<double> bd = pdiff<MI>(a, j, i);
        const double dx = bd.x, dy = bd.y, dz = bd.z;
        const double k = a.bond_k[t], r0 = a.bond_r0[t];
        const double r2 = dx * dx + dy * dy + dz * dz;
        bool done = false;
        if (kMixed && r2 > 0.0) {
            // mixed path: r - r0 = (r^2 - r0^2) / (r + r0), the cancelling
            // difference r^2 - r0^2 in FP64 and the rest in FP32 (the FP64
            // pipe is the bottleneck of this kernel); a bond stretched by
            // half an angstrom or more takes the FP64 branch below
            const float r = sqrtf((float)r2);
            const float dr = (float)fma(-r0, r0, r2) / (r + (float)r0);
            if (fabsf(dr) < 0.5f && r > 1e-3f) {
                const float kf = (float)k;
                e = (double)(kf * dr * dr);
                const float g = 2.f * kf * dr / r;
                const float fx = g * (float)dx, fy = g * (float)dy, fz = g * (float)dz;
                add_force<float>(a.force, n, i, fx, fy, fz, bad);
                add_force<float>(a.force, n, j, -fx, -fy, -fz, bad);
                done = true;
            }
        }
        if (!done && r2 > 0.0) {
            const double r = sqrt(r2);
            const double dr = r - r0;
            e = k * dr * dr;
            const double g = 2.0 * k * dr / r;
            add_force<double>(a.force, n, i, g * dx, g * dy, g * dz, bad);
            add_force<double>(a.force, n, j, -g * dx, -g * dy, -g * dz, bad);
        }
    } else if (t < a.n_bonds + a.n_angles) {
        // force/bonded.rs:44-102, V = k (theta - theta0)^2
        const int q = t - a.n_bonds;
        const int i = a.angle_i[q], j = a.angle_j[q], kk = a.angle_k[q];
        first = i;
        const V3<T> b1 = term_diff<T, MI>(a, i, j), b2 = term_diff<T, MI>(a, kk, j);
        const T r1 = sqrt(dot(b1, b1)), r2 = sqrt(dot(b2, b2));
        if (kMixed && r1 != (T)0 && r2 != (T)0) {
            // mixed path: theta - theta0 = atan2(sin(theta - theta0),
            // cos(theta - theta0)), both from FP64 products
            //   |d1||d2| sin(theta - theta0) = |d1 x d2| cos theta0 - (d1 . d2) sin theta0
            //   |d1||d2| cos(theta - theta0) = (d1 . d2) cos theta0 + |d1 x d2| sin theta0
            // with |d1 x d2| from an FP32 square root and one Newton step in
            // FP64; no FP64 acos, square root or division
            const V3<double> d1 = pdiff<MI>(a, i, j), d2 = pdiff<MI>(a, kk, j);
            const double dd = dot(d1, d2);
            const V3<double> cr = cross(d1, d2);
            const double q2 = dot(cr, cr);
            const float s32 = sqrtf((float)q2);
            double sx = (double)s32;
            if (s32 > 0.f) sx = fma(fma(-sx, sx, q2), (double)(0.5f / s32), sx);
            const double2 cs0 = a.angle_cs[q];
            const double y = sx * cs0.x - dd * cs0.y, x = dd * cs0.x + sx * cs0.y;
            const float dth = atan2f((float)y, (float)x);
            const float k = (float)a.angle_kth[q];
            e = (double)(k * dth * dth);
            const float ir12 = 1.f / (float)(r1 * r2), ir11 = 1.f / (float)(r1 * r1), ir22 = 1.f / (float)(r2 * r2);
            const float c = (float)dd * ir12;
            float sn = (float)sx * ir12;
            sn = sn > 1e-8f ? sn : 1e-8f;
            const float aa = 2.f * k * dth / sn;
            const V3<float> fi = {aa * ((float)b2.x * ir12 - c * (float)b1.x * ir11), aa * ((float)b2.y * ir12 - c * (float)b1.y * ir11),
                                  aa * ((float)b2.z * ir12 - c * (float)b1.z * ir11)};
            const V3<float> fk = {aa * ((float)b1.x * ir12 - c * (float)b2.x * ir22), aa * ((float)b1.y * ir12 - c * (float)b2.y * ir22),
                                  aa * ((float)b1.z * ir12 - c * (float)b2.z * ir22)};
            add_force<float>(a.force, n, i, fi.x, fi.y, fi.z, bad);
            add_force<float>(a.force, n, kk, fk.x, fk.y, fk.z, bad);
            add_force<float>(a.force, n, j, -(fi.x + fk.x), -(fi.y + fk.y), -(fi.z + fk.z), bad);
        } else if (r1 != (T)0 && r2 != (T)0) {
            // theta - theta0 in FP64 in both paths: an FP32 acos is off by
            // ~1e-7 rad, i.e. ~1e-5 kcal/mol/A at k = 50, which a structure
            // near equilibrium cannot absorb
            const V3<double> d1 = pdiff<MI>(a, i, j), d2 = pdiff<MI>(a, kk, j);
            double c64 = dot(d1, d2) / sqrt(dot(d1, d1) * dot(d2, d2));
            c64 = c64 < -1.0 ? -1.0 : (c64 > 1.0 ? 1.0 : c64);
            const T c = (T)c64;
            T sn = (T)sqrt(1.0 - c64 * c64);
            sn = sn > (T)1e-8 ? sn : (T)1e-8;
            const double dth = acos(c64) - a.angle_th0[q];
            const T k = (T)a.angle_kth[q];
            e = a.angle_kth[q] * dth * dth;
            const T th = (T)dth, th0 = (T)0;
            const T aa = (T)2 * k * (th - th0) / sn;
            const T ir12 = (T)1 / (r1 * r2), ir11 = (T)1 / (r1 * r1), ir22 = (T)1 / (r2 * r2);
            const V3<T> fi = {aa * (b2.x * ir12 - c * b1.x * ir11), aa * (b2.y * ir12 - c * b1.y * ir11),
                              aa * (b2.z * ir12 - c * b1.z * ir11)};
            const V3<T> fk = {aa * (b1.x * ir12 - c * b2.x * ir22), aa * (b1.y * ir12 - c * b2.y * ir22),
                              aa * (b1.z * ir12 - c * b2.z * ir22)};
            add_force<T>(a.force, n, i, fi.x, fi.y, fi.z, bad);
            add_force<T>(a.force, n, kk, fk.x, fk.y, fk.z, bad);
            add_force<T>(a.force, n, j, -(fi.x + fk.x), -(fi.y + fk.y), -(fi.z + fk.z), bad);
        }
    } else if (t < a.n_bonds + a.n_angles + a.n_diheds) {
        // force/bonded.rs:112-164, V = k [1 + cos(n phi - delta)]
        const int q = t - a.n_bonds - a.n_angles;
        const int i = a.dihed_i[q], j = a.dihed_j[q], k = a.dihed_k[q], l = a.dihed_l[q];
        first = i;
        const V3<T> b1 = term_diff<T, MI>(a, j, i), b2 = term_diff<T, MI>(a, k, j), b3 = term_diff<T, MI>(a, l, k);
        const V3<T> m = cross(b1, b2), nv = cross(b2, b3);
        const T m2 = dot(m, m), n2 = dot(nv, nv), b2l = sqrt(dot(b2, b2));
        if (m2 != (T)0 && n2 != (T)0 && b2l != (T)0) {
            const T x = dot(m, nv);
            const T y = dot(cross(m, nv), b2) / b2l;
            const T phi = gm_atan2(y, x);
            const T kphi = (T)a.dihed_kphi[q], mult = (T)a.dihed_n[q], delta = (T)a.dihed_delta[q];
            const T arg = mult * phi - delta;
            e = (double)(kphi * ((T)1 + cos(arg)));
            const T dv = kphi * mult * sin(arg);  // -dV/dphi
            const T si = -dv * b2l / m2, sl = dv * b2l / n2;
            const V3<T> fi = {m.x * si, m.y * si, m.z * si}, fl = {nv.x * sl, nv.y * sl, nv.z * sl};
            const T ib = (T)1 / (b2l * b2l);
            const T p = dot(b1, b2) * ib, qq = dot(b3, b2) * ib;
            const V3<T> fj = {-(p + (T)1) * fi.x + qq * fl.x, -(p + (T)1) * fi.y + qq * fl.y, -(p + (T)1) * fi.z + qq * fl.z};
            const V3<T> fk = {p * fi.x - (qq + (T)1) * fl.x, p * fi.y - (qq + (T)1) * fl.y, p * fi.z - (qq + (T)1) * fl.z};
            add_force<T>(a.force, n, i, fi.x, fi.y, fi.z, bad);
            add_force<T>(a.force, n, j, fj.x, fj.y, fj.z, bad);
            add_force<T>(a.force, n, k, fk.x, fk.y, fk.z, bad);
            add_force<T>(a.force, n, l, fl.x, fl.y, fl.z, bad);
        }
    }
    // fixed-order block reduction of the energy
    __shared__ double se[256];
    se[threadIdx.x] = e;
    __syncthreads();
    for (int s2 = 128; s2 > 0; s2 >>= 1) {
        if (threadIdx.x < s2) se[threadIdx.x] += se[threadIdx.x + s2];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.epart_bonded[blk] = se[0];
    if (a.e_sys) gm_add_sys_energy(a.e_sys, first >= 0 ? a.atom_sys[first] : -1, e);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(&a.status->error, bad);
}

// Scaled 1-4 pairs (beyond the reference): unswitched, no cutoff; LJ scaled by
// scale14_lj, Coulomb by scale14_coul.  FP64 arithmetic, few pairs.
template <bool MIXED, bool MI>
__device__ __forceinline__ void pair14_block(const ForceArgs &a, int blk) {
    const int t = blk * blockDim.x + threadIdx.x;
    const int n = a.n;
    double e = 0.0;
    unsigned bad = 0;
    int first = -1;
    if (MIXED && t < a.n14) {
        // FP32 pair arithmetic as in the pair kernel, on the FP64 difference
        const int i = a.p14_i[t], j = a.p14_j[t];
        first = i;
        const V3<float> d = term_diff<float, MI>(a, j, i);
        const float dx = d.x, dy = d.y, dz = d.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > 0.f) {
            const float4 p = a.p14par[t];
            float rinv = rsqrtf(r2);
            rinv = fmaf(0.5f * rinv, fmaf(-r2 * rinv, rinv, 1.0f), rinv);
            const float rinv2 = rinv * rinv;
            float v = 0.f, g = 0.f;  // g = F_r / r
            if (p.y != 0.f) {
                const float s2 = p.x * rinv2, s6 = s2 * s2 * s2, s12 = s6 * s6;
                v += p.y * (s12 - s6);
                g += 6.f * p.y * (2.f * s12 - s6) * rinv2;
            }
            if (p.z != 0.f) {
                const float vc = p.z * rinv;
                v += vc;
                g += vc * rinv2;
            }
            e = (double)v;
            add_force<float>(a.force, n, i, -g * dx, -g * dy, -g * dz, bad);
            add_force<float>(a.force, n, j, g * dx, g * dy, g * dz, bad);
        }
    } else if (!MIXED && t < a.n14) {
        const int i = a.p14_i[t], j = a.p14_j[t];
        first = i;
        const V3<double> d = pdiff<MI>(a, j, i);
        const double dx = d.x, dy = d.y, dz = d.z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > 0.0) {
            const double r = sqrt(r2), rinv = 1.0 / r;
            double v = 0.0, fr = 0.0;
            const double sg = 0.5 * (a.sigma[i] + a.sigma[j]), ep = sqrt(a.epsilon[i] * a.epsilon[j]);
            if (a.scale14_lj != 0.0 && ep != 0.0) {
                const double sr = sg * rinv, s2 = sr * sr, s4 = s2 * s2, s6 = s2 * s4, s12 = s6 * s6;
                v += a.scale14_lj * (4.0 * ep * (s12 - s6));
                fr += a.scale14_lj * (24.0 * ep * rinv * (2.0 * s12 - s6));
            }
            if (a.coulomb && a.scale14_coul != 0.0) {
                const double qq = kCoulomb64 * a.charge64[i] * a.charge64[j];
                v += a.scale14_coul * qq * rinv;
                fr += a.scale14_coul * qq * rinv * rinv;
            }
            e = v;
            const double g = fr * rinv;
            add_force<double>(a.force, n, i, -g * dx, -g * dy, -g * dz, bad);
            add_force<double>(a.force, n, j, g * dx, g * dy, g * dz, bad);
        }
    }
    __shared__ double se[256];
    se[threadIdx.x] = e;
    __syncthreads();
    for (int s2 = 128; s2 > 0; s2 >>= 1) {
        if (threadIdx.x < s2) se[threadIdx.x] += se[threadIdx.x + s2];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.epart14[blk] = se[0];
    if (a.e_sys) gm_add_sys_energy(a.e_sys, first >= 0 ? a.atom_sys[first] : -1, e);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(&a.status->error, bad);
}

template <typename T, bool MI>
__global__ void __launch_bounds__(256) bonded_kernel(ForceArgs a) { bonded_block<T, MI>(a, blockIdx.x); }
template <bool MIXED, bool MI>
__global__ void __launch_bounds__(256) pair14_kernel(ForceArgs a) { pair14_block<MIXED, MI>(a, blockIdx.x); }
// Both in one launch: the first bonded_blocks blocks take the bonded terms,
// the rest the 1-4 pairs (independent work; integer force sums).
template <typename T, bool MIXED, bool MI>
__global__ void __launch_bounds__(256) bonded_pair14_kernel(ForceArgs a) {
    if ((int)blockIdx.x < a.bonded_blocks) bonded_block<T, MI>(a, blockIdx.x);
    else pair14_block<MIXED, MI>(a, blockIdx.x - a.bonded_blocks);
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
    return (int)((t + 255) / 256);
}

void gm_launch_pair(const ForceArgs &a, bool fp64, cudaStream_t s) {
    if (a.n == 0) return;
    const int blocks = (a.n_groups + kPairWarps - 1) / kPairWarps;
    const bool batch = a.e_sys != nullptr;
    if (!fp64) {
        const int W = a.pair_warps == 2 || a.pair_warps == 8 ? a.pair_warps : 4;
        int blocks32 = (a.n_groups * a.split + W - 1) / W;
        if (a.pair_grid > 0 && a.pair_grid < blocks32) blocks32 = a.pair_grid;
        const size_t smem = batch ? 0 : sizeof(float2) * (size_t)a.ntypes * a.ntypes;
#define GM_PAIR32W(P, Q, B, WW)                                                                              \
    pair_kernel_f32<P, Q, B, WW><<<blocks32, WW * 32, smem, s>>>(                                            \
        a.n, a.n_slots, a.cap, a.split, a.coord, a.perm, a.list, a.count, a.gmax, a.ntypes, a.tab32, a.rc2, a.rsw, \
        a.inv_wsw, a.box[0], a.box[1], a.box[2], a.inv_box[0], a.inv_box[1], a.inv_box[2], a.force, a.epart, a.status, \
        a.group_sys, a.e_sys)
#define GM_PAIR32(P, Q, B) { if (W == 2) GM_PAIR32W(P, Q, B, 2); else if (W == 8) GM_PAIR32W(P, Q, B, 8); \
                             else GM_PAIR32W(P, Q, B, 4); }
#define GM_PAIR32B(P, Q) { if (batch) GM_PAIR32(P, Q, true) else GM_PAIR32(P, Q, false) }
        if (a.periodic) { if (a.coulomb) GM_PAIR32B(true, true) else GM_PAIR32B(true, false) }
        else { if (a.coulomb) GM_PAIR32B(false, true) else GM_PAIR32B(false, false) }
#undef GM_PAIR32B
#undef GM_PAIR32
#undef GM_PAIR32W
    } else {
        const size_t smem = batch ? 0 : sizeof(double2) * (size_t)a.ntypes * a.ntypes;
#define GM_PAIR64(P, Q, B)                                                                                        \
    pair_kernel_f64<P, Q, B><<<blocks, kPairWarps * 32, smem, s>>>(                                               \
        a.n, a.n_slots, a.cap, a.pos64s, a.type_sorted, a.perm, a.list, a.count, a.gmax, a.ntypes, a.tab64,     \
        a.rc2_64, a.rsw_64, a.rc_64, a.box64[0], a.box64[1], a.box64[2], a.force, a.epart, a.status, a.group_sys, \
        a.e_sys)
#define GM_PAIR64B(P, Q) { if (batch) GM_PAIR64(P, Q, true); else GM_PAIR64(P, Q, false); }
        if (a.periodic) { if (a.coulomb) GM_PAIR64B(true, true) else GM_PAIR64B(true, false) }
        else { if (a.coulomb) GM_PAIR64B(false, true) else GM_PAIR64B(false, false) }
#undef GM_PAIR64B
#undef GM_PAIR64
    }
}

void gm_launch_bonded(const ForceArgs &a, bool fp64, cudaStream_t s) {
    if (a.bonded_blocks == 0) return;
    if (a.bonded_mi) {
        if (fp64) bonded_kernel<double, true><<<a.bonded_blocks, 256, 0, s>>>(a);
        else bonded_kernel<float, true><<<a.bonded_blocks, 256, 0, s>>>(a);
    } else {
        if (fp64) bonded_kernel<double, false><<<a.bonded_blocks, 256, 0, s>>>(a);
        else bonded_kernel<float, false><<<a.bonded_blocks, 256, 0, s>>>(a);
    }
}

void gm_launch_bonded_pair14(const ForceArgs &a, bool fp64, cudaStream_t s) {
    const int blocks = a.bonded_blocks + a.blocks14;
    if (blocks == 0) return;
    if (a.bonded_mi) {
        if (fp64) bonded_pair14_kernel<double, false, true><<<blocks, 256, 0, s>>>(a);
        else bonded_pair14_kernel<float, true, true><<<blocks, 256, 0, s>>>(a);
    } else {
        if (fp64) bonded_pair14_kernel<double, false, false><<<blocks, 256, 0, s>>>(a);
        else bonded_pair14_kernel<float, true, false><<<blocks, 256, 0, s>>>(a);
    }
}

void gm_launch_pair14(const ForceArgs &a, bool fp64, cudaStream_t s) {
    if (a.blocks14 == 0) return;
    if (a.bonded_mi) {
        if (fp64) pair14_kernel<false, true><<<a.blocks14, 256, 0, s>>>(a);
        else pair14_kernel<true, true><<<a.blocks14, 256, 0, s>>>(a);
    } else {
        if (fp64) pair14_kernel<false, false><<<a.blocks14, 256, 0, s>>>(a);
        else pair14_kernel<true, false><<<a.blocks14, 256, 0, s>>>(a);
    }
}

void gm_launch_energy(const ForceArgs &a, cudaStream_t s) {
    energy_kernel<<<1, 256, 0, s>>>(a.epart, a.n_epart_total, a.energy);
}
