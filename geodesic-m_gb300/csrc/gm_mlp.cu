// gm_mlp.cu — constraint warm start: per-constraint features, the 12-64-64-1
// SiLU network (inference, recording of training samples, forward/backward
// and Adam), all on the device.
//
// The quantity predicted is the constraint's total SHAKE multiplier Lambda
// (the sum of the Jacobi lambdas of a cold solve, constraint.rs:62-152),
// made dimensionless as t = Lambda * 2 (1/m_i + 1/m_j).  The first Jacobi
// step alone gives t1 = (|r_trial|^2 - d0^2) / (r_trial . r_ref) exactly
// (constraint.rs:110-115), so the network learns only the correction
// t - t1: the second-order term of an isolated constraint and the coupling
// between constraints sharing an atom, which BF16 then carries to a small
// relative error of the whole.
// Numerics: the matmul weights (W1, W2, w3) and the activations (input,
// both hidden layers) are rounded to BF16 (round to nearest even), biases
// stay FP32, every sum is FP32 in ascending index order, SiLU(z) =
// z / (1 + exp(-z)).  Training gradients treat the BF16 roundings as the
// identity.  Per-block gradient partials are summed in block order, so
// training is run-to-run identical.
#include <cuda_bf16.h>

#include "gm_internal.cuh"

namespace {

constexpr int kIn = GM_WS_IN, kH = GM_WS_H, kNP = GM_WS_NPAR;
constexpr int kTile = GM_WS_TILE;
constexpr int kRow = kH + 1;  // padded shared-memory row (conflict-free per-sample rows)

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }
// The same function for inference: correctly rounded reciprocal of 1 + exp(-z)
// (equal to the division above), no division subroutine.
__device__ __forceinline__ float sigmoid_rcp(float z) { return __frcp_rn(1.0f + expf(-z)); }

__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by, double bz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// Reference bond direction r_k / |r_k| in FP32 (the FP64 difference rounded
// once, then correctly rounded FP32 operations in a fixed order).
__device__ __forceinline__ void ref_unit(const WsFeatureArgs &a, int k, float &ux, float &uy, float &uz) {
    const int i = a.constr_i[k], j = a.constr_j[k], n = a.n_atoms;
    const float rx = (float)__dsub_rn(a.dref[i], a.dref[j]), ry = (float)__dsub_rn(a.dref[n + i], a.dref[n + j]),
                rz = (float)__dsub_rn(a.dref[2 * n + i], a.dref[2 * n + j]);
    const float il = __fdiv_rn(1.0f, __fsqrt_rn(dot3f(rx, ry, rz, rx, ry, rz)));
    ux = __fmul_rn(rx, il);
    uy = __fmul_rn(ry, il);
    uz = __fmul_rn(rz, il);
}

// Pass 1: the constraint's own features 0-7, t1 and the scale.
__global__ void ws_features_kernel(WsFeatureArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_constr) return;
    const int i = a.constr_i[k], j = a.constr_j[k], n = a.n_atoms;
    const double d0sq = a.constr_dsq[k];
    const double rx = __dsub_rn(a.dref[i], a.dref[j]), ry = __dsub_rn(a.dref[n + i], a.dref[n + j]),
                 rz = __dsub_rn(a.dref[2 * n + i], a.dref[2 * n + j]);
    const double tx = __dsub_rn(a.pos[i], a.pos[j]), ty = __dsub_rn(a.pos[n + i], a.pos[n + j]),
                 tz = __dsub_rn(a.pos[2 * n + i], a.pos[2 * n + j]);
    const double t2 = dot3(tx, ty, tz, tx, ty, tz);
    const double dr = dot3(tx, ty, tz, rx, ry, rz);
    const double t1 = dr == 0.0 ? 0.0 : __ddiv_rn(__dsub_rn(t2, d0sq), dr);
    a.t1[k] = t1;
    a.scale[k] = __dmul_rn(2.0, __dadd_rn(a.inv_mass[i], a.inv_mass[j]));
    float *f = a.feat + (size_t)k * kIn;
    f[0] = (float)__ddiv_rn(__dsub_rn(t2, d0sq), d0sq);
    f[1] = (float)__ddiv_rn(dr, d0sq);
    f[2] = (float)__dsqrt_rn(d0sq);
    f[3] = (float)a.inv_mass[i];
    f[4] = (float)a.inv_mass[j];
    f[5] = (float)(a.atom_cstart[i + 1] - a.atom_cstart[i]);
    f[6] = (float)(a.atom_cstart[j + 1] - a.atom_cstart[j]);
    f[7] = (float)t1;
    float ux, uy, uz;
    ref_unit(a, k, ux, uy, uz);
    a.unit[k] = make_float4(ux, uy, uz, 0.f);
}

// Pass 2: coupling to the other constraints on the constraint's two atoms
// (features 8-11) in FP32, atom i's constraints then atom j's, each
// ascending; masses and t1 enter rounded to FP32.
__global__ void ws_coupling_kernel(WsFeatureArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_constr) return;
    const int ends[2] = {a.constr_i[k], a.constr_j[k]};
    const float wk = __fadd_rn((float)a.inv_mass[ends[0]], (float)a.inv_mass[ends[1]]);
    const float4 uk = a.unit[k];
    const float ux = uk.x, uy = uk.y, uz = uk.z;
    float c1 = 0.0f, c2 = 0.0f, cmax = 0.0f, ct = 0.0f;
    for (int e = 0; e < 2; e++) {
        const int at = ends[e];
        const float sk = e == 0 ? 1.0f : -1.0f;
        const float inv_a = (float)a.inv_mass[at];
        for (int q = a.atom_cstart[at]; q < a.atom_cstart[at + 1]; q++) {
            const int ref = a.atom_cref[q];
            const int l = ref >= 0 ? ref : -ref - 1;
            if (l == k) continue;
            const float sl = ref >= 0 ? 1.0f : -1.0f;
            const float4 ul = a.unit[l];
            const float cs = dot3f(ux, uy, uz, ul.x, ul.y, ul.z);
            const float wl = __fadd_rn((float)a.inv_mass[a.constr_i[l]], (float)a.inv_mass[a.constr_j[l]]);
            const float coup = __fmul_rn(__fmul_rn(__fdiv_rn(inv_a, wk), cs), __fmul_rn(sk, sl));
            const float tl = (float)a.t1[l];
            c1 = __fadd_rn(c1, __fdiv_rn(__fmul_rn(__fmul_rn(coup, tl), wk), wl));
            c2 = __fadd_rn(c2, __fmul_rn(coup, coup));
            cmax = fmaxf(cmax, fabsf(cs));
            ct = __fadd_rn(ct, tl);
        }
    }
    float *f = a.feat + (size_t)k * kIn;
    f[8] = c1;
    f[9] = c2;
    f[10] = cmax;
    f[11] = ct;
}

// Weights into shared memory: matmul weights BF16-rounded, biases as is.
// 128-bit loads, four in flight per thread before their stores (every block
// loads the 20 KB, so the latency of one load at a time would dominate a
// short kernel).  The sections start on 16-byte boundaries (offsets are
// multiples of four floats), and so do the shared arrays.
__device__ __forceinline__ float4 bf4(float4 v) { return make_float4(bf(v.x), bf(v.y), bf(v.z), bf(v.w)); }
__device__ __forceinline__ void store_weight4(int o, float4 v, float *sW1, float *sb1, float *sW2, float *sb2,
                                              float *sw3) {
    if (o < GM_WS_OFF_B1) *reinterpret_cast<float4 *>(sW1 + o) = bf4(v);
    else if (o < GM_WS_OFF_W2) *reinterpret_cast<float4 *>(sb1 + o - GM_WS_OFF_B1) = v;
    else if (o < GM_WS_OFF_B2) *reinterpret_cast<float4 *>(sW2 + o - GM_WS_OFF_W2) = bf4(v);
    else if (o < GM_WS_OFF_W3) *reinterpret_cast<float4 *>(sb2 + o - GM_WS_OFF_B2) = v;
    else *reinterpret_cast<float4 *>(sw3 + o - GM_WS_OFF_W3) = bf4(v);
}
__device__ void load_weights(const float *P, float *sW1, float *sb1, float *sW2, float *sb2, float *sw3, float *sb3) {
    const float4 *P4 = reinterpret_cast<const float4 *>(P);
    constexpr int kW4 = GM_WS_OFF_B3 / 4;
    for (int t0 = threadIdx.x; t0 < kW4; t0 += 4 * blockDim.x) {
        float4 v[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int t = t0 + r * (int)blockDim.x;
            v[r] = t < kW4 ? __ldg(P4 + t) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int t = t0 + r * (int)blockDim.x;
            if (t < kW4) store_weight4(4 * t, v[r], sW1, sb1, sW2, sb2, sw3);
        }
    }
    if (threadIdx.x == 0) *sb3 = P[GM_WS_OFF_B3];
}

// Inference: TPC threads per constraint, thread q owning the U = 64 / TPC
// hidden units [U q, U q + U) of both layers.  Weights are read from shared
// memory four at a time (128-bit loads) into U independent accumulations; the
// first layer's activations reach the other threads of the group by
// shuffles.  Every sum keeps the ascending order of the one-thread form (each
// unit over its inputs in index order; the output over the units in index
// order, passed along the group).  Inputs are standardised with the
// correctly rounded reciprocal of the spread (within an ulp of the division,
// before their BF16 rounding) and the SiLU's 1 / (1 + exp(-z)) is a
// correctly rounded reciprocal (equal to the division).
template <int TPC>
__global__ void __launch_bounds__(256) ws_infer_kernel(int n, const float *__restrict__ feat,
                                                       const float *__restrict__ P, const float *__restrict__ norm,
                                                       const double *__restrict__ scale,
                                                       const double *__restrict__ t1, double *lam0, float *y_out) {
    constexpr int U = kH / TPC;
    static_assert(U % 4 == 0, "units per thread in whole 128-bit loads");
    __shared__ __align__(16) float sW1[kIn * kH];
    __shared__ __align__(16) float sW2[kH * kH];
    __shared__ __align__(16) float sb1[kH];
    __shared__ __align__(16) float sb2[kH];
    __shared__ __align__(16) float sw3[kH];
    __shared__ float sb3, snorm[GM_WS_NNORM], sinv[kIn];
    load_weights(P, sW1, sb1, sW2, sb2, sw3, &sb3);
    if (threadIdx.x < GM_WS_NNORM) snorm[threadIdx.x] = norm[threadIdx.x];
    if (threadIdx.x < kIn) sinv[threadIdx.x] = __frcp_rn(norm[kIn + threadIdx.x]);
    __syncthreads();
    const int q = threadIdx.x % TPC, base = (threadIdx.x & 31) - q;
    const int k = blockIdx.x * (blockDim.x / TPC) + threadIdx.x / TPC;
    const bool live = k < n;  // a group past n still joins the shuffles
    const int o0 = U * q;
    float x[kIn];
#pragma unroll
    for (int f = 0; f < kIn; f++) x[f] = live ? bf((feat[(size_t)k * kIn + f] - snorm[f]) * sinv[f]) : 0.f;
    float z[U];
#pragma unroll
    for (int j = 0; j < U; j++) z[j] = sb1[o0 + j];
#pragma unroll
    for (int f = 0; f < kIn; f++) {
        const float4 *w = reinterpret_cast<const float4 *>(sW1 + f * kH + o0);
#pragma unroll
        for (int v = 0; v < U / 4; v++) {
            const float4 w4 = w[v];
            z[4 * v] = fmaf(x[f], w4.x, z[4 * v]);
            z[4 * v + 1] = fmaf(x[f], w4.y, z[4 * v + 1]);
            z[4 * v + 2] = fmaf(x[f], w4.z, z[4 * v + 2]);
            z[4 * v + 3] = fmaf(x[f], w4.w, z[4 * v + 3]);
        }
    }
    float a1[U];
#pragma unroll
    for (int j = 0; j < U; j++) a1[j] = bf(z[j] * sigmoid_rcp(z[j]));
#pragma unroll
    for (int j = 0; j < U; j++) z[j] = sb2[o0 + j];
#pragma unroll
    for (int src = 0; src < TPC; src++) {
#pragma unroll
        for (int jj = 0; jj < U; jj++) {
            const float a = __shfl_sync(0xffffffffu, a1[jj], base + src);  // unit U src + jj
            const float4 *w = reinterpret_cast<const float4 *>(sW2 + (U * src + jj) * kH + o0);
#pragma unroll
            for (int v = 0; v < U / 4; v++) {
                const float4 w4 = w[v];
                z[4 * v] = fmaf(a, w4.x, z[4 * v]);
                z[4 * v + 1] = fmaf(a, w4.y, z[4 * v + 1]);
                z[4 * v + 2] = fmaf(a, w4.z, z[4 * v + 2]);
                z[4 * v + 3] = fmaf(a, w4.w, z[4 * v + 3]);
            }
        }
    }
    // the output: units 0..63 in order, thread 0's, then thread 1's, ...
    float y = sb3;
#pragma unroll
    for (int src = 0; src < TPC; src++) {
        if (q == src) {
#pragma unroll
            for (int j = 0; j < U; j++) y = fmaf(bf(z[j] * sigmoid_rcp(z[j])), sw3[o0 + j], y);
        }
        y = __shfl_sync(0xffffffffu, y, base + src);
    }
    if (!live || q != 0) return;
    if (y_out) y_out[k] = y;
    if (lam0) lam0[k] = (t1[k] + ((double)y * (double)snorm[25] + (double)snorm[24])) / scale[k];
}

__global__ void ws_record_kernel(int nc, const float *feat, const double *lam_sum, const double *scale,
                                 const double *t1, float *rec_feat, float *rec_t, int stride, int cap,
                                 const DevStatus *st) {
    if (st->error || stride <= 0 || st->step % (unsigned long long)stride) return;
    const unsigned slot = st->rec_n;
    if (slot >= (unsigned)cap) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nc) return;
    const size_t base = (size_t)slot * nc;
    for (int f = 0; f < kIn; f++) rec_feat[(base + k) * kIn + f] = feat[(size_t)k * kIn + f];
    rec_t[base + k] = (float)(lam_sum[k] * scale[k] - t1[k]);
}

__global__ void ws_record_advance(int stride, int cap, DevStatus *st) {
    if (st->error || stride <= 0 || st->step % (unsigned long long)stride) return;
    if (st->rec_n < (unsigned)cap) st->rec_n += 1;
}

// Column sums and sums of squares (13 columns: 12 features, target) per block.
constexpr int kStatThreads = 128;

__global__ void __launch_bounds__(kStatThreads) ws_stats_partial(long long n, const float *feat, const float *t,
                                                                 double *partial) {
    __shared__ double sh[26][kStatThreads];
    double s[13], q[13];
    for (int c = 0; c < 13; c++) s[c] = q[c] = 0.0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < kIn; c++) {
            const double v = feat[r * kIn + c];
            s[c] += v;
            q[c] += v * v;
        }
        const double v = t[r];
        s[12] += v;
        q[12] += v * v;
    }
    for (int c = 0; c < 13; c++) { sh[c][threadIdx.x] = s[c]; sh[13 + c][threadIdx.x] = q[c]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 26; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 26) partial[blockIdx.x * 26 + threadIdx.x] = sh[threadIdx.x][0];
}

// Means and scales; a column with (near) zero spread keeps scale 1.
__global__ void ws_stats_final(int blocks, const double *partial, long long n, float *norm) {
    const int c = threadIdx.x;
    if (c >= 13) return;
    double S = 0.0, Q = 0.0;
    for (int b = 0; b < blocks; b++) { S += partial[b * 26 + c]; Q += partial[b * 26 + 13 + c]; }
    const double mean = n > 0 ? S / (double)n : 0.0;
    const double var = n > 0 ? fmax(Q / (double)n - mean * mean, 0.0) : 0.0;
    double sd = sqrt(var);
    if (!(sd > 1e-6 * fmax(1.0, fabs(mean)))) sd = 1.0;
    if (c < kIn) { norm[c] = (float)mean; norm[kIn + c] = (float)sd; }
    else { norm[24] = (float)mean; norm[25] = (float)sd; }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    // splitmix64 finaliser
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Shared-memory layout of the training kernel (floats).
constexpr int kSmW = kIn * kH + kH + kH * kH + kH + kH + 4;
constexpr int kSmX = kTile * (kIn + 1);
constexpr int kSmRows = kTile * kRow;
constexpr size_t kGradSmem = sizeof(float) * ((size_t)kSmW + kSmX + 4 * (size_t)kSmRows + 2 * kTile);

// Forward and backward over one tile of 128 samples; one thread per sample
// for the passes, then one thread per parameter group for the block sums.
__global__ void __launch_bounds__(kTile) ws_grad_kernel(long long n, const float *__restrict__ feat,
                                                        const float *__restrict__ tt, const float *__restrict__ norm,
                                                        int standardized, const float *__restrict__ P,
                                                        unsigned long long seed, long long iter, long long n_valid,
                                                        float inv_batch, float *__restrict__ partial) {
    extern __shared__ float sm[];
    float *sW1 = sm, *sb1 = sW1 + kIn * kH, *sW2 = sb1 + kH, *sb2 = sW2 + kH * kH, *sw3 = sb2 + kH, *sb3 = sw3 + kH;
    float *xb = sm + kSmW;
    float *a1b = xb + kSmX, *a2b = a1b + kSmRows, *d2 = a2b + kSmRows, *d1 = d2 + kSmRows;
    float *sdy = d1 + kSmRows, *sloss = sdy + kTile;
    load_weights(P, sW1, sb1, sW2, sb2, sw3, sb3);
    __syncthreads();
    const int s = threadIdx.x;
    const long long row = (long long)blockIdx.x * kTile + s;
    const bool valid = row < n_valid;
    long long sample;
    if (iter < 0) sample = row < n ? row : n - 1;
    else sample = (long long)(mix64(seed ^ mix64((unsigned long long)iter * 0x100000001B3ull + (unsigned long long)row)) %
                              (unsigned long long)n);
    // forward
    float *xs = xb + s * (kIn + 1);
    for (int f = 0; f < kIn; f++) {
        const float v = feat[sample * kIn + f];
        xs[f] = bf(standardized ? v : (v - norm[f]) / norm[kIn + f]);
    }
    const float t = standardized ? tt[sample] : (tt[sample] - norm[24]) / norm[25];
    float sd1[kH];
    float *a1s = a1b + s * kRow, *a2s = a2b + s * kRow, *d2s = d2 + s * kRow, *d1s = d1 + s * kRow;
#pragma unroll
    for (int o = 0; o < kH; o++) {
        float z = sb1[o];
        for (int f = 0; f < kIn; f++) z = fmaf(xs[f], sW1[f * kH + o], z);
        const float g = sigmoid(z);
        a1s[o] = bf(z * g);
        sd1[o] = g * (1.0f + z * (1.0f - g));
    }
    float y = *sb3;
    for (int o = 0; o < kH; o++) {
        float z = sb2[o];
        for (int q = 0; q < kH; q++) z = fmaf(a1s[q], sW2[q * kH + o], z);
        const float g = sigmoid(z);
        const float a2 = bf(z * g);
        a2s[o] = a2;
        d2s[o] = g * (1.0f + z * (1.0f - g));
        y = fmaf(a2, sw3[o], y);
    }
    const float r = y - t;
    const float dy = valid ? 2.0f * r * inv_batch : 0.0f;
    sdy[s] = dy;
    sloss[s] = valid ? r * r : 0.0f;
    // backward through layer 3 and 2
    for (int o = 0; o < kH; o++) d2s[o] = sw3[o] * dy * d2s[o];
#pragma unroll
    for (int q = 0; q < kH; q++) {
        float da = 0.0f;
        for (int o = 0; o < kH; o++) da = fmaf(sW2[q * kH + o], d2s[o], da);
        d1s[q] = da * sd1[q];
    }
    __syncthreads();
    // block sums over the tile's samples, ascending
    float *out = partial + (size_t)blockIdx.x * (kNP + 1);
    {
        const int k = s >> 1, o0 = (s & 1) * 32;
        float acc[32];
#pragma unroll
        for (int j = 0; j < 32; j++) acc[j] = 0.0f;
        for (int q = 0; q < kTile; q++) {
            const float a = a1b[q * kRow + k];
#pragma unroll
            for (int j = 0; j < 32; j++) acc[j] = fmaf(a, d2[q * kRow + o0 + j], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 32; j++) out[GM_WS_OFF_W2 + k * kH + o0 + j] = acc[j];
    }
    for (int e = s; e < kIn * kH; e += kTile) {
        const int f = e / kH, o = e % kH;
        float acc = 0.0f;
        for (int q = 0; q < kTile; q++) acc = fmaf(xb[q * (kIn + 1) + f], d1[q * kRow + o], acc);
        out[GM_WS_OFF_W1 + e] = acc;
    }
    if (s < kH) {
        float g1 = 0.0f, g3 = 0.0f;
        for (int q = 0; q < kTile; q++) {
            g1 += d1[q * kRow + s];
            g3 = fmaf(a2b[q * kRow + s], sdy[q], g3);
        }
        out[GM_WS_OFF_B1 + s] = g1;
        out[GM_WS_OFF_W3 + s] = g3;
    } else {
        const int o = s - kH;
        float g2 = 0.0f;
        for (int q = 0; q < kTile; q++) g2 += d2[q * kRow + o];
        out[GM_WS_OFF_B2 + o] = g2;
        if (o == 0) {
            float gb = 0.0f, l = 0.0f;
            for (int q = 0; q < kTile; q++) { gb += sdy[q]; l += sloss[q]; }
            out[GM_WS_OFF_B3] = gb;
            out[kNP] = l;
        }
    }
}

// Sum of the block partials (block order, FP64), then Adam or a copy out.
__global__ void ws_update_kernel(int blocks, const float *partial, float *P, float *m, float *v, float lr, float b1,
                                 float b2, float eps, int t, float *grad_out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kNP) return;
    double g = 0.0;
    for (int b = 0; b < blocks; b++) g += partial[(size_t)b * (kNP + 1) + p];
    if (!m) {
        if (grad_out) grad_out[p] = (float)g;
        return;
    }
    if (p == kNP) {
        if (grad_out) grad_out[0] = (float)g;
        return;
    }
    const float gf = (float)g;
    const float mm = b1 * m[p] + (1.0f - b1) * gf;
    const float vv = b2 * v[p] + (1.0f - b2) * gf * gf;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.0f - powf(b1, (float)t));
    const float vh = vv / (1.0f - powf(b2, (float)t));
    P[p] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

void gm_launch_ws_features(const WsFeatureArgs &a, cudaStream_t s) {
    if (a.n_constr == 0) return;
    ws_features_kernel<<<(a.n_constr + 255) / 256, 256, 0, s>>>(a);
    ws_coupling_kernel<<<(a.n_constr + 255) / 256, 256, 0, s>>>(a);
}

void gm_launch_ws_infer(int n, const float *feat, const float *params, const float *norm, const double *scale,
                        const double *t1, double *lam0, float *y_out, cudaStream_t s) {
    if (n == 0) return;
    constexpr int kTPC = 16, kThreads = 256, kPerBlock = kThreads / kTPC;
    ws_infer_kernel<kTPC><<<(n + kPerBlock - 1) / kPerBlock, kThreads, 0, s>>>(n, feat, params, norm, scale, t1, lam0,
                                                                              y_out);
}

void gm_launch_ws_record(int n_constr, const float *feat, const double *lam_sum, const double *scale, const double *t1,
                         float *rec_feat, float *rec_t, int stride, int cap_slots, DevStatus *st, cudaStream_t s) {
    if (n_constr == 0) return;
    ws_record_kernel<<<(n_constr + 255) / 256, 256, 0, s>>>(n_constr, feat, lam_sum, scale, t1, rec_feat, rec_t,
                                                             stride, cap_slots, st);
    ws_record_advance<<<1, 1, 0, s>>>(stride, cap_slots, st);
}

void gm_launch_ws_stats(long long n, const float *feat, const float *t, double *partial, int blocks, float *norm,
                        cudaStream_t s) {
    ws_stats_partial<<<blocks, kStatThreads, 0, s>>>(n, feat, t, partial);
    ws_stats_final<<<1, 32, 0, s>>>(blocks, partial, n, norm);
}

void gm_launch_ws_grad(long long n, const float *feat, const float *t, const float *norm, bool standardized,
                       const float *params, int blocks, unsigned long long seed, long long iter, long long n_valid,
                       float *partial, cudaStream_t s) {
    static bool attr = false;  // per process; the attribute is a property of the kernel
    if (!attr) {
        cudaFuncSetAttribute(ws_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
        attr = true;
    }
    const float inv_batch = 1.0f / (float)(n_valid < (long long)blocks * kTile ? n_valid : (long long)blocks * kTile);
    ws_grad_kernel<<<blocks, kTile, kGradSmem, s>>>(n, feat, t, norm, standardized ? 1 : 0, params, seed, iter,
                                                     n_valid, inv_batch, partial);
}

void gm_launch_ws_update(int blocks, const float *partial, float *params, float *m, float *v, float lr, float b1,
                         float b2, float eps, int t, float *grad_out, cudaStream_t s) {
    ws_update_kernel<<<(kNP + 1 + 255) / 256, 256, 0, s>>>(blocks, partial, params, m, v, lr, b1, b2, eps, t,
                                                            grad_out);
}
