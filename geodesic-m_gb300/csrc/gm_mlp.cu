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
// stay FP32, SiLU(z) = z / (1 + exp(-z)).  Inference runs both hidden layers
// on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation,
// in the tensor cores' own summation order), fused with the feature pass:
// one kernel per SHAKE solve.  The training kernels sum in FP32 in ascending
// index order and treat the BF16 roundings as the identity; per-block
// gradient partials are summed in block order, so training is run-to-run
// identical.
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

// t1 = (|r_trial|^2 - d0^2) / (r_trial . r_ref) of constraint k, FP64.
__device__ __forceinline__ double t1_of(const WsFeatureArgs &a, int k, double *t2o = nullptr, double *dro = nullptr) {
    const int i = a.constr_i[k], j = a.constr_j[k], n = a.n_atoms;
    const double d0sq = a.constr_dsq[k];
    const double rx = __dsub_rn(a.dref[i], a.dref[j]), ry = __dsub_rn(a.dref[n + i], a.dref[n + j]),
                 rz = __dsub_rn(a.dref[2 * n + i], a.dref[2 * n + j]);
    const double tx = __dsub_rn(a.pos[i], a.pos[j]), ty = __dsub_rn(a.pos[n + i], a.pos[n + j]),
                 tz = __dsub_rn(a.pos[2 * n + i], a.pos[2 * n + j]);
    const double t2 = dot3(tx, ty, tz, tx, ty, tz);
    const double dr = dot3(tx, ty, tz, rx, ry, rz);
    if (t2o) *t2o = t2;
    if (dro) *dro = dr;
    return dr == 0.0 ? 0.0 : __ddiv_rn(__dsub_rn(t2, d0sq), dr);
}

// The constraint's own features 0-7, its t1 and its scale 2 (1/m_i + 1/m_j).
__device__ __forceinline__ void own_features(const WsFeatureArgs &a, int k, float *f, double &t1, double &scale) {
    const int i = a.constr_i[k], j = a.constr_j[k];
    const double d0sq = a.constr_dsq[k];
    double t2, dr;
    t1 = t1_of(a, k, &t2, &dr);
    scale = __dmul_rn(2.0, __dadd_rn(a.inv_mass[i], a.inv_mass[j]));
    f[0] = (float)__ddiv_rn(__dsub_rn(t2, d0sq), d0sq);
    f[1] = (float)__ddiv_rn(dr, d0sq);
    f[2] = (float)__dsqrt_rn(d0sq);
    f[3] = (float)a.inv_mass[i];
    f[4] = (float)a.inv_mass[j];
    f[5] = (float)(a.atom_cstart[i + 1] - a.atom_cstart[i]);
    f[6] = (float)(a.atom_cstart[j + 1] - a.atom_cstart[j]);
    f[7] = (float)t1;
}

// Coupling to the other constraints on the constraint's two atoms (features
// 8-11) in FP32, atom i's constraints then atom j's, each ascending; masses
// and the neighbours' t1 enter rounded to FP32.
__device__ __forceinline__ void coupling_features(const WsFeatureArgs &a, int k, float *f) {
    const int ends[2] = {a.constr_i[k], a.constr_j[k]};
    const float wk = __fadd_rn((float)a.inv_mass[ends[0]], (float)a.inv_mass[ends[1]]);
    float ux, uy, uz;
    ref_unit(a, k, ux, uy, uz);
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
            float vx, vy, vz;
            ref_unit(a, l, vx, vy, vz);
            const float cs = dot3f(ux, uy, uz, vx, vy, vz);
            const float wl = __fadd_rn((float)a.inv_mass[a.constr_i[l]], (float)a.inv_mass[a.constr_j[l]]);
            const float coup = __fmul_rn(__fmul_rn(__fdiv_rn(inv_a, wk), cs), __fmul_rn(sk, sl));
            const float tl = (float)t1_of(a, l);
            c1 = __fadd_rn(c1, __fdiv_rn(__fmul_rn(__fmul_rn(coup, tl), wk), wl));
            c2 = __fadd_rn(c2, __fmul_rn(coup, coup));
            cmax = fmaxf(cmax, fabsf(cs));
            ct = __fadd_rn(ct, tl);
        }
    }
    f[8] = c1;
    f[9] = c2;
    f[10] = cmax;
    f[11] = ct;
}

// ---- the network on the tensor cores ----------------------------------
//
// A warp takes 32 constraints (rows) at a time as two m16 tiles.  Layer 1:
// X [16 x 16] (12 features, 4 zero columns) times W1 [16 x 64]: eight
// m16n8k16 MMAs.  Its accumulators, after bias, SiLU and BF16 rounding, are
// already laid out as the A operand of layer 2 (an m16n8 accumulator pair
// (n-tiles 2kk, 2kk + 1) is the A fragment of k-step kk), so layer 2, [16 x
// 64] times W2 [64 x 64], is 32 MMAs without leaving registers.  Layer 3 (64
// -> 1) is a dot product per row over the lane quad that holds it.  The B
// operands (W1, W2 as BF16 pairs) sit in shared memory in fragment order:
// one conflict-free 64-bit load per lane per MMA.

struct MlpSmem {
    uint2 b1f[8][32];     // W1 fragments per n-tile
    uint2 b2f[4][8][32];  // W2 fragments per (k-step, n-tile)
    float b1[kH], b2[kH], w3[kH];
    float b3;
    float mean[kIn], inv[kIn], tmean, tscale;
};

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ float silu(float z) { return z * sigmoid_rcp(z); }

// The parameters in fragment order (BF16 pairs: the lower column index in
// the low half), biases and the input standardisation (norm may be null:
// inputs already standardised).
__device__ void load_mlp(const float *__restrict__ P, const float *__restrict__ norm, MlpSmem &S) {
    for (int e = threadIdx.x; e < 8 * 32; e += blockDim.x) {
        const int j = e >> 5, l = e & 31, g = l >> 2, t = l & 3, n = 8 * j + g;
        float w[4];
        const int ks[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] = ks[q] < kIn ? P[GM_WS_OFF_W1 + ks[q] * kH + n] : 0.0f;
        S.b1f[j][l] = make_uint2(pack_bf2(w[0], w[1]), pack_bf2(w[2], w[3]));
    }
    for (int e = threadIdx.x; e < 4 * 8 * 32; e += blockDim.x) {
        const int kk = e >> 8, j = (e >> 5) & 7, l = e & 31, g = l >> 2, t = l & 3;
        const int n = 8 * j + g, k0 = 16 * kk + 2 * t;
        const float *W2 = P + GM_WS_OFF_W2;
        S.b2f[kk][j][l] = make_uint2(pack_bf2(W2[k0 * kH + n], W2[(k0 + 1) * kH + n]),
                                     pack_bf2(W2[(k0 + 8) * kH + n], W2[(k0 + 9) * kH + n]));
    }
    for (int o = threadIdx.x; o < kH; o += blockDim.x) {
        S.b1[o] = P[GM_WS_OFF_B1 + o];
        S.b2[o] = P[GM_WS_OFF_B2 + o];
        S.w3[o] = bf(P[GM_WS_OFF_W3 + o]);
    }
    if (threadIdx.x < kIn) {
        S.mean[threadIdx.x] = norm ? norm[threadIdx.x] : 0.0f;
        S.inv[threadIdx.x] = norm ? __frcp_rn(norm[kIn + threadIdx.x]) : 1.0f;
    }
    if (threadIdx.x == 0) {
        S.b3 = P[GM_WS_OFF_B3];
        S.tmean = norm ? norm[24] : 0.0f;
        S.tscale = norm ? norm[25] : 1.0f;
    }
}

// y of the warp's 32 rows: sX[row][c] holds the BF16 input pair (2c, 2c + 1)
// of the row (c < 6; 6 and 7 are zero); y goes to sy[row].
__device__ __forceinline__ void mlp_rows32(const MlpSmem &S, const uint32_t (*sX)[8], float *sy) {
    const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        const uint32_t a0 = sX[r0][t], a1 = sX[r1][t], a2 = sX[r0][t + 4], a3 = sX[r1][t + 4];
        float z1[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float c0 = S.b1[8 * j + 2 * t], c1 = S.b1[8 * j + 2 * t + 1];
            z1[j][0] = c0; z1[j][1] = c1; z1[j][2] = c0; z1[j][3] = c1;
            mma_bf16(z1[j], a0, a1, a2, a3, S.b1f[j][l]);
        }
        uint32_t A2[4][4];
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            A2[kk][0] = pack_bf2(silu(z1[2 * kk][0]), silu(z1[2 * kk][1]));
            A2[kk][1] = pack_bf2(silu(z1[2 * kk][2]), silu(z1[2 * kk][3]));
            A2[kk][2] = pack_bf2(silu(z1[2 * kk + 1][0]), silu(z1[2 * kk + 1][1]));
            A2[kk][3] = pack_bf2(silu(z1[2 * kk + 1][2]), silu(z1[2 * kk + 1][3]));
        }
        float z2[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float c0 = S.b2[8 * j + 2 * t], c1 = S.b2[8 * j + 2 * t + 1];
            z2[j][0] = c0; z2[j][1] = c1; z2[j][2] = c0; z2[j][3] = c1;
        }
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
#pragma unroll
            for (int j = 0; j < 8; j++) mma_bf16(z2[j], A2[kk][0], A2[kk][1], A2[kk][2], A2[kk][3], S.b2f[kk][j][l]);
        float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = 8 * j + 2 * t;
            y0 = fmaf(bf(silu(z2[j][0])), S.w3[c], y0);
            y0 = fmaf(bf(silu(z2[j][1])), S.w3[c + 1], y0);
            y1 = fmaf(bf(silu(z2[j][2])), S.w3[c], y1);
            y1 = fmaf(bf(silu(z2[j][3])), S.w3[c + 1], y1);
        }
        y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
        y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
        if (t == 0) {
            sy[r0] = S.b3 + y0;
            sy[r1] = S.b3 + y1;
        }
    }
}

constexpr int kPredWarps = 4;

// One kernel per SHAKE solve: each lane computes one constraint's features
// (written out for the recorder, with t1 and the scale), and with `infer`
// the warp runs the network on its 32 constraints and writes the predicted
// multipliers lam0 = (t1 + y t_scale + t_mean) / scale.
__global__ void __launch_bounds__(kPredWarps * 32) ws_predict_kernel(WsFeatureArgs a, const float *__restrict__ P,
                                                                   const float *__restrict__ norm, double *lam0,
                                                                   int infer) {
    __shared__ MlpSmem S;
    __shared__ uint32_t sX[kPredWarps][32][8];
    __shared__ float sy[kPredWarps][32];
    if (infer) load_mlp(P, norm, S);
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int n_tiles = (a.n_constr + 31) / 32;
    for (int tile = blockIdx.x * kPredWarps + w; tile < n_tiles; tile += gridDim.x * kPredWarps) {
        const int k = tile * 32 + l;
        const bool live = k < a.n_constr;
        float f[kIn];
#pragma unroll
        for (int q = 0; q < kIn; q++) f[q] = 0.0f;
        double t1 = 0.0, scale = 1.0;
        if (live) {
            own_features(a, k, f, t1, scale);
            coupling_features(a, k, f);
            float *fo = a.feat + (size_t)k * kIn;
#pragma unroll
            for (int q = 0; q < kIn; q++) fo[q] = f[q];
            a.t1[k] = t1;
            a.scale[k] = scale;
        }
        if (!infer) continue;  // warp-uniform
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int q0 = 2 * c, q1 = 2 * c + 1;
            sX[w][l][c] = (live && c < kIn / 2)
                              ? pack_bf2((f[q0] - S.mean[q0]) * S.inv[q0], (f[q1] - S.mean[q1]) * S.inv[q1])
                              : 0u;
        }
        __syncwarp();
        mlp_rows32(S, sX[w], sy[w]);
        __syncwarp();
        if (live) lam0[k] = (t1 + ((double)sy[w][l] * (double)S.tscale + (double)S.tmean)) / scale;
        __syncwarp();
    }
}

// The network on m standardised inputs x[m][12] (tests and the C ABI's
// gm_ws_forward): the same tensor-core code as the step's inference.
__global__ void __launch_bounds__(kPredWarps * 32) ws_forward_kernel(int m, const float *__restrict__ x,
                                                                   const float *__restrict__ P, float *y) {
    __shared__ MlpSmem S;
    __shared__ uint32_t sX[kPredWarps][32][8];
    __shared__ float sy[kPredWarps][32];
    load_mlp(P, nullptr, S);
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int n_tiles = (m + 31) / 32;
    for (int tile = blockIdx.x * kPredWarps + w; tile < n_tiles; tile += gridDim.x * kPredWarps) {
        const int k = tile * 32 + l;
        const bool live = k < m;
#pragma unroll
        for (int c = 0; c < 8; c++)
            sX[w][l][c] = (live && c < kIn / 2) ? pack_bf2(x[(size_t)k * kIn + 2 * c], x[(size_t)k * kIn + 2 * c + 1])
                                                : 0u;
        __syncwarp();
        mlp_rows32(S, sX[w], sy[w]);
        __syncwarp();
        if (live) y[k] = sy[w][l];
        __syncwarp();
    }
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

int gm_ws_predict_blocks(int n_constr) {
    const int tiles = (n_constr + 31) / 32;
    return (tiles + kPredWarps - 1) / kPredWarps;
}

void gm_launch_ws_predict(const WsFeatureArgs &a, const float *params, const float *norm, double *lam0, bool infer,
                          cudaStream_t s) {
    if (a.n_constr == 0) return;
    ws_predict_kernel<<<gm_ws_predict_blocks(a.n_constr), kPredWarps * 32, 0, s>>>(a, params, norm, lam0,
                                                                                  infer ? 1 : 0);
}

void gm_launch_ws_forward(int m, const float *x, const float *params, float *y, cudaStream_t s) {
    if (m == 0) return;
    ws_forward_kernel<<<gm_ws_predict_blocks(m), kPredWarps * 32, 0, s>>>(m, x, params, y);
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
