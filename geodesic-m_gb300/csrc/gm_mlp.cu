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
// in the tensor cores' own summation order), fused with the coupling pass:
// two kernels per SHAKE solve.  Training runs its forward pass, the backward
// products and the tile's weight-gradient sums on the tensor cores too (the
// deltas as a BF16 high part plus a BF16 remainder), treats the BF16
// roundings of the forward pass as the identity, and sums the per-block
// gradient partials in block order, so training is run-to-run identical.
#include <cuda_bf16.h>

#include "gm_internal.cuh"

namespace {

constexpr int kIn = GM_WS_IN, kH = GM_WS_H, kNP = GM_WS_NPAR;
constexpr int kTile = GM_WS_TILE;

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

// The constraint's own features 0-7, its t1 and its scale 2 (1/m_i + 1/m_j).
// FP64 only where it cancels: the coordinate differences, |r_trial|^2 - d0^2
// and r_trial . r_ref; each is then rounded once to FP32, and the ratios,
// t1 = (|r_trial|^2 - d0^2) / (r_trial . r_ref) and d0 are correctly rounded
// FP32 operations (the network's inputs are FP32, and t1 only seeds the
// solve, which then iterates to the unchanged tolerance).
__device__ __forceinline__ void own_features(const WsFeatureArgs &a, int k, float *f, double &t1, double &scale) {
    const int i = a.constr_i[k], j = a.constr_j[k], n = a.n_atoms;
    const double d0sq = a.constr_dsq[k];
    const double rx = __dsub_rn(a.dref[i], a.dref[j]), ry = __dsub_rn(a.dref[n + i], a.dref[n + j]),
                 rz = __dsub_rn(a.dref[2 * n + i], a.dref[2 * n + j]);
    const double tx = __dsub_rn(a.pos[i], a.pos[j]), ty = __dsub_rn(a.pos[n + i], a.pos[n + j]),
                 tz = __dsub_rn(a.pos[2 * n + i], a.pos[2 * n + j]);
    const float num = (float)__dsub_rn(dot3(tx, ty, tz, tx, ty, tz), d0sq);
    const float dr = (float)dot3(tx, ty, tz, rx, ry, rz);
    const float d0f = (float)d0sq;
    const float t1f = dr == 0.0f ? 0.0f : __fdiv_rn(num, dr);
    t1 = (double)t1f;
    scale = __dmul_rn(2.0, __dadd_rn(a.inv_mass[i], a.inv_mass[j]));
    f[0] = __fdiv_rn(num, d0f);
    f[1] = __fdiv_rn(dr, d0f);
    f[2] = __fsqrt_rn(d0f);
    f[3] = (float)a.inv_mass[i];
    f[4] = (float)a.inv_mass[j];
    f[5] = (float)(a.atom_cstart[i + 1] - a.atom_cstart[i]);
    f[6] = (float)(a.atom_cstart[j + 1] - a.atom_cstart[j]);
    f[7] = t1f;
}

// Coupling to the other constraints on the constraint's two atoms (features
// 8-11) in FP32, atom i's constraints then atom j's, each ascending; masses
// and the neighbours' t1 enter rounded to FP32.  Reads every constraint's
// (reference direction, t1) from the first pass and its FP32 inverse-mass sum
// w (two independent loads per neighbour).
__device__ __forceinline__ void coupling_features(const WsFeatureArgs &a, int k, float *f) {
    const int ends[2] = {a.constr_i[k], a.constr_j[k]};
    const float wk = a.w[k];
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
            const float wl = a.w[l];
            const float coup = __fmul_rn(__fmul_rn(__fdiv_rn(inv_a, wk), cs), __fmul_rn(sk, sl));
            const float tl = ul.w;
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
// of the row (c < 6; 6 and 7 are zero); y goes to sy[row].  The two m16
// tiles go through each layer together, so every step of the dependent
// chain (layer-1 MMAs, SiLU, layer-2 MMAs, layer 3) has both tiles'
// independent work in flight; each row's arithmetic is the same as one tile
// at a time.
__device__ __forceinline__ void mlp_rows32(const MlpSmem &S, const uint32_t (*sX)[8], float *sy) {
    const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
    uint32_t a[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        a[mt][0] = sX[r0][t];
        a[mt][1] = sX[r1][t];
        a[mt][2] = sX[r0][t + 4];
        a[mt][3] = sX[r1][t + 4];
    }
    float z1[2][8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float c0 = S.b1[8 * j + 2 * t], c1 = S.b1[8 * j + 2 * t + 1];
        const uint2 bw = S.b1f[j][l];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            z1[mt][j][0] = c0; z1[mt][j][1] = c1; z1[mt][j][2] = c0; z1[mt][j][3] = c1;
            mma_bf16(z1[mt][j], a[mt][0], a[mt][1], a[mt][2], a[mt][3], bw);
        }
    }
    uint32_t A2[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            A2[mt][kk][0] = pack_bf2(silu(z1[mt][2 * kk][0]), silu(z1[mt][2 * kk][1]));
            A2[mt][kk][1] = pack_bf2(silu(z1[mt][2 * kk][2]), silu(z1[mt][2 * kk][3]));
            A2[mt][kk][2] = pack_bf2(silu(z1[mt][2 * kk + 1][0]), silu(z1[mt][2 * kk + 1][1]));
            A2[mt][kk][3] = pack_bf2(silu(z1[mt][2 * kk + 1][2]), silu(z1[mt][2 * kk + 1][3]));
        }
    float z2[2][8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float c0 = S.b2[8 * j + 2 * t], c1 = S.b2[8 * j + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            z2[mt][j][0] = c0; z2[mt][j][1] = c1; z2[mt][j][2] = c0; z2[mt][j][3] = c1;
        }
    }
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint2 bw = S.b2f[kk][j][l];
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
                mma_bf16(z2[mt][j], A2[mt][kk][0], A2[mt][kk][1], A2[mt][kk][2], A2[mt][kk][3], bw);
        }
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = 8 * j + 2 * t;
            y0 = fmaf(bf(silu(z2[mt][j][0])), S.w3[c], y0);
            y0 = fmaf(bf(silu(z2[mt][j][1])), S.w3[c + 1], y0);
            y1 = fmaf(bf(silu(z2[mt][j][2])), S.w3[c], y1);
            y1 = fmaf(bf(silu(z2[mt][j][3])), S.w3[c + 1], y1);
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

// The network's parameters and input standardisation in the shared-memory
// layout of the inference (fragment order), once per change of the
// parameters, so that each inference block copies them instead of packing.
__global__ void __launch_bounds__(256) ws_pack_kernel(const float *P, const float *norm, MlpSmem *out) {
    load_mlp(P, norm, *out);
}

// Pass 1, one thread per constraint: its own features 0-7, t1, the scale and
// the reference bond direction, each computed once (the FP64 part).
__global__ void __launch_bounds__(256) ws_own_kernel(WsFeatureArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_constr) return;
    float f[8];
    double t1, scale;
    own_features(a, k, f, t1, scale);
    float *fo = a.feat + (size_t)k * kIn;
#pragma unroll
    for (int q = 0; q < 8; q++) fo[q] = f[q];
    a.t1[k] = t1;
    a.scale[k] = scale;
    float ux, uy, uz;
    ref_unit(a, k, ux, uy, uz);
    a.unit[k] = make_float4(ux, uy, uz, f[7]);
}

// Pass 2: each lane takes one constraint's coupling features 8-11 (written
// out for the recorder), and with `infer` the warp runs the network on its 32
// constraints and writes the predicted multipliers
// lam0 = (t1 + y t_scale + t_mean) / scale.
__global__ void __launch_bounds__(kPredWarps * 32) ws_predict_kernel(WsFeatureArgs a,
                                                                   const MlpSmem *__restrict__ packed,
                                                                   double *lam0, int infer) {
    __shared__ MlpSmem S;
    __shared__ uint32_t sX[kPredWarps][32][8];
    __shared__ float sy[kPredWarps][32];
    if (infer) {
        // the weights already in fragment order (ws_pack_kernel): a copy
        const uint2 *src = reinterpret_cast<const uint2 *>(packed);
        uint2 *dst = reinterpret_cast<uint2 *>(&S);
        for (int i = threadIdx.x; i < (int)(sizeof(MlpSmem) / sizeof(uint2)); i += blockDim.x) dst[i] = src[i];
    }
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
            float *fo = a.feat + (size_t)k * kIn;
#pragma unroll
            for (int q = 0; q < 8; q++) f[q] = fo[q];
            coupling_features(a, k, f);
#pragma unroll
            for (int q = 8; q < kIn; q++) fo[q] = f[q];
            t1 = a.t1[k];
            scale = a.scale[k];
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

// ---- training on the tensor cores -------------------------------------
//
// One block of 4 warps per tile of 128 samples (warp w: samples 32 w ..
// 32 w + 31, two m16 tiles).  Per sample: the forward pass of mlp_rows32,
// keeping z1, the BF16 layer-1 activations (as layer 2's A fragments) and z2;
// the residual y - t; delta2 = dy w3 SiLU'(z2); delta_a1 = delta2 W2^T as
// MMAs (delta2 split into a BF16 high part and a BF16 remainder, two MMAs
// each, so the operand rounding stays near FP32); delta1 = delta_a1
// SiLU'(z1).  Then the tile's parameter gradients as MMAs whose K dimension
// is the 128 samples, read from shared memory: dW2 = A1^T delta2 (one m16
// tile of W2's rows per warp) and dW1 = X^T delta1 (two n-tiles per warp),
// again with the deltas as high + remainder.  Bias and w3 gradients and the
// loss are FP32 sums over the samples in ascending order.  Every sum has a
// fixed order, so training is run-to-run identical.

struct GradSmem {
    MlpSmem m;                          // forward fragments, biases, w3
    uint2 b2t[4][8][32];                // W2^T fragments (B[k = o][n = q] = W2[q][o])
    uint32_t x[kTile][8];               // inputs, BF16 pairs
    __nv_bfloat16 a1[kTile][kH];        // layer-1 activations (BF16, exact)
    __nv_bfloat16 a2[kTile][kH];        // layer-2 activations
    __nv_bfloat16 d2h[kTile][kH], d2l[kTile][kH];  // delta2, high part and remainder
    __nv_bfloat16 d1h[kTile][kH], d1l[kTile][kH];  // delta1
    float dy[kTile], loss[kTile];
};

__device__ __forceinline__ float sig_d(float z) {
    // d SiLU / dz = g (1 + z (1 - g)), g = sigmoid(z)
    const float g = sigmoid(z);
    return g * (1.0f + z * (1.0f - g));
}

__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(kTile) ws_grad_mma_kernel(long long n, const float *__restrict__ feat,
                                                            const float *__restrict__ tt,
                                                            const float *__restrict__ norm, int standardized,
                                                            const float *__restrict__ P, unsigned long long seed,
                                                            long long iter, long long n_valid, float inv_batch,
                                                            float *__restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smraw[];
    GradSmem &G = *reinterpret_cast<GradSmem *>(smraw);
    load_mlp(P, nullptr, G.m);
    for (int e = threadIdx.x; e < 4 * 8 * 32; e += blockDim.x) {
        const int kk = e >> 8, j = (e >> 5) & 7, l = e & 31, g = l >> 2, t = l & 3;
        const int nq = 8 * j + g, k0 = 16 * kk + 2 * t;  // B[k = o][n = q] = W2[q][o]
        const float *W2 = P + GM_WS_OFF_W2;
        G.b2t[kk][j][l] = make_uint2(pack_bf2(W2[nq * kH + k0], W2[nq * kH + k0 + 1]),
                                     pack_bf2(W2[nq * kH + k0 + 8], W2[nq * kH + k0 + 9]));
    }
    // the tile's samples and their standardised inputs
    {
        const int s = threadIdx.x;
        const long long row = (long long)blockIdx.x * kTile + s;
        long long sample;
        if (iter < 0) sample = row < n ? row : n - 1;
        else sample = (long long)(mix64(seed ^ mix64((unsigned long long)iter * 0x100000001B3ull +
                                                     (unsigned long long)row)) % (unsigned long long)n);
        float xv[kIn];
        for (int f = 0; f < kIn; f++) {
            const float v = feat[sample * kIn + f];
            xv[f] = standardized ? v : (v - norm[f]) / norm[kIn + f];
        }
        for (int c = 0; c < 8; c++) G.x[s][c] = c < kIn / 2 ? pack_bf2(xv[2 * c], xv[2 * c + 1]) : 0u;
        const float tv = standardized ? tt[sample] : (tt[sample] - norm[24]) / norm[25];
        G.dy[s] = tv;  // the target, replaced by dy below
        G.loss[s] = row < n_valid ? 1.0f : 0.0f;  // validity, replaced by the squared residual
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, g = l >> 2, t = l & 3;
#pragma unroll 1
    for (int mt = 0; mt < 2; mt++) {
        const int r0 = 32 * w + 16 * mt + g, r1 = r0 + 8;
        const uint32_t a0 = G.x[r0][t], a1 = G.x[r1][t], a2 = G.x[r0][t + 4], a3 = G.x[r1][t + 4];
        float z1[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float c0 = G.m.b1[8 * j + 2 * t], c1 = G.m.b1[8 * j + 2 * t + 1];
            z1[j][0] = c0; z1[j][1] = c1; z1[j][2] = c0; z1[j][3] = c1;
            mma_bf16(z1[j], a0, a1, a2, a3, G.m.b1f[j][l]);
        }
        uint32_t A2[4][4];
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            A2[kk][0] = pack_bf2(silu(z1[2 * kk][0]), silu(z1[2 * kk][1]));
            A2[kk][1] = pack_bf2(silu(z1[2 * kk][2]), silu(z1[2 * kk][3]));
            A2[kk][2] = pack_bf2(silu(z1[2 * kk + 1][0]), silu(z1[2 * kk + 1][1]));
            A2[kk][3] = pack_bf2(silu(z1[2 * kk + 1][2]), silu(z1[2 * kk + 1][3]));
        }
        // layer-1 activations to shared memory (rows r0, r1; columns of n-tile j: 8 j + 2 t, + 1)
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int c = 16 * kk + 8 * h + 2 * t;
                *reinterpret_cast<uint32_t *>(&G.a1[r0][c]) = A2[kk][2 * h];
                *reinterpret_cast<uint32_t *>(&G.a1[r1][c]) = A2[kk][2 * h + 1];
            }
        float z2[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float c0 = G.m.b2[8 * j + 2 * t], c1 = G.m.b2[8 * j + 2 * t + 1];
            z2[j][0] = c0; z2[j][1] = c1; z2[j][2] = c0; z2[j][3] = c1;
        }
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
#pragma unroll
            for (int j = 0; j < 8; j++) mma_bf16(z2[j], A2[kk][0], A2[kk][1], A2[kk][2], A2[kk][3], G.m.b2f[kk][j][l]);
        float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = 8 * j + 2 * t;
            const float v0 = bf(silu(z2[j][0])), v1 = bf(silu(z2[j][1])), v2 = bf(silu(z2[j][2])),
                        v3 = bf(silu(z2[j][3]));
            G.a2[r0][c] = __float2bfloat16_rn(v0);
            G.a2[r0][c + 1] = __float2bfloat16_rn(v1);
            G.a2[r1][c] = __float2bfloat16_rn(v2);
            G.a2[r1][c + 1] = __float2bfloat16_rn(v3);
            y0 = fmaf(v0, G.m.w3[c], y0);
            y0 = fmaf(v1, G.m.w3[c + 1], y0);
            y1 = fmaf(v2, G.m.w3[c], y1);
            y1 = fmaf(v3, G.m.w3[c + 1], y1);
        }
        y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
        y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
        const float res0 = G.m.b3 + y0 - G.dy[r0], res1 = G.m.b3 + y1 - G.dy[r1];
        const bool v0ok = G.loss[r0] != 0.0f, v1ok = G.loss[r1] != 0.0f;
        const float dy0 = v0ok ? 2.0f * res0 * inv_batch : 0.0f, dy1 = v1ok ? 2.0f * res1 * inv_batch : 0.0f;
        __syncwarp();
        if (t == 0) {
            G.dy[r0] = dy0;
            G.dy[r1] = dy1;
            G.loss[r0] = v0ok ? res0 * res0 : 0.0f;
            G.loss[r1] = v1ok ? res1 * res1 : 0.0f;
        }
        // delta2 = dy w3 SiLU'(z2), as high + remainder, to shared memory and
        // as A fragments of delta_a1 = delta2 W2^T
        uint32_t Dh[4][4], Dl[4][4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = 8 * j + 2 * t;
            float d[4];
            d[0] = dy0 * G.m.w3[c] * sig_d(z2[j][0]);
            d[1] = dy0 * G.m.w3[c + 1] * sig_d(z2[j][1]);
            d[2] = dy1 * G.m.w3[c] * sig_d(z2[j][2]);
            d[3] = dy1 * G.m.w3[c + 1] * sig_d(z2[j][3]);
            __nv_bfloat16 hi[4], lo[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                hi[q] = __float2bfloat16_rn(d[q]);
                lo[q] = __float2bfloat16_rn(d[q] - __bfloat162float(hi[q]));
            }
            G.d2h[r0][c] = hi[0]; G.d2h[r0][c + 1] = hi[1]; G.d2h[r1][c] = hi[2]; G.d2h[r1][c + 1] = hi[3];
            G.d2l[r0][c] = lo[0]; G.d2l[r0][c + 1] = lo[1]; G.d2l[r1][c] = lo[2]; G.d2l[r1][c + 1] = lo[3];
            const int kk = j >> 1, h = j & 1;
            Dh[kk][2 * h] = pack_raw(hi[0], hi[1]);
            Dh[kk][2 * h + 1] = pack_raw(hi[2], hi[3]);
            Dl[kk][2 * h] = pack_raw(lo[0], lo[1]);
            Dl[kk][2 * h + 1] = pack_raw(lo[2], lo[3]);
        }
        float da[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) da[j][0] = da[j][1] = da[j][2] = da[j][3] = 0.0f;
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
#pragma unroll
            for (int j = 0; j < 8; j++) {
                mma_bf16(da[j], Dh[kk][0], Dh[kk][1], Dh[kk][2], Dh[kk][3], G.b2t[kk][j][l]);
                mma_bf16(da[j], Dl[kk][0], Dl[kk][1], Dl[kk][2], Dl[kk][3], G.b2t[kk][j][l]);
            }
        // delta1 = delta_a1 SiLU'(z1)
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = 8 * j + 2 * t;
            float d[4];
            d[0] = da[j][0] * sig_d(z1[j][0]);
            d[1] = da[j][1] * sig_d(z1[j][1]);
            d[2] = da[j][2] * sig_d(z1[j][2]);
            d[3] = da[j][3] * sig_d(z1[j][3]);
            const int rr[4] = {r0, r0, r1, r1}, cc[4] = {c, c + 1, c, c + 1};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const __nv_bfloat16 hi = __float2bfloat16_rn(d[q]);
                G.d1h[rr[q]][cc[q]] = hi;
                G.d1l[rr[q]][cc[q]] = __float2bfloat16_rn(d[q] - __bfloat162float(hi));
            }
        }
    }
    __syncthreads();
    float *out = partial + (size_t)blockIdx.x * (kNP + 1);
    // dW2[q][o] = sum_s A1[s][q] delta2[s][o]: warp w takes rows q in [16 w, 16 w + 16)
    {
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
        const int q0 = 16 * w + g, q1 = q0 + 8;
#pragma unroll 1
        for (int kk = 0; kk < kTile / 16; kk++) {
            const int s0 = 16 * kk + 2 * t;
            const uint32_t A0 = pack_raw(G.a1[s0][q0], G.a1[s0 + 1][q0]);
            const uint32_t A1 = pack_raw(G.a1[s0][q1], G.a1[s0 + 1][q1]);
            const uint32_t A2r = pack_raw(G.a1[s0 + 8][q0], G.a1[s0 + 9][q0]);
            const uint32_t A3 = pack_raw(G.a1[s0 + 8][q1], G.a1[s0 + 9][q1]);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int o = 8 * j + g;
                const uint2 bh = make_uint2(pack_raw(G.d2h[s0][o], G.d2h[s0 + 1][o]),
                                            pack_raw(G.d2h[s0 + 8][o], G.d2h[s0 + 9][o]));
                const uint2 bl = make_uint2(pack_raw(G.d2l[s0][o], G.d2l[s0 + 1][o]),
                                            pack_raw(G.d2l[s0 + 8][o], G.d2l[s0 + 9][o]));
                mma_bf16(acc[j], A0, A1, A2r, A3, bh);
                mma_bf16(acc[j], A0, A1, A2r, A3, bl);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int o = 8 * j + 2 * t;
            out[GM_WS_OFF_W2 + q0 * kH + o] = acc[j][0];
            out[GM_WS_OFF_W2 + q0 * kH + o + 1] = acc[j][1];
            out[GM_WS_OFF_W2 + q1 * kH + o] = acc[j][2];
            out[GM_WS_OFF_W2 + q1 * kH + o + 1] = acc[j][3];
        }
    }
    // dW1[f][o] = sum_s X[s][f] delta1[s][o]: one m16 tile of f (rows 12-15
    // are the zero padding), warp w takes n-tiles 2 w and 2 w + 1
    {
        float acc[2][4];
#pragma unroll
        for (int jj = 0; jj < 2; jj++) acc[jj][0] = acc[jj][1] = acc[jj][2] = acc[jj][3] = 0.0f;
        const __nv_bfloat16 *xs = reinterpret_cast<const __nv_bfloat16 *>(G.x);  // [s][16]
#pragma unroll 1
        for (int kk = 0; kk < kTile / 16; kk++) {
            const int s0 = 16 * kk + 2 * t;
            auto X = [&](int sv, int f) { return xs[sv * 16 + f]; };
            const uint32_t A0 = pack_raw(X(s0, g), X(s0 + 1, g));
            const uint32_t A1 = pack_raw(X(s0, g + 8), X(s0 + 1, g + 8));
            const uint32_t A2r = pack_raw(X(s0 + 8, g), X(s0 + 9, g));
            const uint32_t A3 = pack_raw(X(s0 + 8, g + 8), X(s0 + 9, g + 8));
#pragma unroll
            for (int jj = 0; jj < 2; jj++) {
                const int o = 8 * (2 * w + jj) + g;
                const uint2 bh = make_uint2(pack_raw(G.d1h[s0][o], G.d1h[s0 + 1][o]),
                                            pack_raw(G.d1h[s0 + 8][o], G.d1h[s0 + 9][o]));
                const uint2 bl = make_uint2(pack_raw(G.d1l[s0][o], G.d1l[s0 + 1][o]),
                                            pack_raw(G.d1l[s0 + 8][o], G.d1l[s0 + 9][o]));
                mma_bf16(acc[jj], A0, A1, A2r, A3, bh);
                mma_bf16(acc[jj], A0, A1, A2r, A3, bl);
            }
        }
#pragma unroll
        for (int jj = 0; jj < 2; jj++) {
            const int o = 8 * (2 * w + jj) + 2 * t;
            if (g < kIn) {
                out[GM_WS_OFF_W1 + g * kH + o] = acc[jj][0];
                out[GM_WS_OFF_W1 + g * kH + o + 1] = acc[jj][1];
            }
            if (g + 8 < kIn) {
                out[GM_WS_OFF_W1 + (g + 8) * kH + o] = acc[jj][2];
                out[GM_WS_OFF_W1 + (g + 8) * kH + o + 1] = acc[jj][3];
            }
        }
    }
    // biases, w3 and the loss: FP32 sums over the samples, ascending
    {
        const int s = threadIdx.x;
        if (s < kH) {
            float g1 = 0.0f, g3 = 0.0f;
            for (int q = 0; q < kTile; q++) {
                g1 += __bfloat162float(G.d1h[q][s]) + __bfloat162float(G.d1l[q][s]);
                g3 = fmaf(__bfloat162float(G.a2[q][s]), G.dy[q], g3);
            }
            out[GM_WS_OFF_B1 + s] = g1;
            out[GM_WS_OFF_W3 + s] = g3;
        } else {
            const int o = s - kH;
            float g2 = 0.0f;
            for (int q = 0; q < kTile; q++) g2 += __bfloat162float(G.d2h[q][o]) + __bfloat162float(G.d2l[q][o]);
            out[GM_WS_OFF_B2 + o] = g2;
            if (o == 0) {
                float gb = 0.0f, lsum = 0.0f;
                for (int q = 0; q < kTile; q++) { gb += G.dy[q]; lsum += G.loss[q]; }
                out[GM_WS_OFF_B3] = gb;
                out[kNP] = lsum;
            }
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

void gm_launch_ws_predict(const WsFeatureArgs &a, const void *packed, double *lam0, bool infer, cudaStream_t s) {
    if (a.n_constr == 0) return;
    ws_own_kernel<<<(a.n_constr + 255) / 256, 256, 0, s>>>(a);
    ws_predict_kernel<<<gm_ws_predict_blocks(a.n_constr), kPredWarps * 32, 0, s>>>(
        a, static_cast<const MlpSmem *>(packed), lam0, infer ? 1 : 0);
}

size_t gm_ws_packed_bytes() { return sizeof(MlpSmem); }

void gm_launch_ws_pack(const float *params, const float *norm, void *packed, cudaStream_t s) {
    ws_pack_kernel<<<1, 256, 0, s>>>(params, norm, static_cast<MlpSmem *>(packed));
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
        cudaFuncSetAttribute(ws_grad_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem));
        attr = true;
    }
    const float inv_batch = 1.0f / (float)(n_valid < (long long)blocks * kTile ? n_valid : (long long)blocks * kTile);
    ws_grad_mma_kernel<<<blocks, kTile, sizeof(GradSmem), s>>>(n, feat, t, norm, standardized ? 1 : 0, params, seed,
                                                                iter, n_valid, inv_batch, partial);
}

void gm_launch_ws_update(int blocks, const float *partial, float *params, float *m, float *v, float lr, float b1,
                         float b2, float eps, int t, float *grad_out, cudaStream_t s) {
    ws_update_kernel<<<(kNP + 1 + 255) / 256, 256, 0, s>>>(blocks, partial, params, m, v, lr, b1, b2, eps, t,
                                                            grad_out);
}
