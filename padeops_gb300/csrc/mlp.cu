// Learned SGS closure: an MLP 10 -> 64 -> 64 -> 1 (GELU, softplus output = Cs^2) that
// replaces the dynamic procedure's coefficient in the eddy viscosity nu = Cs^2 Delta^2 |S|.
// It has no counterpart in the reference; it plugs into the slot where getTauSGS calls
// DoStandardDynamicProcedure (sgsmod_igrid.F90:176-183).
//
// Kernels
//  * k_mlp_infer: per point, the features (9 velocity gradients / |S|, ln(1 + Delta/eta))
//    from the nine FP64 gradient arrays, computed in FP32 from an integer FP64 -> FP32
//    conversion (the FP64 pipe is 1/64 of the FP32 rate on this part and the network reads
//    BF16), the MLP on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
//    accumulation; layer-1 accumulators are re-used in registers as layer-2 operands; GELU
//    with the hardware tanh approximation), softplus, and nu = Cs^2 Delta^2 |S| written in
//    FP64.  80 B/point of HBM traffic against ~10 kflop/point.
//  * k_mlp_train_tile: forward and backward of a 128-sample tile in FP32 (shared memory
//    activations), writing the tile's partial gradient; k_mlp_reduce sums the tiles in a
//    fixed order (deterministic); k_mlp_adamw applies AdamW.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "operators.h"
#include "spectral_internal.h"

using namespace pade;

namespace {

constexpr int NIN = 10, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
static_assert(NPARAM == PADE_MLP_NPARAM, "parameter count");
constexpr float C_GELU = 0.7978845608028654f;  // sqrt(2/pi)

__device__ __forceinline__ float gelu(float x) {
    return 0.5f * x * (1.0f + tanhf(C_GELU * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float t = tanhf(C_GELU * (x + 0.044715f * x * x * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * C_GELU * (1.0f + 3.0f * 0.044715f * x * x);
}
// GELU with the hardware tanh approximation (inference, whose activations are then BF16)
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu_fast(float x) {
    return 0.5f * x * (1.0f + tanh_approx(C_GELU * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float softplus(float z) { return z > 20.0f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float sigmoid(float z) { return 0.5f * (1.0f + tanhf(0.5f * z)); }

struct Grad9 {
    const double* p[9];
};

// FP64 -> FP32 on the bits (rounded half up; zero below the FP32 normal range, infinity
// above it): integer work, no FP64 instructions
__device__ __forceinline__ float d2f_bits(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned sign = hi & 0x80000000u;
    if (e < 897) return __uint_as_float(sign);
    if (e > 1150) return __uint_as_float(sign | 0x7F800000u);
    const unsigned b = sign | ((unsigned)(e - 896) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    return __uint_as_float(b + ((lo >> 28) & 1u));
}

// 2^k as a float, -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float((unsigned)(k + 127) << 23); }

// Features of point e in FP32 (the network sees them in BF16): the nine gradients over
// |S| = sqrt(2 S_ij S_ij), and ln(1 + Delta sqrt(|S| / nu)).  The gradients are scaled by a
// power of two near their largest magnitude first, so S_ij S_ij cannot overflow.  Returns |S|.
__device__ __forceinline__ float point_features(const Grad9& d, long e, float delta, float nu, float* x) {
    float g[9];
    float gm = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        g[i] = d2f_bits(d.p[i][e]);
        gm = fmaxf(gm, fabsf(g[i]));
    }
    if (!(gm > 0.0f) || !(gm <= 3.0e38f)) {  // zero gradients (or non-finite ones): zero features
#pragma unroll
        for (int i = 0; i < NIN; i++) x[i] = 0.0f;
        return gm > 0.0f ? gm : 0.0f;
    }
    const int k = (int)((__float_as_uint(gm) >> 23) & 0xFFu) - 127;  // gm in [2^k, 2^(k+1))
    const float sc = pow2f(max(-126, -k));
#pragma unroll
    for (int i = 0; i < 9; i++) g[i] *= sc;
    const float s1 = g[0], s2 = 0.5f * (g[1] + g[3]), s3 = 0.5f * (g[2] + g[6]), s4 = g[4],
                s5 = 0.5f * (g[5] + g[7]), s6 = g[8];
    const float s = s1 * s1 + 2.0f * s2 * s2 + 2.0f * s3 * s3 + s4 * s4 + 2.0f * s5 * s5 + s6 * s6;
    const float ms = sqrtf(2.0f * s);  // |S| * sc
    const float inv = ms > 0.0f ? 1.0f / ms : 0.0f;
#pragma unroll
    for (int i = 0; i < 9; i++) x[i] = g[i] * inv;
    const float mag = ms / sc;
    x[9] = log1pf(delta * sqrtf(mag / nu));
    return mag;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int TILE = 128;  // points per CTA iteration (4 warps x 2 m-tiles of 16)
constexpr int XS = 24;     // bf16 row stride of the feature tile and W1 (bank-conflict padding)
constexpr int W2S = 72;    // bf16 row stride of W2

// weights for inference: W1 (64 x 16, k padded with zeros) and W2 (64 x 64) as BF16,
// biases and w3 in FP32
struct InferWeights {
    __nv_bfloat16 w1[NH * XS];
    __nv_bfloat16 w2[NH * W2S];
    float b1[NH], b2[NH], w3[NH], b3;
    // training range of the features (pade_mlp_set_range); has_range = 0: no range check
    float lo[NIN], hi[NIN];
    int has_range;
};

__global__ void __launch_bounds__(128) k_mlp_infer(Grad9 d, long n, double delta, double nu,
                                                   const InferWeights* __restrict__ wg, double* __restrict__ nu_out,
                                                   float* __restrict__ cs2_out, const MlpFallback fb) {
    __shared__ InferWeights W;
    __shared__ __align__(16) __nv_bfloat16 X[TILE * XS];
    __shared__ float mag[TILE];
    __shared__ unsigned char fbk[TILE];  // point takes the fallback coefficient
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(wg);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&W);
        for (int i = threadIdx.x; i < (int)(sizeof(InferWeights) / 4); i += blockDim.x) dst[i] = src[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const double d2 = delta * delta;
    const float delta_f = (float)delta, nu_f = (float)nu;
    const bool fb_on = fb.lam != nullptr;
    const bool fb_all = fb_on && fb.all && *fb.all != 0;
    for (long base = (long)blockIdx.x * TILE; base < n; base += (long)gridDim.x * TILE) {
        __syncthreads();  // weights loaded / previous tile consumed
        {
            const long e = base + threadIdx.x;
            float x[NIN];
            float m = 0.0f;
            if (e < n) {
                m = point_features(d, e, delta_f, nu_f, x);
            } else {
#pragma unroll
                for (int i = 0; i < NIN; i++) x[i] = 0.0f;
            }
            mag[threadIdx.x] = m;
            // features outside the training range (or the judge's switch) send the point to
            // the fallback coefficient
            bool out = fb_all;
            if (fb_on && W.has_range) {
#pragma unroll
                for (int i = 0; i < NIN; i++) out = out || !(x[i] >= W.lo[i] && x[i] <= W.hi[i]);
            }
            fbk[threadIdx.x] = out ? 1 : 0;
            if (fb.count) {
                const unsigned bal = __ballot_sync(0xffffffffu, out && e < n);
                if ((threadIdx.x & 31) == 0 && bal) atomicAdd(fb.count, (unsigned long long)__popc(bal));
            }
            uint32_t* row = reinterpret_cast<uint32_t*>(X + threadIdx.x * XS);
#pragma unroll
            for (int i = 0; i < 5; i++) row[i] = pack_bf16(x[2 * i], x[2 * i + 1]);
#pragma unroll
            for (int i = 5; i < 8; i++) row[i] = 0u;
        }
        __syncthreads();
#pragma unroll 1
        for (int mt = 0; mt < 2; mt++) {
            const int r0 = warp * 32 + mt * 16;  // first row of this m-tile
            uint32_t a[4];
            const uint32_t* xr0 = reinterpret_cast<const uint32_t*>(X + (r0 + g) * XS);
            const uint32_t* xr1 = reinterpret_cast<const uint32_t*>(X + (r0 + g + 8) * XS);
            a[0] = xr0[t];
            a[1] = xr1[t];
            a[2] = xr0[t + 4];
            a[3] = xr1[t + 4];
            // layer 1: 8 n-tiles of 8 hidden units
            float h[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                h[nt][0] = h[nt][1] = h[nt][2] = h[nt][3] = 0.0f;
                const uint32_t* wr = reinterpret_cast<const uint32_t*>(W.w1 + (nt * 8 + g) * XS);
                mma_bf16(h[nt], a, wr[t], wr[t + 4]);
                const int c = nt * 8 + 2 * t;
                h[nt][0] = gelu_fast(h[nt][0] + W.b1[c]);
                h[nt][1] = gelu_fast(h[nt][1] + W.b1[c + 1]);
                h[nt][2] = gelu_fast(h[nt][2] + W.b1[c]);
                h[nt][3] = gelu_fast(h[nt][3] + W.b1[c + 1]);
            }
            // layer 2: the layer-1 accumulators of n-tiles (2kt, 2kt+1) form the A operand of k-tile kt
            float o[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) o[nt][0] = o[nt][1] = o[nt][2] = o[nt][3] = 0.0f;
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                uint32_t a2[4];
                a2[0] = pack_bf16(h[2 * kt][0], h[2 * kt][1]);
                a2[1] = pack_bf16(h[2 * kt][2], h[2 * kt][3]);
                a2[2] = pack_bf16(h[2 * kt + 1][0], h[2 * kt + 1][1]);
                a2[3] = pack_bf16(h[2 * kt + 1][2], h[2 * kt + 1][3]);
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    const uint32_t* wr = reinterpret_cast<const uint32_t*>(W.w2 + (nt * 8 + g) * W2S + kt * 16);
                    mma_bf16(o[nt], a2, wr[t], wr[t + 4]);
                }
            }
            // layer 3 (FP32): rows g and g+8, this lane's 16 columns, then the 4 lanes of the row
            float z0 = 0.0f, z1 = 0.0f;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c = nt * 8 + 2 * t;
                z0 += W.w3[c] * gelu_fast(o[nt][0] + W.b2[c]) + W.w3[c + 1] * gelu_fast(o[nt][1] + W.b2[c + 1]);
                z1 += W.w3[c] * gelu_fast(o[nt][2] + W.b2[c]) + W.w3[c + 1] * gelu_fast(o[nt][3] + W.b2[c + 1]);
            }
            z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
            z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
            z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
            z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
            if (t == 0) {
#pragma unroll
                for (int hr = 0; hr < 2; hr++) {
                    const int r = r0 + g + 8 * hr;
                    const long e = base + r;
                    if (e < n) {
                        if (fbk[r]) {
                            const double c = fb.lam[e / fb.plane];  // Cs^2 Delta^2 of the fallback
                            nu_out[e] = c * (double)mag[r];
                            if (cs2_out) cs2_out[e] = (float)(c / d2);
                        } else {
                            const float cs2 = softplus((hr ? z1 : z0) + W.b3);
                            nu_out[e] = (double)cs2 * d2 * (double)mag[r];
                            if (cs2_out) cs2_out[e] = cs2;
                        }
                    }
                }
            }
        }
    }
}

// features of n points into X (row-major n x 10, FP32) for building training sets
__global__ void k_mlp_features(Grad9 d, long n, double delta, double nu, float* __restrict__ X) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        float x[NIN];
        point_features(d, e, (float)delta, (float)nu, x);
#pragma unroll
        for (int i = 0; i < NIN; i++) X[e * NIN + i] = x[i];
    }
}

// ---- training (FP32)
constexpr int TT = 128;  // samples per training tile

// dynamic shared memory: X[TT][NIN], Z1[TT][NH], H1[TT][NH], Z2[TT][NH], P[NPARAM], z3[TT], dz3[TT]
__global__ void __launch_bounds__(256) k_mlp_train_tile(const float* __restrict__ X, const float* __restrict__ y,
                                                        int B, const float* __restrict__ prm,
                                                        float* __restrict__ part, float* __restrict__ loss_part) {
    extern __shared__ float sm[];
    float* sx = sm;
    float* z1 = sx + TT * NIN;
    float* h1 = z1 + TT * NH;
    float* z2 = h1 + TT * NH;
    float* P = z2 + TT * NH;
    float* z3 = P + NPARAM;
    float* dz3 = z3 + TT;
    __shared__ float red[8];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int s0 = blockIdx.x * TT;
    const int ns = min(TT, B - s0);
    for (int i = tid; i < NPARAM; i += nth) P[i] = prm[i];
    for (int i = tid; i < TT * NIN; i += nth) sx[i] = (i / NIN) < ns ? X[(long)s0 * NIN + i] : 0.0f;
    __syncthreads();
    const float* W1 = P + OFF_W1;
    const float* b1 = P + OFF_B1;
    const float* W2 = P + OFF_W2;
    const float* b2 = P + OFF_B2;
    const float* w3 = P + OFF_W3;
    // forward
    for (int i = tid; i < TT * NH; i += nth) {
        const int s = i / NH, j = i % NH;
        float a = b1[j];
        for (int k = 0; k < NIN; k++) a += W1[j * NIN + k] * sx[s * NIN + k];
        z1[i] = a;
        h1[i] = gelu(a);
    }
    __syncthreads();
    for (int i = tid; i < TT * NH; i += nth) {
        const int s = i / NH, j = i % NH;
        float a = b2[j];
        for (int k = 0; k < NH; k++) a += W2[j * NH + k] * h1[s * NH + k];
        z2[i] = a;
    }
    __syncthreads();
    float lsum = 0.0f;
    for (int s = tid; s < TT; s += nth) {
        float a = P[OFF_B3];
        for (int j = 0; j < NH; j++) a += w3[j] * gelu(z2[s * NH + j]);
        z3[s] = a;
        if (s < ns) {
            const float r = softplus(a) - y[s0 + s];
            lsum += r * r;
            dz3[s] = (2.0f / (float)B) * r * sigmoid(a);
        } else {
            dz3[s] = 0.0f;
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) red[tid >> 5] = lsum;
    __syncthreads();
    float* g = part + (long)blockIdx.x * NPARAM;
    if (tid == 0) {
        float tsum = 0.0f;
        for (int w = 0; w < nth / 32; w++) tsum += red[w];
        loss_part[blockIdx.x] = tsum;
        float db3 = 0.0f;
        for (int s = 0; s < TT; s++) db3 += dz3[s];
        g[OFF_B3] = db3;
    }
    // dw3 and dZ2 (stored over z2), h2 recomputed
    for (int j = tid; j < NH; j += nth) {
        float a = 0.0f;
        for (int s = 0; s < TT; s++) a += dz3[s] * gelu(z2[s * NH + j]);
        g[OFF_W3 + j] = a;
    }
    __syncthreads();
    for (int i = tid; i < TT * NH; i += nth) {
        const int s = i / NH, j = i % NH;
        z2[i] = dz3[s] * w3[j] * gelu_grad(z2[i]);
    }
    __syncthreads();
    // dW2, db2
    for (int i = tid; i < NH * NH; i += nth) {
        const int j = i / NH, k = i % NH;
        float a = 0.0f;
        for (int s = 0; s < TT; s++) a += z2[s * NH + j] * h1[s * NH + k];
        g[OFF_W2 + i] = a;
    }
    for (int j = tid; j < NH; j += nth) {
        float a = 0.0f;
        for (int s = 0; s < TT; s++) a += z2[s * NH + j];
        g[OFF_B2 + j] = a;
    }
    __syncthreads();
    // dZ1 (over h1)
    for (int i = tid; i < TT * NH; i += nth) {
        const int s = i / NH, k = i % NH;
        float a = 0.0f;
        for (int j = 0; j < NH; j++) a += z2[s * NH + j] * W2[j * NH + k];
        h1[i] = a * gelu_grad(z1[i]);
    }
    __syncthreads();
    for (int i = tid; i < NH * NIN; i += nth) {
        const int j = i / NIN, k = i % NIN;
        float a = 0.0f;
        for (int s = 0; s < TT; s++) a += h1[s * NH + j] * sx[s * NIN + k];
        g[OFF_W1 + i] = a;
    }
    for (int j = tid; j < NH; j += nth) {
        float a = 0.0f;
        for (int s = 0; s < TT; s++) a += h1[s * NH + j];
        g[OFF_B1 + j] = a;
    }
}

__global__ void k_mlp_reduce(const float* __restrict__ part, int tiles, float* __restrict__ grad,
                             const float* __restrict__ loss_part, int B, float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) {
        float a = 0.0f;
        for (int t = 0; t < tiles; t++) a += part[(long)t * NPARAM + p];
        grad[p] = a;
    }
    if (p == 0) {
        float a = 0.0f;
        for (int t = 0; t < tiles; t++) a += loss_part[t];
        *loss = a / (float)B;  // mean squared error
    }
}

__global__ void k_mlp_adamw(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                            float* __restrict__ v, float lr, float wd, float b1, float b2, float eps, float c1,
                            float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.0f - b1) * g;
    const float vv = b2 * v[p] + (1.0f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / c1, vh = vv / c2;
    prm[p] = prm[p] - lr * (mh / (sqrtf(vh) + eps) + wd * prm[p]);
}

__global__ void k_mlp_pack_infer(const float* __restrict__ prm, InferWeights* __restrict__ w) {
    for (int i = threadIdx.x; i < NH * XS; i += blockDim.x) {
        const int j = i / XS, k = i % XS;
        w->w1[i] = __float2bfloat16_rn(k < NIN ? prm[OFF_W1 + j * NIN + k] : 0.0f);
    }
    for (int i = threadIdx.x; i < NH * W2S; i += blockDim.x) {
        const int j = i / W2S, k = i % W2S;
        w->w2[i] = __float2bfloat16_rn(k < NH ? prm[OFF_W2 + j * NH + k] : 0.0f);
    }
    for (int i = threadIdx.x; i < NH; i += blockDim.x) {
        w->b1[i] = prm[OFF_B1 + i];
        w->b2[i] = prm[OFF_B2 + i];
        w->w3[i] = prm[OFF_W3 + i];
    }
    if (threadIdx.x == 0) w->b3 = prm[OFF_B3];
}

}  // namespace

struct pade_mlp_s {
    float* prm = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    float* loss = nullptr;
    float* part = nullptr;
    float* loss_part = nullptr;
    int part_tiles = 0;
    InferWeights* iw = nullptr;
    bool packed = false;
    int has_range = 0;
    int t = 0;  // AdamW step count
};

namespace {

size_t train_smem() { return sizeof(float) * (TT * NIN + 3 * TT * NH + NPARAM + 2 * TT); }

int ensure_part(pade_mlp h, int tiles) {
    if (tiles <= h->part_tiles) return PS_OK;
    cudaFree(h->part);
    cudaFree(h->loss_part);
    h->part = nullptr;
    h->loss_part = nullptr;
    h->part_tiles = 0;
    if (dalloc((void**)&h->part, sizeof(float) * (size_t)tiles * NPARAM) != PS_OK) return PS_ENOMEM;
    if (dalloc((void**)&h->loss_part, sizeof(float) * (size_t)tiles) != PS_OK) return PS_ENOMEM;
    h->part_tiles = tiles;
    return PS_OK;
}

int gradient(pade_mlp h, const float* X, const float* y, int B, cudaStream_t s) {
    const int tiles = (B + TT - 1) / TT;
    int rc = ensure_part(h, tiles);
    if (rc != PS_OK) return rc;
    const size_t smem = train_smem();
    if (cudaFuncSetAttribute(k_mlp_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return PS_ECUDA;
    k_mlp_train_tile<<<tiles, 256, smem, s>>>(X, y, B, h->prm, h->part, h->loss_part);
    k_mlp_reduce<<<(NPARAM + 255) / 256, 256, 0, s>>>(h->part, tiles, h->grad, h->loss_part, B, h->loss);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

}  // namespace

extern "C" {

int pade_mlp_create(pade_mlp* out) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    auto* h = new pade_mlp_s();
    int rc = PS_OK;
    for (float** p : {&h->prm, &h->m, &h->v, &h->grad})
        if (rc == PS_OK) rc = dalloc((void**)p, sizeof(float) * NPARAM);
    if (rc == PS_OK) rc = dalloc((void**)&h->loss, sizeof(float));
    if (rc == PS_OK) rc = dalloc((void**)&h->iw, sizeof(InferWeights));
    if (rc == PS_OK && cudaMemset(h->iw, 0, sizeof(InferWeights)) != cudaSuccess) rc = PS_ECUDA;  // no range
    if (rc == PS_OK) {
        for (float* p : {h->prm, h->m, h->v, h->grad})
            if (cudaMemset(p, 0, sizeof(float) * NPARAM) != cudaSuccess) rc = PS_ECUDA;
    }
    if (rc != PS_OK) {
        pade_mlp_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_mlp_destroy(pade_mlp h) {
    if (!h) return PS_OK;
    for (void* p : {(void*)h->prm, (void*)h->m, (void*)h->v, (void*)h->grad, (void*)h->loss, (void*)h->part,
                    (void*)h->loss_part, (void*)h->iw})
        cudaFree(p);
    delete h;
    return PS_OK;
}

int pade_mlp_set_params(pade_mlp h, const float* host) {
    if (!h || !host) return PS_EINVAL;
    if (cudaMemcpy(h->prm, host, sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess) return PS_ECUDA;
    if (cudaMemset(h->m, 0, sizeof(float) * NPARAM) != cudaSuccess) return PS_ECUDA;
    if (cudaMemset(h->v, 0, sizeof(float) * NPARAM) != cudaSuccess) return PS_ECUDA;
    h->t = 0;
    h->packed = false;
    return PS_OK;
}

int pade_mlp_get_params(pade_mlp h, float* host) {
    if (!h || !host) return PS_EINVAL;
    return cudaMemcpy(host, h->prm, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost) == cudaSuccess ? PS_OK
                                                                                                : PS_ECUDA;
}

int pade_mlp_loss_grad(pade_mlp h, const float* X, const float* y, int B, float* loss, float* grad_host,
                       void* stream) {
    if (!h || B < 1 || !device_ptr(X) || !device_ptr(y)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = gradient(h, X, y, B, s);
    if (rc != PS_OK) return rc;
    if (loss && cudaMemcpyAsync(loss, h->loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return PS_ECUDA;
    if (grad_host && cudaMemcpyAsync(grad_host, h->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s) !=
                         cudaSuccess)
        return PS_ECUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? PS_OK : PS_ECUDA;
}

int pade_mlp_train_step(pade_mlp h, const float* X, const float* y, int B, float lr, float wd, float* loss,
                        void* stream) {
    if (!h || B < 1 || !device_ptr(X) || !device_ptr(y) || !(lr >= 0.0f) || !(wd >= 0.0f)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = gradient(h, X, y, B, s);
    if (rc != PS_OK) return rc;
    h->t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)h->t), c2 = 1.0f - std::pow(b2, (float)h->t);
    k_mlp_adamw<<<(NPARAM + 255) / 256, 256, 0, s>>>(h->prm, h->grad, h->m, h->v, lr, wd, b1, b2, 1e-8f, c1, c2);
    if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
    h->packed = false;
    if (loss) {
        if (cudaMemcpyAsync(loss, h->loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return PS_ECUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return PS_ECUDA;
    }
    return PS_OK;
}

int pade_mlp_features(const double* const* duidxj, long n, double delta, double nu, float* X, void* stream) {
    if (!duidxj || n < 0 || !device_ptr(X) || !(delta > 0) || !(nu > 0)) return PS_EINVAL;
    Grad9 d;
    for (int i = 0; i < 9; i++) {
        if (!device_ptr(duidxj[i])) return PS_EINVAL;
        d.p[i] = duidxj[i];
    }
    if (n == 0) return PS_OK;
    k_mlp_features<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(d, n, delta, nu, X);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

int pade_mlp_set_range(pade_mlp h, const float* lo, const float* hi) {
    if (!h || (!lo) != (!hi)) return PS_EINVAL;
    InferWeights tmp;
    int has = lo ? 1 : 0;
    for (int i = 0; i < NIN; i++) {
        tmp.lo[i] = lo ? lo[i] : 0.0f;
        tmp.hi[i] = hi ? hi[i] : 0.0f;
        if (lo && !(lo[i] <= hi[i])) return PS_EINVAL;
    }
    const size_t off = offsetof(InferWeights, lo);
    const size_t bytes = sizeof(InferWeights) - off;
    tmp.has_range = has;
    if (cudaMemcpy(reinterpret_cast<char*>(h->iw) + off, reinterpret_cast<const char*>(&tmp) + off, bytes,
                   cudaMemcpyHostToDevice) != cudaSuccess)
        return PS_ECUDA;
    h->has_range = has;
    return PS_OK;
}

int pade_mlp_infer_nu(pade_mlp h, const double* const* duidxj, long n, double delta, double nu, double* nu_out,
                      float* cs2_out, void* stream) {
    return mlp_infer_nu_fb(h, duidxj, n, delta, nu, nu_out, cs2_out, MlpFallback{nullptr, 1, nullptr, nullptr},
                           static_cast<cudaStream_t>(stream));
}

}  // extern "C"

int pade::mlp_infer_nu_fb(pade_mlp h, const double* const* duidxj, long n, double delta, double nu, double* nu_out,
                          float* cs2_out, const MlpFallback& fb, cudaStream_t s) {
    if (!h || !duidxj || n < 0 || !device_ptr(nu_out) || !(delta > 0) || !(nu > 0)) return PS_EINVAL;
    if (fb.lam && fb.plane < 1) return PS_EINVAL;
    if (cs2_out && !device_ptr(cs2_out)) return PS_EINVAL;
    Grad9 d;
    for (int i = 0; i < 9; i++) {
        if (!device_ptr(duidxj[i])) return PS_EINVAL;
        d.p[i] = duidxj[i];
    }
    if (!h->packed) {
        k_mlp_pack_infer<<<1, 256, 0, s>>>(h->prm, h->iw);
        if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
        h->packed = true;
    }
    if (n == 0) return PS_OK;
    const long tiles = (n + TILE - 1) / TILE;
    const unsigned g = (unsigned)std::min<long>(tiles, 152L * 8);
    k_mlp_infer<<<g, 128, 0, s>>>(d, n, delta, nu, h->iw, nu_out, cs2_out, fb);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}
