// Learned SGS closure: an MLP 10 -> 64 -> 64 -> 1 (GELU, softplus output = Cs^2) that
// replaces the dynamic procedure's coefficient in the eddy viscosity nu = Cs^2 Delta^2 |S|.
// It has no counterpart in the reference; it plugs into the slot where getTauSGS calls
// DoStandardDynamicProcedure (sgsmod_igrid.F90:176-183).
//
// Kernels
//  * k_mlp_infer_tc: per point, the features (9 velocity gradients / |S|, ln(1 + Delta/eta))
//    from the nine FP64 gradient arrays, computed in FP32 from an integer FP64 -> FP32
//    conversion (the FP64 pipe is 1/64 of the FP32 rate on this part and the network reads
//    BF16); the three layers as tcgen05.mma (BF16 operands from shared memory, FP32
//    accumulators in tensor memory, biases folded into the MMAs); GELU on BF16 pairs between
//    the layers; softplus; nu = Cs^2 Delta^2 |S| written in FP64.  84 B/point of HBM traffic
//    (72 read, 8 written, plus 4 when Cs^2 is kept) against ~10 kflop/point.
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
#include "dfmath.cuh"
#include "operators.h"
#include "spectral_internal.h"
#include "tc_common.cuh"

using namespace pade;
using namespace pade::tc;

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

// Features of one point in FP32 (the network sees them in BF16) from its nine FP64
// gradients g: the gradients over |S| = sqrt(2 S_ij S_ij), and ln(1 + Delta sqrt(|S| / nu)).
// The gradients are scaled by a power of two near their largest magnitude first, so
// S_ij S_ij cannot overflow.  Returns |S|.
__device__ __forceinline__ float point_features(const double* gd, float delta, float nu, float* x) {
    float g[9];
    float gm = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        g[i] = d2f_bits(gd[i]);
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
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // lo in the low half (lower address)
    return *reinterpret_cast<const uint32_t*>(&v);
}

// ---- inference on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in TMEM)
//
// A CTA of 128 threads takes tiles of 128 points; thread r owns point r of the tile, which
// is row r of every MMA's A operand and lane r of tensor memory.  Per tile:
//   features -> X (128 x 16 BF16: 10 features, then 1, 1 at K = 10, 11 to carry the biases)
//   D  = X W1ext^T                         (1 MMA, N = 64)      -> GELU -> H (128 x 64 BF16)
//   D  = H W2^T + X B2ext^T                (4 + 1 MMAs, N = 64) -> GELU -> H
//   D  = H W3ext^T + X B3ext^T             (4 + 1 MMAs, N = 16) -> z = column 0
//   Cs^2 = softplus(z), nu = Cs^2 Delta^2 |S|.
// Each bias is split into two BF16 parts (value and remainder, ~2^-17 relative) that
// multiply the two 1-features, so the tensor cores add it.  The three D share 64 TMEM
// columns (each is read out before the next MMA overwrites it).  GELU runs on BF16 pairs
// (packed FMA and the hardware tanh approximation on two values per instruction), the
// activations being BF16 anyway.  The next tile's gradients are loaded while the current
// one goes through the network; four CTAs share an SM.  Thread 0 waits on the MMA barrier
// (bounded: a timeout sets g_mlp_err, the CTA frees its tensor memory and returns) while
// the other threads sleep in the CTA barrier that follows.
constexpr int TILE = 128;              // points per tile (MMA M)
constexpr uint32_t kTmemCols = 64;     // one FP32 accumulator of N <= 64
constexpr int kInferCtasPerSm = 4;
constexpr unsigned kMlpWaitLimit = 1u << 22;

// Inference weights: pre-swizzled shared-memory images (K-major rows of 128 bytes) of the
// MMAs' B operands, then the features' training range.
//   wsmall, 64 rows:  K 0..15  W1 row n (K 0..9), b1[n] as BF16 value + remainder (K 10, 11)
//                     K 16..31 b2[n] the same way (K 26, 27)
//                     K 32..47 rows 0..15: b3 (row 0, K 42, 43), zeros elsewhere
//   w2, 64 rows:      W2[n][k]
//   w3, 16 rows:      row 0 = w3, rows 1..15 zero (N = 16 is the smallest M = 128 shape)
struct TcWeights {
    uint8_t wsmall[64 * 128];
    uint8_t w2[64 * 128];
    uint8_t w3[16 * 128];
    // training range of the features (pade_mlp_set_range); has_range = 0: no range check
    float lo[NIN], hi[NIN];
    int has_range;
};
constexpr size_t kImgBytes = 64 * 128 + 64 * 128 + 16 * 128;
static_assert(offsetof(TcWeights, lo) == kImgBytes, "image layout");
static_assert(kImgBytes % 1024 == 0, "tiles after the images stay 1024-byte aligned");
constexpr size_t kInferSmem = 1024 + kImgBytes + 2 * (size_t)TILE * 128;  // alignment slack, images, X, H

__device__ unsigned g_mlp_err;  // 1: a tensor-core wait timed out

__device__ __forceinline__ uint32_t bf2_u32(__nv_bfloat162 v) { return *reinterpret_cast<const uint32_t*>(&v); }
__device__ __forceinline__ __nv_bfloat162 u32_bf2(uint32_t u) { return *reinterpret_cast<const __nv_bfloat162*>(&u); }

// GELU (tanh form) of two BF16 values, in BF16 arithmetic
__device__ __forceinline__ uint32_t gelu_bf2(uint32_t xu) {
    const __nv_bfloat162 x = u32_bf2(xu);
    const __nv_bfloat162 k1 = __float2bfloat162_rn(C_GELU * 0.044715f), k0 = __float2bfloat162_rn(C_GELU);
    const __nv_bfloat162 half = __float2bfloat162_rn(0.5f);
    const __nv_bfloat162 u = __hmul2(x, __hfma2(__hmul2(x, x), k1, k0));  // sqrt(2/pi) (x + 0.044715 x^3)
    uint32_t t;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(bf2_u32(u)));
    return bf2_u32(__hmul2(x, __hfma2(u32_bf2(t), half, half)));
}

// D (64 FP32 columns of this thread's lane) -> GELU -> row r of the BF16 tile H
__device__ __forceinline__ void gelu_row(uint32_t trow, uint8_t* H, int r) {
#pragma unroll
    for (int cb = 0; cb < 4; cb++) {
        uint32_t v[16];
        tmem_ld16(trow + (uint32_t)(cb * 16), v);
        uint32_t w[8];
#pragma unroll
        for (int i = 0; i < 8; i++) w[i] = gelu_bf2(pack_bf16(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1])));
        *reinterpret_cast<uint4*>(H + swz(r, 2 * cb)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4*>(H + swz(r, 2 * cb + 1)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

__device__ __forceinline__ bool mlp_wait(uint64_t* bar, unsigned phase) {
    unsigned it = 0;
    while (!mbar_try_wait(bar, phase))
        if (++it > kMlpWaitLimit) return false;
    return true;
}

__global__ void __launch_bounds__(TILE, kInferCtasPerSm)
    k_mlp_infer_tc(Grad9 d, long n, double delta, double nu, const TcWeights* __restrict__ wg,
                   double* __restrict__ nu_out, float* __restrict__ cs2_out, const MlpFallback fb) {
    extern __shared__ uint8_t sm_raw[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    __shared__ float lo_s[NIN], hi_s[NIN];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* Wsm = base;
    uint8_t* W2 = base + 64 * 128;
    uint8_t* W3 = base + 2 * 64 * 128;
    uint8_t* X = base + kImgBytes;
    uint8_t* H = X + TILE * 128;
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        const uint4* src = reinterpret_cast<const uint4*>(wg);
        uint4* dst = reinterpret_cast<uint4*>(base);
        for (int i = tid; i < (int)(kImgBytes / 16); i += TILE) dst[i] = __ldg(src + i);
    }
    if (tid < NIN) {
        lo_s[tid] = wg->lo[tid];
        hi_s[tid] = wg->hi[tid];
    }
    const bool has_range = wg->has_range != 0;
    if (warp == 0) tmem_alloc(&tslot, kTmemCols);
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    fence_async_smem();  // the weight images, written by the threads, are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
    constexpr uint32_t id64 = idesc_bf16_m128(64), id16 = idesc_bf16_m128(16);
    const uint32_t ONES = 0x3F803F80u;  // two BF16 1.0
    const float delta_f = (float)delta, nu_f = (float)nu, d2f = (float)(delta * delta);
    const double d2 = delta * delta;
    const bool fb_on = fb.lam != nullptr;
    const bool fb_all = fb_on && fb.all && *fb.all != 0;
    const long ntiles = (n + TILE - 1) / TILE;
    unsigned ph = 0;
    int tout = 0;  // this thread's wait timed out

    double g[9];
    auto load = [&](long t) {
        const long e = t * TILE + tid;
        const bool ok = t < ntiles && e < n;
#pragma unroll
        for (int i = 0; i < 9; i++) g[i] = ok ? __ldg(d.p[i] + e) : 0.0;
    };
    load(blockIdx.x);
    for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long e = tile * TILE + tid;
        float x[NIN];
        float mag = 0.0f;
        if (e < n) {
            mag = point_features(g, delta_f, nu_f, x);
        } else {
#pragma unroll
            for (int i = 0; i < NIN; i++) x[i] = 0.0f;
        }
        // features outside the training range (or the judge's switch) send the point to the
        // fallback coefficient
        bool out = fb_all;
        if (fb_on && has_range) {
#pragma unroll
            for (int i = 0; i < NIN; i++) out = out || !(x[i] >= lo_s[i] && x[i] <= hi_s[i]);
        }
        if (fb.count) {
            const unsigned bal = __ballot_sync(0xffffffffu, out && e < n);
            if ((tid & 31) == 0 && bal) atomicAdd(fb.count, (unsigned long long)__popc(bal));
        }
        *reinterpret_cast<uint4*>(X + swz(tid, 0)) =
            make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
        *reinterpret_cast<uint4*>(X + swz(tid, 1)) = make_uint4(pack_bf16(x[8], x[9]), ONES, 0u, 0u);
        load(tile + gridDim.x);  // the next tile's gradients load while this one runs
        fence_async_smem();
        tc_fence_before();
        if (__syncthreads_or(tout)) break;
        // layer 1
        if (tid == 0) {
            tc_fence_after();
            mma_f16(tmem, desc_sw128(su32(X)), desc_sw128(su32(Wsm)), id64, 0u);
            mma_commit(&bar);
        }
        if (tid == 0 && !mlp_wait(&bar, ph)) tout = 1;  // one waiter; the others sleep in the barrier
        ph ^= 1u;
        if (__syncthreads_or(tout)) break;
        tc_fence_after();
        gelu_row(trow, H, tid);
        fence_async_smem();
        tc_fence_before();
        if (__syncthreads_or(tout)) break;
        // layer 2 (+ b2 from the 1-features)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_f16(tmem, desc_sw128(su32(H + kk * 32)), desc_sw128(su32(W2 + kk * 32)), id64, kk > 0 ? 1u : 0u);
            mma_f16(tmem, desc_sw128(su32(X)), desc_sw128(su32(Wsm + 32)), id64, 1u);
            mma_commit(&bar);
        }
        if (tid == 0 && !mlp_wait(&bar, ph)) tout = 1;  // one waiter; the others sleep in the barrier
        ph ^= 1u;
        if (__syncthreads_or(tout)) break;
        tc_fence_after();
        gelu_row(trow, H, tid);
        fence_async_smem();
        tc_fence_before();
        if (__syncthreads_or(tout)) break;
        // layer 3 (+ b3)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_f16(tmem, desc_sw128(su32(H + kk * 32)), desc_sw128(su32(W3 + kk * 32)), id16, kk > 0 ? 1u : 0u);
            mma_f16(tmem, desc_sw128(su32(X)), desc_sw128(su32(Wsm + 64)), id16, 1u);
            mma_commit(&bar);
        }
        if (tid == 0 && !mlp_wait(&bar, ph)) tout = 1;  // one waiter; the others sleep in the barrier
        ph ^= 1u;
        if (__syncthreads_or(tout)) break;
        tc_fence_after();
        const float z = __uint_as_float(tmem_ld1(trow));
        tc_fence_before();
        if (e < n) {
            if (out) {
                const double c = fb.lam[e / fb.plane];  // Cs^2 Delta^2 of the fallback
                nu_out[e] = c * (double)mag;
                if (cs2_out) cs2_out[e] = (float)(c / d2);
            } else {
                const float cs2 = softplus(z);
                nu_out[e] = float_bits_to_double(cs2 * d2f * mag);  // exact FP32 -> FP64 on the bits
                if (cs2_out) cs2_out[e] = cs2;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (tout) atomicOr(&g_mlp_err, 1u);
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// features of n points into X (row-major n x 10, FP32) for building training sets
__global__ void k_mlp_features(Grad9 d, long n, double delta, double nu, float* __restrict__ X) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double gd[9];
#pragma unroll
        for (int i = 0; i < 9; i++) gd[i] = d.p[i][e];
        float x[NIN];
        point_features(gd, (float)delta, (float)nu, x);
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

// BF16 value v at (row, K index k) of a 128-byte-swizzled K-major image
__device__ __forceinline__ void put_bf16(uint8_t* img, int row, int k, float v) {
    *reinterpret_cast<__nv_bfloat16*>(img + swz(row, k >> 3) + ((k & 7) << 1)) = __float2bfloat16_rn(v);
}

// bias b as a BF16 value and its BF16 remainder at K = k, k + 1 of row n
__device__ __forceinline__ void put_bias(uint8_t* img, int row, int k, float b) {
    const float h = __bfloat162float(__float2bfloat16_rn(b));
    put_bf16(img, row, k, h);
    put_bf16(img, row, k + 1, b - h);
}

// the parameters (FP32, flat) -> the inference images (one CTA)
__global__ void k_mlp_pack_tc(const float* __restrict__ prm, TcWeights* __restrict__ w) {
    uint32_t* z = reinterpret_cast<uint32_t*>(w);
    for (int i = threadIdx.x; i < (int)(kImgBytes / 4); i += blockDim.x) z[i] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < NH * NIN; i += blockDim.x) put_bf16(w->wsmall, i / NIN, i % NIN, prm[OFF_W1 + i]);
    for (int i = threadIdx.x; i < NH * NH; i += blockDim.x) put_bf16(w->w2, i / NH, i % NH, prm[OFF_W2 + i]);
    for (int i = threadIdx.x; i < NH; i += blockDim.x) {
        put_bias(w->wsmall, i, 10, prm[OFF_B1 + i]);
        put_bias(w->wsmall, i, 26, prm[OFF_B2 + i]);
        put_bf16(w->w3, 0, i, prm[OFF_W3 + i]);
    }
    if (threadIdx.x == 0) put_bias(w->wsmall, 0, 42, prm[OFF_B3]);
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
    TcWeights* iw = nullptr;
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
    if (rc == PS_OK) rc = dalloc((void**)&h->iw, sizeof(TcWeights));
    if (rc == PS_OK && cudaMemset(h->iw, 0, sizeof(TcWeights)) != cudaSuccess) rc = PS_ECUDA;  // no range
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
    TcWeights tmp;
    int has = lo ? 1 : 0;
    for (int i = 0; i < NIN; i++) {
        tmp.lo[i] = lo ? lo[i] : 0.0f;
        tmp.hi[i] = hi ? hi[i] : 0.0f;
        if (lo && !(lo[i] <= hi[i])) return PS_EINVAL;
    }
    const size_t off = offsetof(TcWeights, lo);
    const size_t bytes = sizeof(TcWeights) - off;
    tmp.has_range = has;
    if (cudaMemcpy(reinterpret_cast<char*>(h->iw) + off, reinterpret_cast<const char*>(&tmp) + off, bytes,
                   cudaMemcpyHostToDevice) != cudaSuccess)
        return PS_ECUDA;
    h->has_range = has;
    return PS_OK;
}

int pade_mlp_status(int* timed_out) {
    if (!timed_out) return PS_EINVAL;
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, g_mlp_err, sizeof(unsigned)) != cudaSuccess) return PS_ECUDA;
    *timed_out = (int)v;
    if (v) {
        const unsigned z = 0;
        if (cudaMemcpyToSymbol(g_mlp_err, &z, sizeof(unsigned)) != cudaSuccess) return PS_ECUDA;
    }
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
        k_mlp_pack_tc<<<1, 256, 0, s>>>(h->prm, h->iw);
        if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
        h->packed = true;
    }
    if (n == 0) return PS_OK;
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
            return PS_ECUDA;
    }
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem) !=
            cudaSuccess)
            return PS_ECUDA;
        attr = true;
    }
    const long tiles = (n + TILE - 1) / TILE;
    const unsigned g = (unsigned)std::min<long>(tiles, (long)nsm * kInferCtasPerSm);
    k_mlp_infer_tc<<<g, TILE, kInferSmem, s>>>(d, n, delta, nu, h->iw, nu_out, cs2_out, fb);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}
