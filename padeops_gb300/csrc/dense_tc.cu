// Dense operator path on the 5th-generation tensor cores (tcgen05, TF32 kind).
//
// A compact operator is a dense matrix D = A^-1 B (n_out x n_in).  Along x the lines are
// contiguous, so applying it to a field is one GEMM per tile of lines:
//     out[line][m] = sum_k D[m][k] f[line][k]       (M = n_out, N = lines, K = n_in)
// with D as the K-major A operand and the field as the K-major B operand.  "3xTF32":
// D = Dh + Dl and f = fh + fl with every part exact in TF32 (11 significant bits), and
// D f ~ Dh fh + Dh fl + Dl fh accumulates in one FP32 accumulator in tensor memory; the
// error is set by the FP32 accumulation (~2^-24 of sum |D||f|) and the dropped Dl fl term
// (~2^-22).  This is the reduced-precision variant of the operator (~1e-6), next to the
// double-float banded path (1e-12).
//
// Per CTA (128 threads): 128 lines; TMEM holds n_out/128 accumulators of 128 x 128 FP32.
// For each K chunk of 32: all threads stage D's rows (hi, lo) and the 128 lines' FP64
// values converted to TF32 pairs (integer split, no FP64 instruction) in shared memory in
// the 128-byte-swizzled K-major layout; one thread issues the tcgen05.mma instructions
// (3 per K=8 step per 128-row half) and commits them to an mbarrier; every wait on it is
// bounded (a timeout sets the error word, frees TMEM and returns).  The epilogue reads the
// accumulators with tcgen05.ld (a warp per 32 rows) and stores FP64, coalesced along x.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "capi_internal.h"
#include "dfmath.cuh"
#include "engine.h"
#include "operators.h"
#include "spectral_internal.h"

using namespace pade;

namespace {

constexpr int NT = 128;             // lines per CTA (MMA N)
constexpr int KC = 32;              // K per chunk: 32 TF32 = one 128-byte swizzle row
constexpr unsigned kWaitLimit = 1u << 22;

__device__ unsigned g_dense_err;    // 1: an mbarrier wait timed out

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;            // descriptor version
    d |= (uint64_t)2 << 61;            // SWIZZLE_128B
    return d;
}

// instruction descriptor: D FP32, A/B TF32, both K-major, M = 128, N = NT
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NT >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// FP64 -> (hi, lo) TF32 pair with integer instructions and FP32 arithmetic
__device__ __forceinline__ void split_tf32(double v, float& h, float& l, unsigned& bad) {
    const dfv d = df_from_double(v, bad);
    h = tf32_rna(d.h);
    l = tf32_rna(__fadd_rn(__fsub_rn(d.h, h), d.l));
}

// byte offset of 16-byte chunk `ch` of row `r` in a 128-byte-swizzled K-major tile
__device__ __forceinline__ uint32_t swz(int r, int ch) { return (uint32_t)(r * 128 + ((ch ^ (r & 7)) << 4)); }

__global__ void __launch_bounds__(128) k_dense_x_tf32(const double* __restrict__ f, double* __restrict__ out,
                                                      const float* __restrict__ Dh, const float* __restrict__ Dl,
                                                      int nin, int nout, long nlines, unsigned* __restrict__ rangeflag) {
    extern __shared__ uint8_t dsm_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ int abort_flag;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* Ah = base;
    uint8_t* Al = Ah + (size_t)nout * 128;
    uint8_t* Bh = Al + (size_t)nout * 128;
    uint8_t* Bl = Bh + (size_t)NT * 128;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = (uint32_t)nout;  // nout/128 accumulators of NT = 128 columns
    const long l0 = (long)blockIdx.x * NT;
    if (warp == 0) tmem_alloc(&tslot, ncols);
    if (tid == 0) {
        mbar_init(&mbar, 1);
        fence_barrier_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    unsigned bad = 0;
    unsigned phase = 0;
    const int nchunks = nin / KC;
    for (int c = 0; c < nchunks; c++) {
        // D rows, hi and lo: nout rows x 8 chunks of 16 B each
        for (int idx = tid; idx < nout * 8 * 2; idx += blockDim.x) {
            const int which = idx / (nout * 8), rem = idx % (nout * 8);
            const int r = rem >> 3, ch = rem & 7;
            const float4 v = *reinterpret_cast<const float4*>((which ? Dl : Dh) + (size_t)r * nin + c * KC + ch * 4);
            *reinterpret_cast<float4*>((which ? Al : Ah) + swz(r, ch)) = v;
        }
        // 128 lines x 16 double2 of this chunk
        for (int idx = tid; idx < NT * 16; idx += blockDim.x) {
            const int ln = idx >> 4, q = idx & 15;
            const long line = l0 + ln;
            double2 v = make_double2(0.0, 0.0);
            if (line < nlines) v = *reinterpret_cast<const double2*>(f + line * nin + c * KC + 2 * q);
            float h0, l0f, h1, l1f;
            split_tf32(v.x, h0, l0f, bad);
            split_tf32(v.y, h1, l1f, bad);
            const uint32_t off = swz(ln, q >> 1) + ((q & 1) << 3);
            *reinterpret_cast<float2*>(Bh + off) = make_float2(h0, h1);
            *reinterpret_cast<float2*>(Bl + off) = make_float2(l0f, l1f);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            for (int mh = 0; mh < nout / 128; mh++) {
                const uint32_t d = tmem + (uint32_t)(mh * NT);
                for (int kk = 0; kk < KC / 8; kk++) {
                    const uint64_t ah = desc_sw128(su32(Ah + mh * 128 * 128 + kk * 32));
                    const uint64_t al = desc_sw128(su32(Al + mh * 128 * 128 + kk * 32));
                    const uint64_t bh = desc_sw128(su32(Bh + kk * 32));
                    const uint64_t bl = desc_sw128(su32(Bl + kk * 32));
                    mma_tf32(d, ah, bh, kIdesc, (c > 0 || kk > 0) ? 1u : 0u);
                    mma_tf32(d, ah, bl, kIdesc, 1u);
                    mma_tf32(d, al, bh, kIdesc, 1u);
                }
            }
            mma_commit(&mbar);
        }
        // the MMAs of this chunk finish before its shared memory is rewritten
        unsigned it = 0;
        while (!mbar_try_wait(&mbar, phase)) {
            if (++it > kWaitLimit) {
                atomicOr(&g_dense_err, 1u);
                abort_flag = 1;
                break;
            }
        }
        phase ^= 1u;
        __syncthreads();
        if (abort_flag) break;
    }
    if (bad) atomicOr(rangeflag, 1u);
    tc_fence_after();
    if (!abort_flag) {
        for (int mh = 0; mh < nout / 128; mh++) {
            const int row = mh * 128 + warp * 32 + lane;  // output point along x
            for (int cb = 0; cb < NT / 16; cb++) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mh * NT + cb * 16), r);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const long line = l0 + cb * 16 + j;
                    if (line < nlines) out[line * nout + row] = float_bits_to_double(__uint_as_float(r[j]));
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

struct DenseMat {
    float* Dh = nullptr;
    float* Dl = nullptr;
    int nin = 0, nout = 0;
};

std::mutex g_dense_mu;
std::map<std::pair<const void*, int>, DenseMat> g_dense;  // (handle, plan key) -> split matrix

float tf32_host(double x) {
    float f = (float)x;
    uint32_t b;
    std::memcpy(&b, &f, 4);
    if ((b & 0x7F800000u) != 0x7F800000u) b = (b + 0x1000u) & 0xFFFFE000u;
    std::memcpy(&f, &b, 4);
    return f;
}

int dense_for(pade_op h, int opcode, int bc1, int bcn, DenseMat** out) {
    const int key = plan_key(opcode, bc1, bcn);
    std::lock_guard<std::mutex> lock(g_dense_mu);
    auto it = g_dense.find({h, key});
    if (it != g_dense.end()) {
        *out = &it->second;
        return PS_OK;
    }
    auto e = h->plan_err.find(key);
    if (e != h->plan_err.end()) return e->second;
    auto p = h->plans.find(key);
    if (p == h->plans.end()) return PS_EINVAL;
    const OpDef& d = p->second->host().def;
    std::vector<double> M;
    int rc = dense_operator(d, M);
    if (rc != PS_OK) return rc;
    DenseMat dm;
    dm.nin = d.m;
    dm.nout = d.nout;
    std::vector<float> hi(M.size()), lo(M.size());
    for (size_t i = 0; i < M.size(); i++) {
        hi[i] = tf32_host(M[i]);
        lo[i] = tf32_host(M[i] - (double)hi[i]);
    }
    if ((rc = upload(&dm.Dh, hi)) != PS_OK) return rc;
    if ((rc = upload(&dm.Dl, lo)) != PS_OK) {
        cudaFree(dm.Dh);
        return rc;
    }
    auto ins = g_dense.emplace(std::make_pair((const void*)h, key), dm);
    *out = &ins.first->second;
    return PS_OK;
}

}  // namespace

namespace pade {
// frees the dense matrices of a handle (called by pade_destroy)
void dense_release(const void* h) {
    std::lock_guard<std::mutex> lock(g_dense_mu);
    for (auto it = g_dense.begin(); it != g_dense.end();) {
        if (it->first.first == h) {
            cudaFree(it->second.Dh);
            cudaFree(it->second.Dl);
            it = g_dense.erase(it);
        } else {
            ++it;
        }
    }
}
}  // namespace pade

extern "C" {

int pade_dense_apply(pade_op h, int opcode, int dir, const double* f, double* out, int na, int nb, int bc1, int bcn,
                     void* stream) {
    if (!h || na < 1 || nb < 1) return PS_EINVAL;
    if (dir != 1) return PS_ENOTSUP;
    if (!device_ptr(f) || !device_ptr(out)) return PS_EINVAL;
    if (h->family == F_CD10 || h->family == F_CF90 || h->family == F_GAUSS) {
        if (!bc_valid(bc1) || !bc_valid(bcn)) return PS_EREF_BC;
        if (h->periodic) bc1 = bcn = 0;
    } else {
        bc1 = bcn = 0;
    }
    DenseMat* D = nullptr;
    int rc = dense_for(h, opcode, bc1, bcn, &D);
    if (rc != PS_OK) return rc;
    // TMEM columns = nout must be a power of two (128, 256 or 512)
    if (D->nin % KC != 0 || (D->nout != 128 && D->nout != 256 && D->nout != 512) || D->nin > 4096)
        return PS_ENOTSUP;
    if ((reinterpret_cast<uintptr_t>(f) & 15) || (reinterpret_cast<uintptr_t>(out) & 7)) return PS_EINVAL;
    const long nlines = (long)na * nb;
    const size_t smem = 1024 + (size_t)D->nout * 128 * 2 + (size_t)NT * 128 * 2;
    if (cudaFuncSetAttribute(k_dense_x_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PS_ECUDA;
    const long blocks = (nlines + NT - 1) / NT;
    k_dense_x_tf32<<<(unsigned)blocks, 128, smem, static_cast<cudaStream_t>(stream)>>>(
        f, out, D->Dh, D->Dl, D->nin, D->nout, nlines, h->status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

int pade_dense_status(int* timed_out) {
    if (!timed_out) return PS_EINVAL;
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, g_dense_err, sizeof(unsigned)) != cudaSuccess) return PS_ECUDA;
    *timed_out = (int)v;
    if (v) {
        const unsigned z = 0;
        if (cudaMemcpyToSymbol(g_dense_err, &z, sizeof(unsigned)) != cudaSuccess) return PS_ECUDA;
    }
    return PS_OK;
}

}  // extern "C"
