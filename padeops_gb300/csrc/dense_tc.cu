// Dense operator path on the 5th-generation tensor cores (tcgen05, TF32 kind).
//
// A compact operator is a dense matrix D = A^-1 B (n_out x n_in).  Applying it to the lines
// of a field is one GEMM per tile of 128 lines:
//     out[line][m] = sum_k D[m][k] f[line][k]       (M = n_out, N = lines, K = n_in)
// with D as the K-major A operand and the lines as the K-major B operand, whichever the
// direction: the staging writes the lines K-major into shared memory (x lines are read
// along K, y and z lines across lines), so one tensor-core schedule serves all three.  "3xTF32":
// D = Dh + Dl and f = fh + fl with every part exact in TF32 (11 significant bits), and
// D f ~ Dh fh + Dh fl + Dl fh accumulates in one FP32 accumulator in tensor memory; the
// error is set by the FP32 accumulation (~2^-24 of sum |D||f|) and the dropped Dl fl term
// (~2^-22).  This is the reduced-precision variant of the operator (~1e-6), next to the
// double-float banded path (1e-12).
//
// Per CTA (512 threads): 128 lines; TMEM holds n_out/128 accumulators of 128 x 128 FP32.
// For each K chunk of 32: D's rows (hi, lo) arrive by cp.async and the 128 lines' FP64
// values, converted to TF32 pairs (integer split, no FP64 instruction), are stored by the
// threads, both in the 128-byte-swizzled K-major layout of shared memory; one thread
// issues the tcgen05.mma instructions (3 per K=8 step per 128-row half) and commits them
// to the stage's mbarrier; with two stages the next chunk loads while the tensor cores
// work.  Every wait is bounded (a timeout sets the error word, frees TMEM and returns).  The epilogue reads the
// accumulators with tcgen05.ld (a warp per 32 rows) and stores FP64, coalesced along x.
#include <cuda_runtime.h>

#include <algorithm>
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
#include "tc_common.cuh"

using namespace pade;
using namespace pade::tc;

namespace {

constexpr int NT = 128;             // lines per CTA (MMA N)
constexpr int KC = 32;              // K per chunk: 32 TF32 = one 128-byte swizzle row
constexpr unsigned kWaitLimit = 1u << 22;

__device__ unsigned g_dense_err;    // 1: an mbarrier wait timed out

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
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


__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* g) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// bounded wait for an mbarrier phase; false (and the error word set) on timeout
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned phase) {
    unsigned it = 0;
    while (!mbar_try_wait(bar, phase)) {
        if (++it > kWaitLimit) {
            atomicOr(&g_dense_err, 1u);
            return false;
        }
    }
    return true;
}

constexpr int NTHR = 512;            // threads per CTA: 16 warps share the staging work
constexpr int FPT = NT * 16 / NTHR;  // double2 of the line tile per thread and chunk

// STAGES = 2: the loads of chunk c+1 (D by cp.async, the lines through registers) overlap
// the tensor-core work of chunk c; STAGES = 1 when two stages do not fit in shared memory.
// XL: lines contiguous (x lines, fp == 1): a thread loads double2 along K of one line and
// the epilogue stores rows of consecutive points.  Otherwise (y, z lines) consecutive
// threads take consecutive lines for each K index and the epilogue stores each thread's
// 16 lines at the lines' own addresses.  Line l = a + na*b sits at a*fa + b*fb (input)
// and a*oa + b*ob (output), point p at p*fp / p*op.
template <int STAGES, bool XL>
__global__ void __launch_bounds__(NTHR) k_dense_tf32(const double* __restrict__ f, double* __restrict__ out,
                                                    const float* __restrict__ Dh, const float* __restrict__ Dl,
                                                    int nin, int nout, const LineSet ls,
                                                    unsigned* __restrict__ rangeflag, int resid) {
    const long nlines = ls.nlines;
    extern __shared__ uint8_t dsm_raw[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t tslot;
    __shared__ int abort_flag;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~(uintptr_t)1023);
    const size_t a_bytes = (size_t)nout * 128, b_bytes = (size_t)NT * 128;
    const size_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = (uint32_t)nout;  // nout/128 accumulators of NT = 128 columns
    const long l0 = (long)blockIdx.x * NT;
    if (warp == 0) tmem_alloc(&tslot, ncols);
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_barrier_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    unsigned bad = 0;
    unsigned ph[2] = {0u, 0u};
    const int nchunks = nin / KC;

    auto stage_ptr = [&](int s) { return base + (size_t)s * stage_bytes; };
    // D rows of chunk c (hi then lo) into stage s, 16-byte asynchronous copies
    auto issue_D = [&](int c, int s) {
        uint8_t* Ah = stage_ptr(s);
        uint8_t* Al = Ah + a_bytes;
        for (int idx = tid; idx < nout * 16; idx += blockDim.x) {
            const int which = idx / (nout * 8), rem = idx % (nout * 8);
            const int r = rem >> 3, ch = rem & 7;
            const float* src = (which ? Dl : Dh) + (size_t)r * nin + c * KC + ch * 4;
            cp_async16(su32((which ? Al : Ah) + swz(r, ch)), src);
        }
        cp_async_commit();
    };
    auto load_F = [&](int c, double2* R) {
#pragma unroll
        for (int i = 0; i < FPT; i++) {
            const int idx = tid + i * NTHR;
            if (XL) {
                const int ln = idx >> 4, q = idx & 15;
                const long line = l0 + ln;
                R[i] = line < nlines ? __ldg(reinterpret_cast<const double2*>(f + line * ls.fa + c * KC + 2 * q))
                                     : make_double2(0.0, 0.0);
            } else {
                // two K indices per entry: k = 2*(idx / NT) + {0, 1}, line ln = idx % NT
                const int ln = idx % NT, k = 2 * (idx / NT);
                const long line = l0 + ln;
                if (line < nlines) {
                    const long a = line % ls.na, b = line / ls.na;
                    const double* src = f + a * ls.fa + b * ls.fb + (long)(c * KC + k) * ls.fp;
                    R[i] = make_double2(__ldg(src), __ldg(src + ls.fp));
                } else {
                    R[i] = make_double2(0.0, 0.0);
                }
            }
        }
    };
    auto store_F = [&](int s, const double2* R) {
        uint8_t* Bh = stage_ptr(s) + 2 * a_bytes;
        uint8_t* Bl = Bh + b_bytes;
#pragma unroll
        for (int i = 0; i < FPT; i++) {
            const int idx = tid + i * NTHR;
            float h0, lo0, h1, lo1;
            split_tf32(R[i].x, h0, lo0, bad);
            split_tf32(R[i].y, h1, lo1, bad);
            if (XL) {
                const int ln = idx >> 4, q = idx & 15;
                const uint32_t off = swz(ln, q >> 1) + ((q & 1) << 3);
                *reinterpret_cast<float2*>(Bh + off) = make_float2(h0, h1);
                *reinterpret_cast<float2*>(Bl + off) = make_float2(lo0, lo1);
            } else {
                const int ln = idx % NT, k = 2 * (idx / NT);  // k even: both values in one 16-byte chunk
                const uint32_t off = swz(ln, k >> 2) + ((k & 3) << 2);
                *reinterpret_cast<float2*>(Bh + off) = make_float2(h0, h1);
                *reinterpret_cast<float2*>(Bl + off) = make_float2(lo0, lo1);
            }
        }
    };

    double2 R[FPT];
    issue_D(0, 0);
    load_F(0, R);
    store_F(0, R);
    for (int c = 0; c < nchunks; c++) {
        const int s = STAGES == 2 ? (c & 1) : 0;
        cp_async_wait_all();
        fence_async_smem();
        __syncthreads();
        if (abort_flag) break;
        if (tid == 0) {
            tc_fence_after();
            uint8_t* Ah = stage_ptr(s);
            uint8_t* Al = Ah + a_bytes;
            uint8_t* Bh = Al + a_bytes;
            uint8_t* Bl = Bh + b_bytes;
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
            mma_commit(&mbar[s]);
        }
        if (c + 1 < nchunks) {
            const int s2 = STAGES == 2 ? (s ^ 1) : 0;
            load_F(c + 1, R);  // global loads in flight while the tensor cores work
            // stage s2 was last read by chunk c-1 (two stages) or chunk c (one stage)
            if (STAGES == 1 || c >= 1) {
                if (!mbar_wait_bounded(&mbar[s2], ph[s2])) abort_flag = 1;
                ph[s2] ^= 1u;
            }
            if (!abort_flag) {
                issue_D(c + 1, s2);
                store_F(s2, R);
            }
        }
    }
    // the last one or two commits
    if (!abort_flag) {
        if (STAGES == 2 && nchunks >= 2) {
            const int sp = (nchunks - 2) & 1;
            if (!mbar_wait_bounded(&mbar[sp], ph[sp])) abort_flag = 1;
            ph[sp] ^= 1u;
        }
        const int sl = STAGES == 2 ? ((nchunks - 1) & 1) : 0;
        if (!abort_flag && !mbar_wait_bounded(&mbar[sl], ph[sl])) abort_flag = 1;
    }
    __syncthreads();
    if (bad) atomicOr(rangeflag, 1u);
    tc_fence_after();
    if (!abort_flag) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (the lanes it may access) and the
        // column blocks cb = w / 4, w / 4 + 4, ...
        const int lq = warp & 3;
        for (int mh = 0; mh < nout / 128; mh++) {
            const int row = mh * 128 + lq * 32 + lane;  // output point along x
            for (int cb = warp >> 2; cb < NT / 16; cb += NTHR / 128) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(mh * NT + cb * 16), r);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const long line = l0 + cb * 16 + j;
                    if (line >= nlines) continue;
                    const double v = float_bits_to_double(__uint_as_float(r[j]));
                    if (XL) {
                        out[line * ls.oa + row] = resid ? __ldg(f + line * ls.fa + row) - v : v;
                    } else {
                        const long a = line % ls.na, b = line / ls.na;
                        out[a * ls.oa + b * ls.ob + (long)row * ls.op] =
                            resid ? __ldg(f + a * ls.fa + b * ls.fb + (long)row * ls.fp) - v : v;
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ------------------------------------------------------------------------------------
// k_dense_ws: persistent, warp-specialised pipeline (n_out <= 256, two stages)
// ------------------------------------------------------------------------------------
// Each CTA walks one stream of (tile, K chunk) items over its 128-line tiles.
//  * Warps 0..15 produce: they keep the lines of the next two items in flight in
//    registers while they split the current one into TF32 pairs and store it into the
//    stage's B tile, then arrive on the stage's "full" barrier.
//  * Warp 16 (one lane) issues the MMAs: it waits for "full", issues the chunk's MMAs and
//    commits them to the stage's "empty" barrier; after a tile's last chunk it commits to
//    the accumulator's "acc full" barrier.
//  * Warp 17 (one lane) loads D: as soon as "empty" releases a stage it fills the stage's
//    A tiles with the item's D chunk, one bulk copy of D's pre-swizzled image completing
//    on the stage's "full" barrier by transaction bytes.  (Issuing MMAs can block the
//    issuing thread, so the copies have a thread of their own.)
//  * Warps 18..21 (one per TMEM lane quadrant) read the accumulators (tcgen05.ld), store
//    FP64 and arrive on "acc empty"; two TMEM accumulators let a tile's epilogue run while
//    the next tile computes.
// Waits are bounded: a timeout sets the error word and the abort flag, every role runs out
// its loops without waiting, the loader waits (bounded) for the copies it issued, and
// TMEM is freed.
constexpr int WS_PROD_WARPS = 16;
constexpr int WS_EPI_WARPS = 4;  // one per TMEM lane quadrant
constexpr int WS_STAGES = 2;
constexpr int WS_FPT = NT * 16 / (WS_PROD_WARPS * 32);  // double2 per producer thread and item
constexpr uint32_t kBulkPiece = 16384;                  // bytes per bulk copy
// warps: producers 0..15, MMA issuer 16, D loader 17, epilogue 18..21
constexpr int WS_THREADS = (WS_PROD_WARPS + 2 + WS_EPI_WARPS) * 32;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}

// RESID: the matrix is I - D of a filter in residual form, and the epilogue outputs f minus
// the accumulator (a variant of its own, so the plain operators keep their epilogue as is)
template <bool XL, bool RESID>
__global__ void __launch_bounds__(WS_THREADS, 1)
    k_dense_ws(const double* __restrict__ f, double* __restrict__ out, const float* __restrict__ Dimg, int nin,
               int nout, const LineSet ls, long ntiles, unsigned* __restrict__ rangeflag) {
    constexpr int NACC = 2;  // accumulator buffers: the epilogue of a tile overlaps the next
    const long nlines = ls.nlines;
    extern __shared__ uint8_t dsm_raw[];
    __shared__ uint64_t full[WS_STAGES], empty[WS_STAGES], accf[NACC], acce[NACC];
    __shared__ uint32_t tslot;
    __shared__ volatile int abort_flag;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t a_bytes = (uint32_t)nout * 128, b_bytes = (uint32_t)NT * 128;
    const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool producer = warp < WS_PROD_WARPS;
    const bool control = warp == WS_PROD_WARPS && lane == 0;     // MMA issuer
    const bool loader = warp == WS_PROD_WARPS + 1 && lane == 0;  // D copies
    const bool epi_warp = warp > WS_PROD_WARPS + 1;
    const uint32_t ncols = (uint32_t)(nout * NACC);
    const int nchunks = nin / KC;
    if (warp == 0) tmem_alloc(&tslot, ncols);
    if (tid == 0) {
        for (int s = 0; s < WS_STAGES; s++) {
            mbar_init(&full[s], WS_PROD_WARPS + 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC; b++) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], WS_EPI_WARPS);
        }
        fence_barrier_init();
        abort_flag = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tslot;
    unsigned bad = 0;
    auto stage_ptr = [&](int s) { return base + (size_t)s * stage_bytes; };
    auto wait = [&](uint64_t* bar, unsigned parity) {
        if (abort_flag) return;
        if (!mbar_wait_bounded(bar, parity)) abort_flag = 1;
    };
    const long my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const long nitems = my_tiles * nchunks;
    auto tile_of = [&](long it) { return blockIdx.x + it * gridDim.x; };
    long issued[WS_STAGES] = {-1, -1};  // loader: last item whose D copy went to each stage

    // x lines: R[i] holds two consecutive K values of one line (16-byte loads).  y, z lines:
    // thread t takes line t / 4 and K = 4 kq + t % 4 for kq = 2i, 2i + 1, so that a warp's
    // stores cover 8 lines x 4 K values of one 16-byte chunk: all 32 banks of the swizzled
    // tile (consecutive lines on a K index would share 8 banks); its loads read 64-byte row
    // segments of 8 consecutive lines.
    auto load_F = [&](long l0, int c, double2* R) {
#pragma unroll
        for (int i = 0; i < WS_FPT; i++) {
            if (XL) {
                const int idx = tid + i * WS_PROD_WARPS * 32;
                const int ln = idx >> 4, q = idx & 15;
                const long line = l0 + ln;
                R[i] = line < nlines ? __ldg(reinterpret_cast<const double2*>(f + line * ls.fa + c * KC + 2 * q))
                                     : make_double2(0.0, 0.0);
            } else {
                const int ln = tid >> 2, k0 = 8 * i + (tid & 3);
                const long line = l0 + ln;
                if (line < nlines) {
                    const long a = line % ls.na, b = line / ls.na;
                    const double* src = f + a * ls.fa + b * ls.fb + (long)(c * KC + k0) * ls.fp;
                    R[i] = make_double2(__ldg(src), __ldg(src + 4 * ls.fp));
                } else {
                    R[i] = make_double2(0.0, 0.0);
                }
            }
        }
    };
    auto load_item = [&](long q, double2* R) {
        if (q < nitems) load_F(tile_of(q / nchunks) * NT, (int)(q % nchunks), R);
    };
    auto store_F = [&](int s, const double2* R) {
        uint8_t* Bh = stage_ptr(s) + 2 * a_bytes;
        uint8_t* Bl = Bh + b_bytes;
#pragma unroll
        for (int i = 0; i < WS_FPT; i++) {
            float h0, lo0, h1, lo1;
            split_tf32(R[i].x, h0, lo0, bad);
            split_tf32(R[i].y, h1, lo1, bad);
            if (XL) {
                const int idx = tid + i * WS_PROD_WARPS * 32;
                const int ln = idx >> 4, q = idx & 15;
                const uint32_t off = swz(ln, q >> 1) + ((q & 1) << 3);
                *reinterpret_cast<float2*>(Bh + off) = make_float2(h0, h1);
                *reinterpret_cast<float2*>(Bl + off) = make_float2(lo0, lo1);
            } else {
                const int ln = tid >> 2, k0 = 8 * i + (tid & 3), k1 = k0 + 4;
                const uint32_t o0 = swz(ln, k0 >> 2) + ((k0 & 3) << 2), o1 = swz(ln, k1 >> 2) + ((k1 & 3) << 2);
                *reinterpret_cast<float*>(Bh + o0) = h0;
                *reinterpret_cast<float*>(Bl + o0) = lo0;
                *reinterpret_cast<float*>(Bh + o1) = h1;
                *reinterpret_cast<float*>(Bl + o1) = lo1;
            }
        }
    };
    // control: D chunk c of the image into the A tiles of stage s (hi then lo, contiguous)
    auto issue_D = [&](int c, int s) {
        const uint8_t* src = reinterpret_cast<const uint8_t*>(Dimg) + (size_t)c * 2 * a_bytes;
        const uint32_t dst = su32(stage_ptr(s));
        mbar_arrive_expect_tx(&full[s], 2 * a_bytes);
        for (uint32_t o = 0; o < 2 * a_bytes; o += kBulkPiece) {
            const uint32_t n = min(kBulkPiece, 2 * a_bytes - o);
            bulk_g2s(dst + o, src + o, n, &full[s]);
        }
    };
    // epilogue of tile `it` from accumulator b by an epilogue warp: TMEM lane quadrant
    // warp % 4 (rows), 16 columns (lines) per tcgen05.ld.  x lines: lanes hold consecutive
    // rows of a line (contiguous).  y, z lines: a thread holds 16 consecutive lines of one
    // row, contiguous when the lines do not wrap in a (na % 16 == 0): 16-byte stores.
    const bool vec16 = !XL && ls.oa == 1 && ls.na % 16 == 0 && ls.op % 2 == 0 && ls.ob % 2 == 0 &&
                       (reinterpret_cast<uintptr_t>(out) & 15) == 0 &&
                       (!RESID || (ls.fa == 1 && ls.fp % 2 == 0 && ls.fb % 2 == 0 &&
                                   (reinterpret_cast<uintptr_t>(f) & 15) == 0));
    // Residual form: the epilogue re-reads f.  Between a tile's staging loads and its
    // epilogue the producers and the stores move about as many bytes as L2 holds, so many
    // re-reads go to DRAM.  x lines request each group's 16 values before the accumulator
    // read and stream both the re-reads and the stores (whole 256-byte rows per warp
    // instruction), which keeps more of the staged lines in L2: 0.174 -> 0.163 ms per 256^3
    // CF90 launch.  (Streaming the 16-byte stores of y and z lines, or asking L2 for a tile's
    // rows ahead, measured slower.)
    auto put = [&](double* p, double v) {
        if (RESID && XL) __stcs(p, v);
        else *p = v;
    };
    auto epilogue = [&](long it, int b) {
        const long l0 = tile_of(it) * NT;
        const int lq = warp & 3;
        for (int mh = 0; mh < nout / 128; mh++) {
            const int row = mh * 128 + lq * 32 + lane;
            for (int cb = 0; cb < NT / 16; cb++) {
                const long line0 = l0 + cb * 16;
                // residual form (filters): the accumulator holds (I - D) f, the output is f minus it
                double fr[16];
                if (RESID && XL) {
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        fr[j] = line0 + j < nlines ? __ldcs(f + (line0 + j) * ls.fa + row) : 0.0;
                }
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(b * nout + mh * NT + cb * 16), r);
                if (XL) {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const long line = line0 + j;
                        if (line >= nlines) continue;
                        const double v = float_bits_to_double(__uint_as_float(r[j]));
                        put(out + line * ls.oa + row, RESID ? fr[j] - v : v);
                    }
                } else if (vec16 && line0 + 16 <= nlines) {
                    const long a = line0 % ls.na, bb = line0 / ls.na;
                    double* o = out + a + bb * ls.ob + (long)row * ls.op;
                    const double* fi = f + a + bb * ls.fb + (long)row * ls.fp;
#pragma unroll
                    for (int j = 0; j < 16; j += 2) {
                        double2 v = make_double2(float_bits_to_double(__uint_as_float(r[j])),
                                                 float_bits_to_double(__uint_as_float(r[j + 1])));
                        if (RESID) {
                            const double2 x = __ldg(reinterpret_cast<const double2*>(fi + j));
                            v = make_double2(x.x - v.x, x.y - v.y);
                        }
                        *reinterpret_cast<double2*>(o + j) = v;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const long line = line0 + j;
                        if (line >= nlines) continue;
                        const long a = line % ls.na, bb = line / ls.na;
                        const double v = float_bits_to_double(__uint_as_float(r[j]));
                        put(out + a * ls.oa + bb * ls.ob + (long)row * ls.op,
                            RESID ? __ldg(f + a * ls.fa + bb * ls.fb + (long)row * ls.fp) - v : v);
                    }
                }
            }
        }
    };

    if (producer) {
        double2 R0[WS_FPT], R1[WS_FPT];
        load_item(0, R0);
        load_item(1, R1);
        for (long it = 0; it < my_tiles; it++) {
            for (int c = 0; c < nchunks; c++) {
                const long gg = it * nchunks + c;
                const int s = (int)(gg % WS_STAGES);
                double2 R2[WS_FPT];
                load_item(gg + 2, R2);
                if (gg >= WS_STAGES) wait(&empty[s], (unsigned)((gg / WS_STAGES - 1) & 1));
                if (!abort_flag) store_F(s, R0);
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
#pragma unroll
                for (int i = 0; i < WS_FPT; i++) {
                    R0[i] = R1[i];
                    R1[i] = R2[i];
                }
            }
        }
    } else if (control) {
        for (long it = 0; it < my_tiles; it++) {
            const int b = (int)(it % NACC);
            // the accumulator's previous tile has been read out
            if (it >= NACC) wait(&acce[b], (unsigned)((it / NACC - 1) & 1));
            tc_fence_after();
            for (int c = 0; c < nchunks; c++) {
                const long gg = it * nchunks + c;
                const int s = (int)(gg % WS_STAGES);
                wait(&full[s], (unsigned)((gg / WS_STAGES) & 1));
                if (!abort_flag) {
                    tc_fence_after();
                    uint8_t* Ah = stage_ptr(s);
                    uint8_t* Al = Ah + a_bytes;
                    uint8_t* Bh = Al + a_bytes;
                    uint8_t* Bl = Bh + b_bytes;
                    for (int mh = 0; mh < nout / 128; mh++) {
                        const uint32_t d = tmem + (uint32_t)(b * nout + mh * NT);
#pragma unroll
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
                    mma_commit(&empty[s]);
                } else {
                    mbar_arrive(&empty[s]);
                }
            }
            if (!abort_flag) mma_commit(&accf[b]);
            else mbar_arrive(&accf[b]);
        }
    } else if (loader) {
        // each item's D chunk as soon as the MMAs two items back release its stage
        for (long gn = 0; gn < nitems; gn++) {
            const int sn = (int)(gn % WS_STAGES);
            if (gn >= WS_STAGES) wait(&empty[sn], (unsigned)((gn / WS_STAGES - 1) & 1));
            if (!abort_flag) {
                issue_D((int)(gn % nchunks), sn);
                issued[sn] = gn;
            } else {
                mbar_arrive(&full[sn]);  // keep the arrival count; no bytes expected
            }
        }
    } else if (epi_warp) {
        for (long it = 0; it < my_tiles; it++) {
            const int b = (int)(it % NACC);
            wait(&accf[b], (unsigned)((it / NACC) & 1));
            tc_fence_after();
            if (!abort_flag) epilogue(it, b);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[b]);
        }
    }
    if (abort_flag && loader) {
        // the copies issued: a phase cannot complete before its copy's bytes land, so wait
        // (bounded) for the last phase of each stage that received one
        for (int s = 0; s < WS_STAGES; s++) {
            if (issued[s] < 0) continue;
            unsigned k = 0;
            while (!mbar_try_wait(&full[s], (unsigned)((issued[s] / WS_STAGES) & 1)) && ++k < kWaitLimit) {
            }
        }
    }
    if (abort_flag) atomicOr(&g_dense_err, 1u);
    if (bad) atomicOr(rangeflag, 1u);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

struct DenseMat {
    int resid = 0;  // the matrix is I - A^-1 B of a filter in residual form (output f - M f)
    float* Dh = nullptr;
    float* Dl = nullptr;
    float* Dimg = nullptr;  // per K chunk: hi then lo, nout rows of 128 bytes, swizzled as in shared memory
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
    // filters in residual form (cf90): the tensor cores apply I - A^-1 B, whose result is
    // small next to f, and the epilogue subtracts it from f in FP64, so the FP32
    // accumulation's rounding scales with the small part only
    if (d.resid && d.m == d.nout) {
        dm.resid = 1;
        for (int i = 0; i < d.nout; i++)
            for (int j = 0; j < d.m; j++) M[(size_t)i * d.m + j] = (i == j ? 1.0 : 0.0) - M[(size_t)i * d.m + j];
    }
    std::vector<float> hi(M.size()), lo(M.size());
    for (size_t i = 0; i < M.size(); i++) {
        hi[i] = tf32_host(M[i]);
        lo[i] = tf32_host(M[i] - (double)hi[i]);
    }
    // the shared-memory image of every K chunk, for one bulk copy per chunk
    std::vector<float> img;
    if (dm.nin % KC == 0) {
        const int nch = dm.nin / KC;
        img.assign((size_t)nch * 2 * dm.nout * 32, 0.0f);
        for (int c = 0; c < nch; c++)
            for (int hl = 0; hl < 2; hl++)
                for (int r = 0; r < dm.nout; r++)
                    for (int k = 0; k < KC; k++) {
                        const size_t byte = ((size_t)c * 2 + hl) * dm.nout * 128 + (size_t)r * 128 +
                                            (size_t)(((k >> 2) ^ (r & 7)) << 4) + (size_t)(k & 3) * 4;
                        const size_t src = (size_t)r * dm.nin + (size_t)c * KC + k;
                        img[byte / 4] = hl ? lo[src] : hi[src];
                    }
    }
    if ((rc = upload(&dm.Dh, hi)) != PS_OK) return rc;
    if ((rc = upload(&dm.Dl, lo)) != PS_OK) {
        cudaFree(dm.Dh);
        return rc;
    }
    if (!img.empty() && (rc = upload(&dm.Dimg, img)) != PS_OK) {
        cudaFree(dm.Dh);
        cudaFree(dm.Dl);
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
            cudaFree(it->second.Dimg);
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
    if (!h || na < 0 || nb < 0) return PS_EINVAL;
    if (dir < 1 || dir > 3) return PS_EINVAL;
    if (na == 0 || nb == 0) return PS_OK;  // empty arrays: nothing to do
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
    // lines of a (m, na, nb) / (na, m, nb) / (na, nb, m) array, m = nin on input, nout on output
    LineSet ls{};
    const long nlines = (long)na * nb;
    ls.nlines = nlines;
    if (dir == 1) {
        ls.na = nlines; ls.fa = D->nin; ls.fb = 0; ls.fp = 1; ls.oa = D->nout; ls.ob = 0; ls.op = 1;
    } else if (dir == 2) {
        ls.na = na; ls.fa = 1; ls.fb = (long)na * D->nin; ls.fp = na;
        ls.oa = 1; ls.ob = (long)na * D->nout; ls.op = na;
    } else {
        ls.na = nlines; ls.fa = 1; ls.fb = 0; ls.fp = nlines; ls.oa = 1; ls.ob = 0; ls.op = nlines;
    }
    const size_t stage = (size_t)D->nout * 128 * 2 + (size_t)NT * 128 * 2;
    const int stages = 1024 + 2 * stage <= 220 * 1024 ? 2 : 1;
    const size_t smem = 1024 + stages * stage;
    const long blocks = (nlines + NT - 1) / NT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (stages == 2 && D->Dimg) {
        // persistent warp-specialised pipeline: one CTA per SM over the 128-line tiles
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
            return PS_ECUDA;
        auto kw = dir == 1 ? (D->resid ? k_dense_ws<true, true> : k_dense_ws<true, false>)
                           : (D->resid ? k_dense_ws<false, true> : k_dense_ws<false, false>);
        const size_t smem_ws = smem;
        if (cudaFuncSetAttribute(kw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_ws) != cudaSuccess)
            return PS_ECUDA;
        const long grid = std::min<long>(blocks, nsm);
        kw<<<(unsigned)grid, WS_THREADS, smem_ws, s>>>(f, out, D->Dimg, D->nin, D->nout, ls, blocks, h->status);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    auto kern = dir == 1 ? (stages == 2 ? k_dense_tf32<2, true> : k_dense_tf32<1, true>)
                         : (stages == 2 ? k_dense_tf32<2, false> : k_dense_tf32<1, false>);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PS_ECUDA;
    kern<<<(unsigned)blocks, NTHR, smem, s>>>(f, out, D->Dh, D->Dl, D->nin, D->nout, ls, h->status, D->resid);
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
