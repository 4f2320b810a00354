// Register-resident line kernel for periodic (circulant) lines.
//
// The same chunk algorithm as k_line (forward recurrence from a zero state, log-step scan
// of the chunk transfers with the ring wrap, corrected backward recurrence, backward scan,
// correction), laid out for instruction issue rather than shared memory:
//   * each lane loads its own chunk of M rows straight into registers (16-byte loads along
//     contiguous lines; along strided lines the lanes of one chunk row are four consecutive
//     lines, 32-byte segments), so there is no staging pass, no work rows in shared memory
//     and no block barrier;
//   * the chunk halos (H rows each side) come from the neighbouring lanes by warp shuffles,
//     around the ring for the first and last chunk;
//   * the loops over the chunk rows are unrolled, so every row index is a constant: the
//     stencil, recurrence and correction coefficients are kernel parameters read from the
//     constant bank by the arithmetic instructions themselves;
//   * the FP64 input is split with integer instructions against the line's shift, computed
//     once per line (df_split_line: about half the instructions of df_from_double_shift);
//   * residual-form operators (cf90) subtract the solve from the FP64 input in FP64 (the
//     input re-read, an L1/L2 hit) instead of keeping it in registers.
// The unrolled rows make the code large: with FP32 arithmetic (about a third of the
// instructions of double-float) it is the faster kernel; the double-float instantiation
// stalls on instruction fetch (measured) and the shared-memory k_line stays the default there.
// Lines hold ns = P * M rows (P lanes per line, a power of two); 128 threads per CTA.
#pragma once
#include <cuda_runtime.h>

#include "chunk_kernel.cuh"

namespace pade {

constexpr int kRegThreads = 128;
constexpr int kRegMaxM = 32;

struct RegParams {
    int ns, nout, P, nsteps;
    int xdup;      // edges to cells: row ns (edge n + 1) is read as the first row above the top
    int vec_in;    // contiguous input lines at 16-byte aligned starts: 16-byte loads
    int vec_out;   // the same for the output
    F2 c0;
    F2 c[kMaxPairs];
    F2 ca1, ca2;
    F2 phf[kRegMaxM][2];  // response of chunk row j to a unit incoming forward state
    F2 phb[kRegMaxM][2];  // response of the row j from the chunk end to a unit backward state
    const F2* fscan;
    const F2* bscan;
    const F2* fwrap;
    const F2* bwrap;
};

// Split of d * 2^-k into a df value, for lines whose maximum exponent emax gives k = emax -
// 1023 (so every scaled value is below 2).  kb = -(k + 896) << 23 rebiases the exponent
// field of the high part, kc = -(k + 948) << 23 builds the low part's power of two, thr =
// max(949 + k, 1) << 20: values whose scaled exponent is below 2^-74, zeros and subnormals
// give 0 (the kernels' line-relative range).  Exactly the value of df_from_double_shift.
// Row accessor of a chunk and its halos (r in [-H, M + H); constant after unrolling).
template <int M, int H, class V>
__device__ __forceinline__ V row_at(const V (&x)[M], const V (&hl)[H], const V (&hr)[H], int r) {
    return r < 0 ? hl[H + r] : (r >= M ? hr[r - M] : x[r]);
}

// RHS of row j: pairs k = 1..NP about the row (STG = 0) or about the half point j + 1/2
// (STG = +1: offsets k, 1 - k) or j - 1/2 (STG = -1: offsets k - 1, -k); centre c0 for
// symmetric centred stencils.
template <class AR, int M, int H, int NP, bool SYM, int STG>
__device__ __forceinline__ typename AR::V reg_stencil(const typename AR::V (&x)[M], const typename AR::V (&hl)[H],
                                                     const typename AR::V (&hr)[H], int j, const RegParams& cp) {
    using V = typename AR::V;
    constexpr int sh = STG > 0 ? 0 : (STG < 0 ? -1 : 0);
    V acc;
    if constexpr (STG != 0) {
#pragma unroll
        for (int k = 1; k <= NP; k++) {
            const V a = row_at<M, H>(x, hl, hr, j + k + sh), b = row_at<M, H>(x, hl, hr, j + 1 - k + sh);
            const V d = SYM ? AR::add(a, b) : AR::sub(a, b);
            acc = k == 1 ? AR::mul(d, AR::coef(cp.c[0])) : AR::add(acc, AR::mul(d, AR::coef(cp.c[k - 1])));
        }
    } else {
        if constexpr (SYM) acc = AR::mul(x[j], AR::coef(cp.c0));
#pragma unroll
        for (int k = 1; k <= NP; k++) {
            const V a = row_at<M, H>(x, hl, hr, j + k), b = row_at<M, H>(x, hl, hr, j - k);
            const V d = SYM ? AR::add(a, b) : AR::sub(a, b);
            acc = (!SYM && k == 1) ? AR::mul(d, AR::coef(cp.c[0])) : AR::add(acc, AR::mul(d, AR::coef(cp.c[k - 1])));
        }
    }
    return acc;  // not renormalised: the recurrence's fms folds it in
}

// Out-of-line FP64 assembly for line scales beyond 2^+-800 (rare)
template <class AR>
__device__ __noinline__ double reg_store_checked(typename AR::V v, int kl) {
    return AR::store_scaled(v, kl);
}

template <class AR, int Q, int NP, bool SYM, int M, int STG, bool RESID, int MINB>
__global__ void __launch_bounds__(kRegThreads, MINB)
    k_lreg(const RegParams cp, const typename AR::IO* __restrict__ f, typename AR::IO* __restrict__ out,
           const LineSet ls, unsigned* __restrict__ status) {
    using V = typename AR::V;
    using IO = typename AR::IO;
    constexpr int H = NP;
    const int P = cp.P;
    const int t = threadIdx.x & (P - 1);
    const long line = (long)blockIdx.x * (kRegThreads / P) + threadIdx.x / P;
    const bool active = line < ls.nlines;
    long bin = 0, bout = 0;
    if (active) {
        const long a = line % ls.na, b = line / ls.na;
        bin = a * ls.fa + b * ls.fb;
        bout = a * ls.oa + b * ls.ob;
    }
    const IO* src = f + bin;
    const long r0 = (long)t * M;  // first row of this lane's chunk

    // ---- load the chunk ----
    IO v[M];
    if (!active) {
#pragma unroll
        for (int r = 0; r < M; r++) v[r] = (IO)0;
    } else if (cp.vec_in) {
        if constexpr (sizeof(IO) == 8) {
            const double2* s2 = reinterpret_cast<const double2*>(src + r0);
#pragma unroll
            for (int r = 0; r < M / 2; r++) {
                const double2 q = __ldg(s2 + r);
                v[2 * r] = q.x;
                v[2 * r + 1] = q.y;
            }
        } else {
            const float4* s4 = reinterpret_cast<const float4*>(src + r0);
#pragma unroll
            for (int r = 0; r < M / 4; r++) {
                const float4 q = __ldg(s4 + r);
                v[4 * r] = q.x;
                v[4 * r + 1] = q.y;
                v[4 * r + 2] = q.z;
                v[4 * r + 3] = q.w;
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < M; r++) v[r] = __ldg(src + (r0 + r) * ls.fp);
    }

    // ---- split (df: scaled by the line's largest exponent) ----
    V x[M];
    unsigned bad = 0;
    int kl = 0;
    if constexpr (AR::kScaled) {
        int mx = 0;
#pragma unroll
        for (int r = 0; r < M; r++) mx = max(mx, bexp(v[r]));
        for (int o = 1; o < P; o <<= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o, P));
        bad = (unsigned)(mx == 2047);
        kl = mx - 1023;
        const SplitK sk = split_consts(kl);
#pragma unroll
        for (int r = 0; r < M; r++) x[r] = df_split_line(v[r], sk);
    } else {
#pragma unroll
        for (int r = 0; r < M; r++) x[r] = AR::load(v[r], bad);
    }

    // ---- halos from the neighbouring lanes (ring) ----
    V hl[H], hr[H];
    const int tl = (t + P - 1) & (P - 1), tr = (t + 1) & (P - 1);
#pragma unroll
    for (int h = 0; h < H; h++) {
        hl[h] = AR::shfl_idx(x[M - H + h], tl, P);
        hr[h] = AR::shfl_idx(x[h], tr, P);
    }
    if constexpr (STG > 0) {
        // edges to cells: the stored edge n + 1 is the first row above the top
        if (cp.xdup && t == P - 1 && active) {
            const IO e = __ldg(src + (long)cp.ns * ls.fp);
            if constexpr (AR::kScaled) {
                bad |= (unsigned)(bexp(e) == 2047);
                hr[0] = df_split_line(e, split_consts(kl));
            } else {
                hr[0] = AR::load(e, bad);
            }
        }
    }

    // ---- forward: RHS and recurrence from a zero state ----
    const V a1 = AR::coef(cp.ca1), a2 = AR::coef(cp.ca2);
    V y[M];
    V s1 = AR::zero(), s2 = AR::zero();
#pragma unroll
    for (int j = 0; j < M; j++) {
        const V r = reg_stencil<AR, M, H, NP, SYM, STG>(x, hl, hr, j, cp);
        y[j] = (Q == 2) ? AR::fms2(r, a1, s1, a2, s2) : AR::fms1(r, a1, s1);
        s2 = s1;
        s1 = y[j];
    }

    // ---- forward scan of the chunk transfers, then the ring wrap ----
    for (int k = 0; k < cp.nsteps; k++) {
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_up(s1, dlt, P);
        const V o2 = (Q == 2) ? AR::shfl_up(s2, dlt, P) : AR::zero();
        if (t >= (int)dlt) {
            const F2* Fm = cp.fscan + ((size_t)t * kMaxSteps + k) * 4;
            if constexpr (Q == 2) {
                const V n1 = AR::mac2(s1, AR::coef(Fm[0]), o1, AR::coef(Fm[1]), o2);
                const V n2 = AR::mac2(s2, AR::coef(Fm[2]), o1, AR::coef(Fm[3]), o2);
                s1 = n1;
                s2 = n2;
            } else {
                s1 = AR::mac1(s1, AR::coef(Fm[0]), o1);
            }
        }
    }
    V i1 = AR::shfl_up(s1, 1, P);
    V i2 = (Q == 2) ? AR::shfl_up(s2, 1, P) : AR::zero();
    if (t == 0) {
        i1 = AR::zero();
        i2 = AR::zero();
    }
    {
        const V E1 = AR::shfl_idx(s1, P - 1, P);
        const V E2 = (Q == 2) ? AR::shfl_idx(s2, P - 1, P) : AR::zero();
        const F2* Wm = cp.fwrap + (size_t)t * 4;
        if constexpr (Q == 2) {
            const V n1 = AR::mac2(i1, AR::coef(Wm[0]), E1, AR::coef(Wm[1]), E2);
            const V n2 = AR::mac2(i2, AR::coef(Wm[2]), E1, AR::coef(Wm[3]), E2);
            i1 = n1;
            i2 = n2;
        } else {
            i1 = AR::mac1(i1, AR::coef(Wm[0]), E1);
        }
    }

    // ---- backward: forward correction and recurrence from a zero state ----
    V u1 = AR::zero(), u2 = AR::zero();
#pragma unroll
    for (int j = M - 1; j >= 0; j--) {
        const V yy = (Q == 2) ? AR::mac2(y[j], AR::coef(cp.phf[j][0]), i1, AR::coef(cp.phf[j][1]), i2)
                              : AR::mac1(y[j], AR::coef(cp.phf[j][0]), i1);
        const V xx = (Q == 2) ? AR::fms2(yy, a1, u1, a2, u2) : AR::fms1(yy, a1, u1);
        y[j] = xx;
        u2 = u1;
        u1 = xx;
    }

    // ---- backward scan, then the ring wrap ----
    for (int k = 0; k < cp.nsteps; k++) {
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_down(u1, dlt, P);
        const V o2 = (Q == 2) ? AR::shfl_down(u2, dlt, P) : AR::zero();
        if (t + (int)dlt < P) {
            const F2* Bm = cp.bscan + ((size_t)t * kMaxSteps + k) * 4;
            if constexpr (Q == 2) {
                const V n1 = AR::mac2(u1, AR::coef(Bm[0]), o1, AR::coef(Bm[1]), o2);
                const V n2 = AR::mac2(u2, AR::coef(Bm[2]), o1, AR::coef(Bm[3]), o2);
                u1 = n1;
                u2 = n2;
            } else {
                u1 = AR::mac1(u1, AR::coef(Bm[0]), o1);
            }
        }
    }
    V j1 = AR::shfl_down(u1, 1, P);
    V j2 = (Q == 2) ? AR::shfl_down(u2, 1, P) : AR::zero();
    if (t >= P - 1) {
        j1 = AR::zero();
        j2 = AR::zero();
    }
    {
        const V F1 = AR::shfl_idx(u1, 0, P);
        const V F2v = (Q == 2) ? AR::shfl_idx(u2, 0, P) : AR::zero();
        const F2* Wm = cp.bwrap + (size_t)t * 4;
        if constexpr (Q == 2) {
            const V n1 = AR::mac2(j1, AR::coef(Wm[0]), F1, AR::coef(Wm[1]), F2v);
            const V n2 = AR::mac2(j2, AR::coef(Wm[2]), F1, AR::coef(Wm[3]), F2v);
            j1 = n1;
            j2 = n2;
        } else {
            j1 = AR::mac1(j1, AR::coef(Wm[0]), F1);
        }
    }

    // ---- backward correction, FP64 assembly (residual form: input minus the solve) ----
#pragma unroll
    for (int j = 0; j < M; j++)
        y[j] = (Q == 2) ? AR::mac2(y[j], AR::coef(cp.phb[M - 1 - j][0]), j1, AR::coef(cp.phb[M - 1 - j][1]), j2)
                        : AR::mac1(y[j], AR::coef(cp.phb[M - 1 - j][0]), j1);
    IO o[M];
    if constexpr (AR::kScaled) {
        const bool fast = kl >= -800 && kl <= 800;
        if (fast) {
            const unsigned kadd = (unsigned)(896 + kl) << 20;
#pragma unroll
            for (int j = 0; j < M; j++) o[j] = df_to_double_kadd(y[j], kadd);
        } else {
            if constexpr (RESID) {
                // extreme line scales: the subtraction in double-float before the checked
                // assembly (the solve alone could fall below the normal FP64 range)
                const SplitK sk = split_consts(kl);
#pragma unroll
                for (int j = 0; j < M; j++) {
                    const dfv xj = df_split_line(active ? __ldg(src + (r0 + j) * ls.fp) : 0.0, sk);
                    y[j] = df_norm(df_sub(xj, y[j]));
                }
            }
#pragma unroll
            for (int j = 0; j < M; j++) o[j] = reg_store_checked<AR>(y[j], kl);
        }
        if constexpr (RESID) {
            // the FP64 input again (L1/L2): out = f - A^-1 ((A - B) f) in FP64
            if (active && fast) {
                if (cp.vec_in) {
                    const double2* s2 = reinterpret_cast<const double2*>(src + r0);
#pragma unroll
                    for (int r = 0; r < M / 2; r++) {
                        const double2 q = __ldg(s2 + r);
                        o[2 * r] = __dsub_rn(q.x, o[2 * r]);
                        o[2 * r + 1] = __dsub_rn(q.y, o[2 * r + 1]);
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < M; r++) o[r] = __dsub_rn(__ldg(src + (r0 + r) * ls.fp), o[r]);
                }
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < M; j++) {
            V z = y[j];
            if constexpr (RESID) z = AR::sub(x[j], z);
            o[j] = AR::store(z);
        }
    }

    // ---- store ----
    if (active) {
        IO* dst = out + bout;
        if (cp.vec_out) {
            if constexpr (sizeof(IO) == 8) {
                double2* d2 = reinterpret_cast<double2*>(dst + r0);
#pragma unroll
                for (int r = 0; r < M / 2; r++) d2[r] = make_double2(o[2 * r], o[2 * r + 1]);
            } else {
                float4* d4 = reinterpret_cast<float4*>(dst + r0);
#pragma unroll
                for (int r = 0; r < M / 4; r++) d4[r] = make_float4(o[4 * r], o[4 * r + 1], o[4 * r + 2], o[4 * r + 3]);
            }
        } else {
#pragma unroll
            for (int r = 0; r < M; r++) dst[(r0 + r) * ls.op] = o[r];
        }
        // cells-to-edges outputs repeat row 0 as row ns (the periodic edge n + 1)
        if (cp.nout > cp.ns && t == 0) dst[(long)cp.ns * ls.op] = o[0];
    }
    if (bad) atomicOr(status, 1u);
}

}  // namespace pade
