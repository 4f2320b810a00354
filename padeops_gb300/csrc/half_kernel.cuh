// Half-chunk line kernel: periodic (circulant) lines in chunks of 32 rows, double-float
// arithmetic in Blackwell's packed FP32x2 instructions.
//
// k_line runs one lane per 32-row chunk and spends most of its issue slots on the
// double-float sums and products of the right-hand side, the two recurrences and the two
// fundamental-solution corrections, one row at a time.  Here each lane splits its chunk
// into two halves of 16 rows, A (rows 0..15) and B (rows 16..31), and runs the same
// algorithm on both halves at once: rows j and j + 16 travel as the two components of
// packed operands (`add/mul/fma.rn.f32x2`, each component rounded as the scalar
// instruction, so every error-free transformation stays exact), which halves the
// instructions of all five per-row phases.  The halves meet in the lane's chunk transfer
// and in the corrections:
//   * forward: both halves run the recurrence from a zero state; the chunk's outgoing state
//     is B's end state plus A's end state propagated through B by the fundamental solutions
//     of a 16-row block (the first 16 rows of those of a 32-row chunk); after the scan, A is
//     corrected with the incoming state and B with A's corrected end state;
//   * backward: the same from the bottom, with the backward fundamental solutions.
// The lane scan, the ring wrap and every table are those of the 32-row chunk plan.
//
// Layout: a lane's input window holds rows -H .. 15 + H of half A beside rows 16 - H .. 31 + H
// of half B as 16-byte pairs {h_r, h_r+16, l_r, l_r+16} (r = -H .. 15 + H), so one 128-bit
// shared load gives both packed operands; rows 13 .. 18 (for H = 3) sit in two pairs.  Work
// pairs overwrite the window pair H rows up, and the FP64 results of rows j and j + 16
// overwrite work pair j as a double2, which the coalesced store reads back.
// The same runs on 16-row chunks split into halves of 8 (template M = 16, the 16-row chunk
// plan's tables): half the shared memory and staging registers per thread.
#pragma once
#include <cuda_runtime.h>

#include "stencil_kernel.cuh"

namespace pade {

// a plan coefficient broadcast to both components
__device__ __forceinline__ df2 d2_bcast(F2 c) { return d2_bcast(dfv{c.h, c.l}); }

// right-hand side of rows (j, j + 16) from the window pairs p(-NP) .. p(NP) (p(k): pair j + k
// as packed operands); pairs k = 1..NP at offsets (k, -k) about the row (STG = 0), or about a
// half point: (k, 1 - k) (STG = +1, edges to cells) or (k - 1, -k) (STG = -1, cells to
// edges), in k_line's operation order
template <int NP, bool SYM, int STG = 0, class W>
__device__ __forceinline__ df2 half_stencil(const W& p, const df2 (&c)[NP], df2 c0) {
    df2 acc;
    if constexpr (STG != 0) {
        constexpr int sh = STG > 0 ? 0 : -1;
        acc = SYM ? d2_mul(d2_add(p(1 + sh), p(sh)), c[0]) : d2_mul(d2_sub(p(1 + sh), p(sh)), c[0]);
#pragma unroll
        for (int k = 2; k <= NP; k++) {
            const df2 d = SYM ? d2_add(p(k + sh), p(1 - k + sh)) : d2_sub(p(k + sh), p(1 - k + sh));
            acc = d2_add(acc, d2_mul(d, c[k - 1]));
        }
    } else if constexpr (SYM) {
        acc = d2_mul(p(0), c0);
#pragma unroll
        for (int k = 1; k <= NP; k++) acc = d2_add(acc, d2_mul(d2_add(p(k), p(-k)), c[k - 1]));
    } else {
        acc = d2_mul(d2_sub(p(1), p(-1)), c[0]);
#pragma unroll
        for (int k = 2; k <= NP; k++) acc = d2_add(acc, d2_mul(d2_sub(p(k), p(-k)), c[k - 1]));
    }
    return d2_norm(acc);
}

// window pairs per lane (rows -H .. HM - 1 + H of half A, HM = M / 2 rows per half),
// padded to an odd count of 16-byte units so the 8 lanes of a line in one quarter-warp
// read distinct banks
__host__ __device__ constexpr int half_lane_stride(int hm, int np) { return (hm + 2 * np) | 1; }

// 16-byte units per line: odd, so the 16 lines a strided warp instruction touches spread
// over the banks (an even stride such as 8 x 23 = 184 puts all 16 on one bank)
__host__ __device__ constexpr int half_line_stride(int p, int hm, int np) {
    return (p * half_lane_stride(hm, np)) | 1;
}

// Largest line the kernel stages in registers: contiguous lines take ns / 32 rows per lane
// (at most 8); strided lines one row per lane of the line and chunk row (at most M).
constexpr int kHalfRowsContig = 8;

// A lane's coefficients of scan step k (4 for two-term recurrences, 1 otherwise), loaded for
// every step the lane takes part in before the scan starts: one round trip to L1 / L2 instead
// of one per step; the entries of skipped steps are neither read nor used.
template <int Q>
struct ScanCoefs {
    static constexpr int NE = Q == 2 ? 4 : 1;
    F2 m[kMaxSteps][NE];
    __device__ __forceinline__ void load(const F2* tab, int row, int k0, int nsteps, unsigned take) {
#pragma unroll
        for (int k = 0; k < kMaxSteps; k++) {
#pragma unroll
            for (int e = 0; e < NE; e++) m[k][e] = F2{0.0f, 0.0f};
            if (k >= k0 && k < nsteps && ((take >> k) & 1u)) {
#pragma unroll
                for (int e = 0; e < NE; e++) {
                    const float2 v = __ldg(reinterpret_cast<const float2*>(tab) + ((size_t)row * kMaxSteps + k) * 4 + e);
                    m[k][e] = F2{v.x, v.y};
                }
            }
        }
    }
};

// J: coalesced stores of a CTA's lines from the FP64 results in the windows (rows j and
// j + HM of a lane as the double2 over its work pair j: row q of chunk t is double
// 2 (q % HM) + q / HM of its lane); strided lines by pairs, as staged.  An output longer than
// the line (nout > ns) repeats its first rows.  Residual form (nout = ns): f - x, each thread
// reading f at the points it writes (so an in-place call is safe), all of its loads issued
// before its first subtraction instead of one L2 round trip per row.
template <int M, bool RESID>
__device__ __forceinline__ void half_store(const float4* tile, int LT, int SL, int nl, int L, int ns, int nout,
                                           const double* __restrict__ f, double* __restrict__ out,
                                           const long* base_in, const long* base_out, const LineSet& ls) {
    constexpr int HM = M / 2;
    const int tid = threadIdx.x, nth = blockDim.x;
    const double* od = reinterpret_cast<const double*>(tile);
    auto out_pos = [&](int ll, int p) -> int {
        const unsigned tt = (unsigned)p / M, q = (unsigned)p % M;
        return ((ll * LT + (int)tt * SL) << 1) + 2 * (int)(q % HM) + (int)(q / HM);
    };
    if (ls.op == 1) {
        const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
        for (int ll = warp; ll < nl; ll += nw) {
            double* o = out + base_out[ll];
            if constexpr (RESID) {
                const double* fi = f + base_in[ll];
                const int fs = (int)ls.fp;  // 32-bit row offsets (the launchers check that they fit)
                double fv[kHalfRowsContig];
#pragma unroll
                for (int u = 0; u < kHalfRowsContig; u++) {
                    const int p = lane + 32 * u;
                    fv[u] = p < ns ? fi[p * fs] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < kHalfRowsContig; u++) {
                    const int p = lane + 32 * u;
                    if (p < ns) o[p] = __dsub_rn(fv[u], od[out_pos(ll, p)]);
                }
                for (int p = lane + 32 * kHalfRowsContig; p < ns; p += 32)
                    o[p] = __dsub_rn(fi[p * fs], od[out_pos(ll, p)]);
            } else {
                for (int p = lane; p < nout; p += 32) o[p] = od[out_pos(ll, p < ns ? p : p - ns)];
            }
        }
    } else {
        // row offsets in 32 bits (the launchers check that they fit)
        const int ll = tid % L, pstep = nth / L, k0 = tid / L, nk = ns >> 1;
        const int fs = (int)ls.fp, os = (int)ls.op;
        (void)fs;
        if (ll < nl) {
            double* o = out + base_out[ll];
            const double2* od2 = reinterpret_cast<const double2*>(tile) + (size_t)ll * LT;
            if constexpr (RESID) {
                // pstep * HM >= nk: HM pairs per thread cover the line
                const double* fi = f + base_in[ll];
                double2 fv[HM];
#pragma unroll
                for (int i = 0; i < HM; i++) {
                    const int k = k0 + pstep * i;
                    const int p = (k / HM) * M + k % HM;
                    fv[i] = k < nk ? make_double2(fi[p * fs], fi[(p + HM) * fs])
                                   : make_double2(0.0, 0.0);
                }
#pragma unroll
                for (int i = 0; i < HM; i++) {
                    const int k = k0 + pstep * i;
                    if (k < nk) {
                        const int p = (k / HM) * M + k % HM;
                        const double2 x = od2[(k / HM) * SL + k % HM];
                        o[p * os] = __dsub_rn(fv[i].x, x.x);
                        o[(p + HM) * os] = __dsub_rn(fv[i].y, x.y);
                    }
                }
            } else {
                for (int k = k0; k < nk; k += pstep) {
                    const int p = (k / HM) * M + k % HM;
                    const double2 x = od2[(k / HM) * SL + k % HM];
                    o[p * os] = x.x;
                    o[(p + HM) * os] = x.y;
                }
                for (int p = ns + k0; p < nout; p += pstep) o[p * os] = od[out_pos(ll, p - ns)];
            }
        }
    }
}

// M: chunk rows (32, or 16 for twice the resident lines per SM: half the shared memory and
// registers per thread for a longer lane scan).  RESID: a filter in residual form (cf90): the
// solve gives x = A^-1 (A - B) f and the output is f - x, with f read again from the input
// by the coalesced store (L2-resident by then), so the window can still be overwritten.
// STG: the staggered cd06stagg shapes (+1 edges to cells, -1 cells to edges; with xdup the
// stored edge n + 1 is read as the first row above the top, as the reference's periodic RHS
// reads it, cd06stagg.F90:319, 544)
template <int Q, int NP, bool SYM, int M, bool RESID, int STG = 0>
__global__ void __launch_bounds__(kLineThreadsCirc, M == 32 ? 4 : 5)
    k_lhalf(const StencilParams cp, const double* __restrict__ f, double* __restrict__ out, const LineSet ls,
            unsigned* __restrict__ status) {
    using AR = ArDF;
    using V = dfv;
    constexpr int H = NP;
    constexpr int HM = M / 2;                     // rows per half
    constexpr int SL = half_lane_stride(HM, NP);  // 16-byte units per lane
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ns = cp.ns, P = cp.P, L = cp.L;
    const int LT = half_line_stride(P, HM, NP);               // 16-byte units per line
    float4* ctab = reinterpret_cast<float4*>(smem_raw);      // pf1, pf2 (row j), pb1, pb2 (distance d), HM each
    float4* tile = ctab + 4 * HM;                             // L lines x P lanes x SL
    __shared__ int lexp[kLineThreadsCirc];
    __shared__ long base_in[kLineThreadsCirc], base_out[kLineThreadsCirc];

    const int tid = threadIdx.x, nth = blockDim.x;
    const long line0 = (long)blockIdx.x * L;
    const int nl = (int)min((long)L, ls.nlines - line0);
    if (tid < L) {
        lexp[tid] = 0;
        const long lg = line0 + tid;
        const long a = lg % ls.na, b = lg / ls.na;
        base_in[tid] = a * ls.fa + b * ls.fb;
        base_out[tid] = a * ls.oa + b * ls.ob;
    }
    if (tid < 4 * HM) {
        const int k = tid / HM, j = tid % HM;
        const F2 c = (k < 2 ? cp.phf : cp.phb)[2 * j + (k & 1)];
        ctab[tid] = make_float4(c.h, c.h, c.l, c.l);
    }
    __syncthreads();

    // ---- A: stage each line scaled by 2^-(e_max - 1023); row q of chunk t goes to pair
    // q % HM, component q / HM of lane t's window ----
    auto hpos = [&](int l, int p) -> int {  // float index of row p's high part (p >= 0)
        const unsigned t = (unsigned)p / M, q = (unsigned)p % M;
        return ((l * LT + (int)t * SL + H + (int)(q % HM)) << 2) + (int)(q / HM);
    };
    float* tf = reinterpret_cast<float*>(tile);
    unsigned bad = 0;
    if (ls.fp == 1) {
        const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
        const int U = (ns + 31) >> 5;
        for (int l = warp; l < nl; l += nw) {
            const double* src = f + base_in[l];
            double v[kHalfRowsContig];
            int mx = 0;
#pragma unroll
            for (int u = 0; u < kHalfRowsContig; u++) {
                v[u] = (u < U && lane + 32 * u < ns) ? __ldg(src + lane + 32 * u) : 0.0;
                mx = max(mx, bexp(v[u]));
            }
            mx = (int)__reduce_max_sync(0xffffffffu, (unsigned)mx);
            bad |= (unsigned)(mx == 2047);
            if (lane == 0) lexp[l] = mx;
            const SplitK sk = split_consts(mx - 1023);
            float* lf = tf + hpos(l, lane);
#pragma unroll
            for (int u = 0; u < kHalfRowsContig; u++) {
                if (u < U && lane + 32 * u < ns) {
                    const dfv d = df_split_line(v[u], sk);
                    lf[u * (32 / M) * SL * 4] = d.h;
                    lf[u * (32 / M) * SL * 4 + 2] = d.l;
                }
            }
        }
    } else {
        // strided lines by pairs: thread q0 of a line loads both rows of pairs k = q0 + pstep i,
        // rows p = (k / HM) M + k % HM and p + HM, and writes each pair with one 16-byte store
        // (the lines of a quarter-warp on distinct banks; ns is a multiple of M, and
        // ceil(ns / pstep) <= M gives every pair a thread)
        const int pstep = nth / L;
        const int nk = ns >> 1;
        const int l = tid % L, q0 = tid / L;
        const int fs = (int)ls.fp;  // row offsets in 32 bits (the launchers check that they fit)
        double v[M];
        int mx = 0;
        if (l < nl) {
            const double* src = f + base_in[l];
#pragma unroll
            for (int i = 0; i < HM; i++) {
                const int k = q0 + pstep * i;
                const int p = (k / HM) * M + k % HM;
                const bool ok = k < nk;
                v[2 * i] = ok ? __ldg(src + p * fs) : 0.0;
                v[2 * i + 1] = ok ? __ldg(src + (p + HM) * fs) : 0.0;
                mx = max(mx, max(bexp(v[2 * i]), bexp(v[2 * i + 1])));
            }
            atomicMax(&lexp[l], mx);
        }
        __syncthreads();
        if (l < nl) {
            const int mxl = lexp[l];
            bad |= (unsigned)(mxl == 2047);
            const SplitK sk = split_consts(mxl - 1023);
            float4* lt = tile + (size_t)l * LT + H;
#pragma unroll
            for (int i = 0; i < HM; i++) {
                const int k = q0 + pstep * i;
                if (k < nk) {
                    const dfv a = df_split_line(v[2 * i], sk), b = df_split_line(v[2 * i + 1], sk);
                    lt[(k / HM) * SL + k % HM] = make_float4(a.h, b.h, a.l, b.l);
                }
            }
        }
    }
    __syncthreads();

    const int t = tid % cp.Pp, l = tid / cp.Pp;
    const bool active = (l < nl) && (t < P);
    float4* wp = tile + (size_t)l * LT + t * SL + H;  // pair r at wp[r], -H <= r < HM + H

    // ---- halo pairs: rows -H..-1 (previous chunk, around the ring) beside rows HM-H..HM-1,
    // and rows HM..HM-1+H beside rows M..M-1+H (next chunk) ----
    // (row -h is component B of the previous lane's pair HM - h, row HM - h component A of
    // this lane's; row HM - 1 + h component B of this lane's pair h - 1, row M - 1 + h
    // component A of the next lane's: two 16-byte loads and one store per halo pair)
    if (active) {
        const float4* wprev = tile + (size_t)l * LT + (t == 0 ? P - 1 : t - 1) * SL + H;
        const float4* wnext = tile + (size_t)l * LT + (t == P - 1 ? 0 : t + 1) * SL + H;
#pragma unroll
        for (int h = 1; h <= H; h++) {
            const float4 pv = wprev[HM - h], oa = wp[HM - h], ob = wp[h - 1], nx = wnext[h - 1];
            wp[-h] = make_float4(pv.y, oa.x, pv.w, oa.z);
            float4 hi = make_float4(ob.y, nx.x, ob.w, nx.z);
            if constexpr (STG > 0) {
                if (t == P - 1 && h == 1 && cp.xdup) {
                    const double v = __ldg(f + base_in[l] + (long)ns * ls.fp);
                    bad |= (unsigned)(bexp(v) == 2047);
                    const dfv d = df_from_double_shift(v, lexp[l] - 1023);
                    hi.y = d.h;
                    hi.w = d.l;
                }
            }
            wp[HM - 1 + h] = hi;
        }
    }
    // the neighbouring lanes of a line (one warp) read this lane's first and last rows
    // before its work pairs overwrite them
    __syncwarp();

    df2 cc[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) cc[k] = d2_bcast(cp.c[k]);
    const df2 c0 = d2_bcast(cp.c0);
    const df2 a1 = d2_bcast(cp.ca1), a2 = d2_bcast(cp.ca2);
    const dfv a1s = AR::coef(cp.ca1), a2s = AR::coef(cp.ca2);
    const int Pp = cp.Pp;

    // ---- B: right-hand side and forward recurrence of both halves from zero states ----
    df2 S1 = d2_zero(), S2 = d2_zero();
    if (active) {
#pragma unroll 4
        for (int j = 0; j < HM; j++) {
            const df2 r = half_stencil<NP, SYM, STG>([&](int k) { return d2_of(wp[j + k]); }, cc, c0);
            const df2 y = (Q == 2) ? d2_fms2(r, a1, S1, a2, S2) : d2_fms1(r, a1, S1);
            wp[j - H] = d2_f4(y);
            S2 = S1;
            S1 = y;
        }
    }
    // the chunk's outgoing state: half B's end plus half A's end carried through half B
    const dfv yA15 = d2_x(S1), yA14 = d2_x(S2);
    V s1, s2 = AR::zero();
    {
        const dfv p15a = d2c_scalar(ctab[HM - 1]), p14a = d2c_scalar(ctab[HM - 2]);
        if constexpr (Q == 2) {
            const dfv p15b = d2c_scalar(ctab[HM + HM - 1]), p14b = d2c_scalar(ctab[HM + HM - 2]);
            s1 = AR::mac2(d2_y(S1), p15a, yA15, p15b, yA14);
            s2 = AR::mac2(d2_y(S2), p14a, yA15, p14b, yA14);
        } else {
            s1 = AR::mac1(d2_y(S1), p15a, yA15);
        }
    }
    // ---- D: log-step scan of the chunk transfers (then the ring wrap) ----
    ScanCoefs<Q> fsc;
    {
        unsigned take = 0;  // steps k with t >= 2^k
        for (int k = 0; k < kMaxSteps; k++) take |= (t >= (1 << k) ? 1u : 0u) << k;
        fsc.load(cp.fscan, t, 0, cp.nsteps, take);
    }
#pragma unroll
    for (int k = 0; k < kMaxSteps; k++) {
        if (k >= cp.nsteps) break;
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_up(s1, dlt, Pp);
        const V o2 = (Q == 2) ? AR::shfl_up(s2, dlt, Pp) : AR::zero();
        if (t >= (int)dlt) {
            const F2* Fm = fsc.m[k];
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
    V i1 = AR::shfl_up(s1, 1, Pp);
    V i2 = (Q == 2) ? AR::shfl_up(s2, 1, Pp) : AR::zero();
    if (t == 0) {
        i1 = AR::zero();
        i2 = AR::zero();
    }
    {
        const V E1 = AR::shfl_idx(s1, P - 1, Pp);
        const V E2 = (Q == 2) ? AR::shfl_idx(s2, P - 1, Pp) : AR::zero();
        if (t < P) {
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
    }
    // incoming states: half A the chunk's, half B half A's corrected end rows 15 and 14
    df2 I1, I2;
    {
        const dfv p15a = d2c_scalar(ctab[HM - 1]), p14a = d2c_scalar(ctab[HM - 2]);
        if constexpr (Q == 2) {
            const dfv p15b = d2c_scalar(ctab[HM + HM - 1]), p14b = d2c_scalar(ctab[HM + HM - 2]);
            I1 = d2_pack(i1, AR::mac2(yA15, p15a, i1, p15b, i2));
            I2 = d2_pack(i2, AR::mac2(yA14, p14a, i1, p14b, i2));
        } else {
            I1 = d2_pack(i1, AR::mac1(yA15, p15a, i1));
            I2 = d2_zero();
        }
    }
    // ---- E+F: forward correction and backward recurrence of both halves from zero states ----
    df2 U1 = d2_zero(), U2 = d2_zero();
    if (active) {
#pragma unroll 2
        for (int j = HM - 1; j >= 0; j--) {
            const df2 p1 = d2_of(ctab[j]);
            const df2 w = d2_of(wp[j - H]);
            df2 y;
            if constexpr (Q == 2) {
                y = d2_mac2(w, p1, I1, d2_of(ctab[HM + j]), I2);
            } else {
                y = d2_mac1(w, p1, I1);
            }
            const df2 x = (Q == 2) ? d2_fms2(y, a1, U1, a2, U2) : d2_fms1(y, a1, U1);
            wp[j - H] = d2_f4(x);
            U2 = U1;
            U1 = x;
        }
    }
    // outgoing backward state (rows 0 and 1): half A's plus half B's rows 16, 17 carried up
    const dfv xB0 = d2_y(U1), xB1 = d2_y(U2);
    V u1, u2 = AR::zero();
    {
        const dfv q15a = d2c_scalar(ctab[2 * HM + HM - 1]), q14a = d2c_scalar(ctab[2 * HM + HM - 2]);
        if constexpr (Q == 2) {
            const dfv q15b = d2c_scalar(ctab[3 * HM + HM - 1]), q14b = d2c_scalar(ctab[3 * HM + HM - 2]);
            u1 = AR::mac2(d2_x(U1), q15a, xB0, q15b, xB1);
            u2 = AR::mac2(d2_x(U2), q14a, xB0, q14b, xB1);
        } else {
            u1 = AR::mac1(d2_x(U1), q15a, xB0);
        }
    }
    // ---- G: reverse scan (then the ring wrap) ----
    ScanCoefs<Q> bsc;
    {
        unsigned take = 0;  // steps k with t + 2^k < Pp
        for (int k = 0; k < kMaxSteps; k++) take |= (t + (1 << k) < Pp ? 1u : 0u) << k;
        bsc.load(cp.bscan, t, 0, cp.nsteps, take);
    }
#pragma unroll
    for (int k = 0; k < kMaxSteps; k++) {
        if (k >= cp.nsteps) break;
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_down(u1, dlt, Pp);
        const V o2 = (Q == 2) ? AR::shfl_down(u2, dlt, Pp) : AR::zero();
        if (t + (int)dlt < Pp) {
            const F2* Bm = bsc.m[k];
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
    V j1 = AR::shfl_down(u1, 1, Pp);
    V j2 = (Q == 2) ? AR::shfl_down(u2, 1, Pp) : AR::zero();
    if (t >= P - 1) {
        j1 = AR::zero();
        j2 = AR::zero();
    }
    {
        const V F1 = AR::shfl_idx(u1, 0, Pp);
        const V F2v = (Q == 2) ? AR::shfl_idx(u2, 0, Pp) : AR::zero();
        if (t < P) {
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
    }
    // incoming backward states: half B the chunk's, half A half B's corrected rows 16, 17
    df2 J1, J2;
    {
        const dfv q15a = d2c_scalar(ctab[2 * HM + HM - 1]), q14a = d2c_scalar(ctab[2 * HM + HM - 2]);
        if constexpr (Q == 2) {
            const dfv q15b = d2c_scalar(ctab[3 * HM + HM - 1]), q14b = d2c_scalar(ctab[3 * HM + HM - 2]);
            J1 = d2_pack(AR::mac2(xB0, q15a, j1, q15b, j2), j1);
            J2 = d2_pack(AR::mac2(xB1, q14a, j1, q14b, j2), j2);
        } else {
            J1 = d2_pack(AR::mac1(xB0, q15a, j1), j1);
            J2 = d2_zero();
        }
    }
    // ---- H+I: backward correction and FP64 assembly (rows j and j + 16 over work pair j) ----
    // (Running this last correction in FP64 on the assembled values, two FMAs per row, was
    // measured slower: 0.153 -> 0.166 ms per 256^3 launch along x; the whole CTA reaches the
    // phase at once and the FP64 pipe saturates there.)
    if (active) {
        const int kl = lexp[l] - 1023;
        double2* wd = reinterpret_cast<double2*>(wp - H);
        if (kl >= -800 && kl <= 800) {
            const unsigned kadd = (unsigned)(896 + kl) << 20;
#pragma unroll 2
            for (int j = 0; j < HM; j++) {
                const int d = HM - 1 - j;
                const df2 w = d2_of(wp[j - H]);
                const df2 x = (Q == 2) ? d2_mac2(w, d2_of(ctab[2 * HM + d]), J1, d2_of(ctab[3 * HM + d]), J2)
                                       : d2_mac1(w, d2_of(ctab[2 * HM + d]), J1);
                wd[j] = make_double2(df_to_double_kadd(d2_x(x), kadd), df_to_double_kadd(d2_y(x), kadd));
            }
        } else {
#pragma unroll 1
            for (int j = 0; j < HM; j++) {
                const int d = HM - 1 - j;
                const df2 w = d2_of(wp[j - H]);
                const df2 x = (Q == 2) ? d2_mac2(w, d2_of(ctab[2 * HM + d]), J1, d2_of(ctab[3 * HM + d]), J2)
                                       : d2_mac1(w, d2_of(ctab[2 * HM + d]), J1);
                wd[j] = make_double2(AR::store_scaled(d2_x(x), kl), AR::store_scaled(d2_y(x), kl));
            }
        }
    }
    __syncthreads();

    // ---- J: coalesced stores ----
    half_store<M, RESID>(tile, LT, SL, nl, L, ns, cp.nout, f, out, base_in, base_out, ls);
    if (bad) atomicOr(status, 1u);
}

template <int Q, int NP, bool SYM, int M, bool RESID = false, int STG = 0>
int launch_lhalf_t(const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                   cudaStream_t s) {
    constexpr int NT = kLineThreadsCirc;
    const long blocks = (ls.nlines + c.L - 1) / c.L;
    const size_t smem = sizeof(float4) * (4 * (M / 2) + (size_t)c.L * half_line_stride(c.P, M / 2, NP));
    auto kern = k_lhalf<Q, NP, SYM, M, RESID, STG>;
    // the opt-in covers dynamic plus static shared memory (the per-line arrays, 2.5 KB)
    if (smem + 4096 > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
    }
    kern<<<(unsigned)blocks, NT, smem, s>>>(c, (const double*)f, (double*)out, ls, status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}


// ------------------------------------------------------------------------------------
// Banded (non-periodic) lines: the same pairing on the 16-row chunk plan, two chunks per
// lane (chunk 2t is half A, chunk 2t + 1 half B); the plan's own log-step scan is kept, its
// step 0 (chunk 2t + 1 after chunk 2t) inside the lane and steps k >= 1 across lanes
// 2^(k-1) apart.  The nine per-row tables (g, a1, a2, b1, b2, pf1, pf2, pb1, pb2) of a banded
// line differ from row to row only near its ends: the LU factors and the chunk fundamental
// solutions converge to a fixed pattern some rows in from the top (within the first lane for
// cd10, three lanes for cf90, whose matrix is nearly singular at the Nyquist mode) and change
// again only in the closure rows at the bottom.  The plan finds the fewest leading lanes NF
// after which every interior lane's rows equal the last interior lane's within 2^-50 of each
// table's largest value (far below the double-float representation) and ships NF + 2 blocks
// in pair layout: the NF leading lanes' rows, the last lane's and the interior pattern,
// {h(row j), h(row 16 + j), l(row j), l(row 16 + j)} per table and j; 2.3 KB each in shared
// memory instead of 18 KB of per-row tables, which did not fit beside the windows.  The edge
// rows (one-sided closures) are summed in FP64 from the FP64 input as in k_line and replace
// the stencil in their component; halo rows beyond the line ends are zero.
// ------------------------------------------------------------------------------------
constexpr int kHalf = 16;  // rows per half of a 32-row chunk
constexpr int kHalfBandTables = 9;
constexpr int kHalfBandBlock = kHalfBandTables * kHalf;  // float4 per block (first, last, interior)
// blocks sit one 16-byte unit further apart in shared memory than their size: the lanes of a
// line read the same (table, row) of up to NF + 2 different blocks at once, and a stride that
// is a multiple of 128 bytes put all of them on the same banks (one wavefront per block)
constexpr int kHalfBandBlockStride = kHalfBandBlock + 1;

template <int Q, int NP, bool SYM, bool RESID>
__global__ void __launch_bounds__(kLineThreadsCirc, 4)
    k_lhalf_band(const StencilParams cp, const double* __restrict__ f, double* __restrict__ out, const LineSet ls,
                 unsigned* __restrict__ status) {
    using AR = ArDF;
    using V = dfv;
    constexpr int H = NP, M = 32, HM = kHalf;
    constexpr int SL = half_lane_stride(HM, NP);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ns = cp.ns, L = cp.L;
    const int PL = ns / M;         // lanes per line
    const int PLp = cp.Pp >> 1;    // lanes per line, padded to a power of two
    const int LT = half_line_stride(PL, HM, NP);
    const int ne = cp.nlo + cp.nhi, ehi = ns - cp.nhi;
    const int NF = cp.hnf;                                   // leading lanes with tables of their own
    float4* btab = reinterpret_cast<float4*>(smem_raw);     // NF leading lanes, last lane, interior
    float4* tile = btab + (NF + 2) * kHalfBandBlockStride;  // L lines x PL lanes x SL
    V* edge = reinterpret_cast<V*>(tile + (size_t)L * LT);  // L x ne edge-row right-hand sides
    long* base_in = reinterpret_cast<long*>(edge + (size_t)L * ne);
    long* base_out = base_in + L;
    int* lexp = reinterpret_cast<int*>(base_out + L);

    const int tid = threadIdx.x, nth = blockDim.x;
    const long line0 = (long)blockIdx.x * L;
    const int nl = (int)min((long)L, ls.nlines - line0);
    for (int i = tid; i < L; i += nth) {
        lexp[i] = 0;
        const long lg = line0 + i;
        const long a = lg % ls.na, b = lg / ls.na;
        base_in[i] = a * ls.fa + b * ls.fb;
        base_out[i] = a * ls.oa + b * ls.ob;
    }
    {
        const float4* __restrict__ g = reinterpret_cast<const float4*>(cp.hpair);
        for (int i = tid; i < (NF + 2) * kHalfBandBlock; i += nth)
            btab[(i / kHalfBandBlock) * kHalfBandBlockStride + i % kHalfBandBlock] = __ldg(g + i);
    }
    __syncthreads();

    auto hpos = [&](int l, int p) -> int {  // float index of row p's high part (p >= 0)
        const unsigned t = (unsigned)p / M, q = (unsigned)p % M;
        return ((l * LT + (int)t * SL + H + (int)(q % HM)) << 2) + (int)(q / HM);
    };
    float* tf = reinterpret_cast<float*>(tile);
    unsigned bad = 0;
    // ---- A: staging, as for periodic lines ----
    if (ls.fp == 1) {
        const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
        const int U = (ns + 31) >> 5;
        for (int l = warp; l < nl; l += nw) {
            const double* src = f + base_in[l];
            double v[kHalfRowsContig];
            int mx = 0;
#pragma unroll
            for (int u = 0; u < kHalfRowsContig; u++) {
                v[u] = (u < U && lane + 32 * u < ns) ? __ldg(src + lane + 32 * u) : 0.0;
                mx = max(mx, bexp(v[u]));
            }
            mx = (int)__reduce_max_sync(0xffffffffu, (unsigned)mx);
            bad |= (unsigned)(mx == 2047);
            if (lane == 0) lexp[l] = mx;
            const SplitK sk = split_consts(mx - 1023);
            float* lf = tf + hpos(l, lane);
#pragma unroll
            for (int u = 0; u < kHalfRowsContig; u++) {
                if (u < U && lane + 32 * u < ns) {
                    const dfv d = df_split_line(v[u], sk);
                    lf[u * SL * 4] = d.h;
                    lf[u * SL * 4 + 2] = d.l;
                }
            }
        }
    } else {
        // strided lines by pairs: thread q0 of a line loads both rows of pairs k = q0 + pstep i,
        // rows p = (k / HM) M + k % HM and p + HM, and writes each pair with one 16-byte store
        // (the lines of a quarter-warp on distinct banks; ns is a multiple of M, and
        // ceil(ns / pstep) <= M gives every pair a thread)
        const int pstep = nth / L;
        const int nk = ns >> 1;
        const int l = tid % L, q0 = tid / L;
        const int fs = (int)ls.fp;  // row offsets in 32 bits (the launchers check that they fit)
        double v[M];
        int mx = 0;
        if (l < nl) {
            const double* src = f + base_in[l];
#pragma unroll
            for (int i = 0; i < HM; i++) {
                const int k = q0 + pstep * i;
                const int p = (k / HM) * M + k % HM;
                const bool ok = k < nk;
                v[2 * i] = ok ? __ldg(src + p * fs) : 0.0;
                v[2 * i + 1] = ok ? __ldg(src + (p + HM) * fs) : 0.0;
                mx = max(mx, max(bexp(v[2 * i]), bexp(v[2 * i + 1])));
            }
            atomicMax(&lexp[l], mx);
        }
        __syncthreads();
        if (l < nl) {
            const int mxl = lexp[l];
            bad |= (unsigned)(mxl == 2047);
            const SplitK sk = split_consts(mxl - 1023);
            float4* lt = tile + (size_t)l * LT + H;
#pragma unroll
            for (int i = 0; i < HM; i++) {
                const int k = q0 + pstep * i;
                if (k < nk) {
                    const dfv a = df_split_line(v[2 * i], sk), b = df_split_line(v[2 * i + 1], sk);
                    lt[(k / HM) * SL + k % HM] = make_float4(a.h, b.h, a.l, b.l);
                }
            }
        }
    }
    __syncthreads();

    const int t = tid % PLp, l = tid / PLp;
    const bool active = (l < nl) && (t < PL);
    // this lane's tables: its own (leading lanes), the last lane's, or the interior pattern
    const float4* tb = btab + (t < NF ? t : (t >= PL - 1 ? NF : NF + 1)) * kHalfBandBlockStride;
    auto tab = [&](int k, int j) -> df2 { return d2_of(tb[k * HM + j]); };
    float4* wp = tile + (size_t)l * LT + t * SL + H;

    // ---- halo pairs (zero beyond the line ends) ----
    if (active) {
        const float4* wprev = tile + (size_t)l * LT + (t - 1) * SL + H;  // read only when t > 0
        const float4* wnext = tile + (size_t)l * LT + (t + 1) * SL + H;  // read only when t < PL - 1
        const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int h = 1; h <= H; h++) {
            const float4 pv = t > 0 ? wprev[HM - h] : z4, oa = wp[HM - h], ob = wp[h - 1];
            const float4 nx = t < PL - 1 ? wnext[h - 1] : z4;
            wp[-h] = make_float4(pv.y, oa.x, pv.w, oa.z);
            wp[HM - 1 + h] = make_float4(ob.y, nx.x, ob.w, nx.z);
        }
    }
    // ---- edge rows: one-sided right-hand sides in FP64 from the FP64 input, each input
    // scaled by the line's power of two first (exact) ----
    for (int it = tid; it < nl * ne; it += nth) {
        const int ll = it / ne, e = it - ll * ne;
        const double* src = f + base_in[ll];
        const double sc = scalbn(1.0, 1023 - lexp[ll]);
        const int* ti = cp.tidx + e * cp.tw;
        const double* tc = cp.tcd + e * cp.tw;
        double acc = 0.0;
        // the taps' loads in groups of 8 ahead of the (ordered) FMA chain
        for (int k0 = 0; k0 < cp.tw; k0 += 8) {
            double xv[8], cv[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const bool ok = k0 + u < cp.tw;
                const int idx = ok ? __ldg(ti + k0 + u) : 0;
                cv[u] = ok ? __ldg(tc + k0 + u) : 0.0;
                xv[u] = ok ? __ldg(src + (long)idx * ls.fp) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (k0 + u < cp.tw) acc = __fma_rn(cv[u], __dmul_rn(xv[u], sc), acc);
        }
        edge[it] = df_from_double_shift(acc, 0);
    }
    // the neighbouring lanes have read this lane's first and last rows, the edge rows are
    // complete
    __syncthreads();

    df2 cc[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) cc[k] = d2_bcast(cp.c[k]);
    const df2 c0 = d2_bcast(cp.c0);

    // ---- B: right-hand side (edge rows in their component), row scale g, forward
    // recurrence of both halves from zero states ----
    df2 S1 = d2_zero(), S2 = d2_zero();
    if (active) {
        const int iA0 = t * M, iB0 = t * M + HM;
        // (two rows per unrolled step: four measured 1.7-2.7 % slower here, eight slower still)
#pragma unroll 2
        for (int j = 0; j < HM; j++) {
            df2 r = half_stencil<NP, SYM>([&](int k) { return d2_of(wp[j + k]); }, cc, c0);
            if (iA0 + j < cp.nlo) {
                const V e = edge[l * ne + iA0 + j];
                r.h.x = e.h;
                r.l.x = e.l;
            }
            if (iB0 + j >= ehi) {
                const V e = edge[l * ne + cp.nlo + (iB0 + j - ehi)];
                r.h.y = e.h;
                r.l.y = e.l;
            }
            r = d2_mul(r, tab(0, j));
            const df2 y = (Q == 2) ? d2_fms2(r, tab(1, j), S1, tab(2, j), S2) : d2_fms1(r, tab(1, j), S1);
            wp[j - H] = d2_f4(y);
            S2 = S1;
            S1 = y;
        }
    }
    // ---- D: the plan's scan over 16-row chunks; step 0 (chunk 2t + 1 after chunk 2t) in the lane ----
    const dfv yA15 = d2_x(S1), yA14 = d2_x(S2);
    V s1, s2 = AR::zero();
    ScanCoefs<Q> fsc;
    {
        unsigned take = 1u;  // step 0 in the lane, steps k >= 1 with t >= 2^(k-1)
        for (int k = 1; k < kMaxSteps; k++) take |= (t >= (1 << (k - 1)) ? 1u : 0u) << k;
        fsc.load(cp.fscan, 2 * t + 1, 0, cp.nsteps, take);
    }
    {
        const F2* Fm = fsc.m[0];
        if constexpr (Q == 2) {
            s1 = AR::mac2(d2_y(S1), AR::coef(Fm[0]), yA15, AR::coef(Fm[1]), yA14);
            s2 = AR::mac2(d2_y(S2), AR::coef(Fm[2]), yA15, AR::coef(Fm[3]), yA14);
        } else {
            s1 = AR::mac1(d2_y(S1), AR::coef(Fm[0]), yA15);
        }
    }
#pragma unroll
    for (int k = 1; k < kMaxSteps; k++) {
        if (k >= cp.nsteps) break;
        const unsigned dlt = 1u << (k - 1);
        const V o1 = AR::shfl_up(s1, dlt, PLp);
        const V o2 = (Q == 2) ? AR::shfl_up(s2, dlt, PLp) : AR::zero();
        if (t >= (int)dlt) {
            const F2* Fm = fsc.m[k];
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
    V i1 = AR::shfl_up(s1, 1, PLp);
    V i2 = (Q == 2) ? AR::shfl_up(s2, 1, PLp) : AR::zero();
    if (t == 0) {
        i1 = AR::zero();
        i2 = AR::zero();
    }
    // incoming states: half A the lane's, half B half A's corrected rows 15 and 14
    df2 I1, I2;
    {
        const df2 p15 = tab(5, HM - 1), p14 = tab(5, HM - 2);
        if constexpr (Q == 2) {
            const df2 q15 = tab(6, HM - 1), q14 = tab(6, HM - 2);
            I1 = d2_pack(i1, AR::mac2(yA15, d2_x(p15), i1, d2_x(q15), i2));
            I2 = d2_pack(i2, AR::mac2(yA14, d2_x(p14), i1, d2_x(q14), i2));
        } else {
            I1 = d2_pack(i1, AR::mac1(yA15, d2_x(p15), i1));
            I2 = d2_zero();
        }
    }
    // ---- E+F: forward correction and backward recurrence of both halves ----
    df2 U1 = d2_zero(), U2 = d2_zero();
    if (active) {
#pragma unroll 2
        for (int j = HM - 1; j >= 0; j--) {
            const df2 w = d2_of(wp[j - H]);
            const df2 y = (Q == 2) ? d2_mac2(w, tab(5, j), I1, tab(6, j), I2) : d2_mac1(w, tab(5, j), I1);
            const df2 x = (Q == 2) ? d2_fms2(y, tab(3, j), U1, tab(4, j), U2) : d2_fms1(y, tab(3, j), U1);
            wp[j - H] = d2_f4(x);
            U2 = U1;
            U1 = x;
        }
    }
    // ---- G: the plan's reverse scan; step 0 (chunk 2t before chunk 2t + 1) in the lane ----
    const dfv xB0 = d2_y(U1), xB1 = d2_y(U2);
    V u1, u2 = AR::zero();
    ScanCoefs<Q> bsc;
    {
        unsigned take = 1u;  // step 0 in the lane, steps k >= 1 with t + 2^(k-1) < PLp
        for (int k = 1; k < kMaxSteps; k++) take |= (t + (1 << (k - 1)) < PLp ? 1u : 0u) << k;
        bsc.load(cp.bscan, 2 * t, 0, cp.nsteps, take);
    }
    {
        const F2* Bm = bsc.m[0];
        if constexpr (Q == 2) {
            u1 = AR::mac2(d2_x(U1), AR::coef(Bm[0]), xB0, AR::coef(Bm[1]), xB1);
            u2 = AR::mac2(d2_x(U2), AR::coef(Bm[2]), xB0, AR::coef(Bm[3]), xB1);
        } else {
            u1 = AR::mac1(d2_x(U1), AR::coef(Bm[0]), xB0);
        }
    }
#pragma unroll
    for (int k = 1; k < kMaxSteps; k++) {
        if (k >= cp.nsteps) break;
        const unsigned dlt = 1u << (k - 1);
        const V o1 = AR::shfl_down(u1, dlt, PLp);
        const V o2 = (Q == 2) ? AR::shfl_down(u2, dlt, PLp) : AR::zero();
        if (t + (int)dlt < PLp) {
            const F2* Bm = bsc.m[k];
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
    V j1 = AR::shfl_down(u1, 1, PLp);
    V j2 = (Q == 2) ? AR::shfl_down(u2, 1, PLp) : AR::zero();
    if (t >= PL - 1) {
        j1 = AR::zero();
        j2 = AR::zero();
    }
    // incoming backward states: half B the lane's, half A half B's corrected rows 0 and 1
    df2 J1, J2;
    {
        const df2 q0 = tab(7, 0), q1 = tab(7, 1);
        if constexpr (Q == 2) {
            const df2 r0 = tab(8, 0), r1 = tab(8, 1);
            J1 = d2_pack(AR::mac2(xB0, d2_y(q0), j1, d2_y(r0), j2), j1);
            J2 = d2_pack(AR::mac2(xB1, d2_y(q1), j1, d2_y(r1), j2), j2);
        } else {
            J1 = d2_pack(AR::mac1(xB0, d2_y(q0), j1), j1);
            J2 = d2_zero();
        }
    }
    // ---- H+I: backward correction and FP64 assembly (rows j and j + 16 over work pair j) ----
    if (active) {
        const int kl = lexp[l] - 1023;
        double2* wd = reinterpret_cast<double2*>(wp - H);
        if (kl >= -800 && kl <= 800) {
            const unsigned kadd = (unsigned)(896 + kl) << 20;
#pragma unroll 2
            for (int j = 0; j < HM; j++) {
                const df2 w = d2_of(wp[j - H]);
                const df2 x = (Q == 2) ? d2_mac2(w, tab(7, j), J1, tab(8, j), J2) : d2_mac1(w, tab(7, j), J1);
                wd[j] = make_double2(df_to_double_kadd(d2_x(x), kadd), df_to_double_kadd(d2_y(x), kadd));
            }
        } else {
#pragma unroll 1
            for (int j = 0; j < HM; j++) {
                const df2 w = d2_of(wp[j - H]);
                const df2 x = (Q == 2) ? d2_mac2(w, tab(7, j), J1, tab(8, j), J2) : d2_mac1(w, tab(7, j), J1);
                wd[j] = make_double2(AR::store_scaled(d2_x(x), kl), AR::store_scaled(d2_y(x), kl));
            }
        }
    }
    __syncthreads();

    // ---- J: coalesced stores (residual form: f - x) ----
    half_store<M, RESID>(tile, LT, SL, nl, L, ns, ns, f, out, base_in, base_out, ls);
    if (bad) atomicOr(status, 1u);
}

// dynamic shared memory of k_lhalf_band: tables, windows, edge rows, per-line arrays
inline size_t lhalf_band_smem(const StencilParams& c, int np) {
    const size_t tabs = sizeof(float4) * (size_t)(c.hnf + 2) * kHalfBandBlockStride;
    const size_t tile = sizeof(float4) * (size_t)c.L * half_line_stride(c.ns / 32, kHalf, np);
    const size_t edge = sizeof(dfv) * (size_t)c.L * (c.nlo + c.nhi);
    const size_t lines = (2 * sizeof(long) + sizeof(int)) * (size_t)c.L;
    return tabs + tile + ((edge + 7) & ~(size_t)7) + lines;
}

template <int Q, int NP, bool SYM, bool RESID = false>
int launch_lhalf_band_t(const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                        cudaStream_t s) {
    constexpr int NT = kLineThreadsCirc;
    const long blocks = (ls.nlines + c.L - 1) / c.L;
    const size_t smem = lhalf_band_smem(c, NP);
    auto kern = k_lhalf_band<Q, NP, SYM, RESID>;
    if (smem + 1024 > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
    }
    kern<<<(unsigned)blocks, NT, smem, s>>>(c, (const double*)f, (double*)out, ls, status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

int launch_line_half(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s);
int launch_line_half_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                          unsigned* status, cudaStream_t s);

}  // namespace pade
