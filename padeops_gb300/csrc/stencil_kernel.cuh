// Chunked kernel with a compile-time stencil shape (double-float arithmetic with FP64 in
// and out, or FP32 throughout).
//
// The compact derivatives and filters (cd06 / cd10 first and second derivatives, cf90 in
// residual form) have an interior RHS stencil that is symmetric or antisymmetric about the
// row, and a tridiagonal or pentadiagonal LHS.  k_line runs the algorithm of k_chunk
// (forward recurrence from a zero state, log-step scan of the chunk transfers, corrected
// backward recurrence, backward scan, correction) with
//   * the stencil shape as a template (pair k at offsets +-k, optional centre), so the RHS
//     is straight-line code with its coefficients in registers;
//   * each lane's chunk staged with its own halo: periodic lines copy the neighbouring
//     rows around the ring, so every row uses the interior stencil; non-periodic lines
//     take their edge rows (one-sided closures) from a small pre-pass instead;
//   * circulant lines: the recurrence constants in registers and the chunk fundamental
//     solutions per chunk position; banded lines: per-row tables in shared memory, laid
//     out chunk by chunk with an odd stride (conflict-free, like the work rows);
//   * a shift-and-assemble FP64 store without range checks for line scales within
//     2^+-800 (the checked path otherwise).
// Operators without residual form write their work rows over the input window (row j's
// value at window row j - H, which later rows no longer read), halving the shared memory
// per line.  Lines hold a whole number of chunks (ns = P * M, M = 16 or 32), at most 512
// rows.
#pragma once
#include <cuda_runtime.h>

#include "chunk_kernel.cuh"

namespace pade {

// Lane strides (8-byte words) that keep a half-warp's accesses on distinct banks.  Chunks
// of 16: the 16 lanes of a line fill a half-warp, odd S gives 16 distinct bank pairs.
// Chunks of 32 (8 lanes per line on 256-row lines): two lines share a half-warp; S = 2 mod
// 4 puts one line's 8 lanes on 8 distinct even words and, with the odd line stride, the
// other line's on odd words.
template <int M, int H>
struct LineLayout {
    static constexpr int S0 = M + 2 * H;
    static constexpr int S = M == 32 ? (S0 % 4 == 2 ? S0 : S0 + (4 + 2 - S0 % 4) % 4)
                                     : ((S0 % 2 == 0) ? S0 + 1 : S0);  // input window: H + M + H rows
    static constexpr int W = M + 1;  // work rows / row tables
};
static_assert(LineLayout<32, 3>::S % 4 == 2 && LineLayout<32, 4>::S % 4 == 2 && LineLayout<32, 2>::S % 4 == 2,
              "32-row chunk stride");
static_assert(LineLayout<16, 3>::S % 2 == 1 && LineLayout<16, 4>::S % 2 == 1, "16-row chunk stride");

// RHS of one row: pairs k = 1..NP at offsets (k, -k) about the row (STG = 0), or about a
// half point: (k, 1 - k) (STG = +1, edges to cells) or (k - 1, -k) (STG = -1, cells to edges)
template <class AR, int NP, bool SYM, int STG = 0>
__device__ __forceinline__ typename AR::V line_stencil(const typename AR::V* __restrict__ p,
                                                      const typename AR::V (&c)[NP], typename AR::V c0) {
    typename AR::V acc;
    if constexpr (STG != 0) {
        constexpr int sh = STG > 0 ? 0 : -1;
        acc = SYM ? AR::mul(AR::add(p[1 + sh], p[sh]), c[0]) : AR::mul(AR::sub(p[1 + sh], p[sh]), c[0]);
#pragma unroll
        for (int k = 2; k <= NP; k++) {
            const typename AR::V d = SYM ? AR::add(p[k + sh], p[1 - k + sh]) : AR::sub(p[k + sh], p[1 - k + sh]);
            acc = AR::add(acc, AR::mul(d, c[k - 1]));
        }
    } else if constexpr (SYM) {
        acc = AR::mul(p[0], c0);
#pragma unroll
        for (int k = 1; k <= NP; k++) acc = AR::add(acc, AR::mul(AR::add(p[k], p[-k]), c[k - 1]));
    } else {
        acc = AR::mul(AR::sub(p[1], p[-1]), c[0]);
#pragma unroll
        for (int k = 2; k <= NP; k++) acc = AR::add(acc, AR::mul(AR::sub(p[k], p[-k]), c[k - 1]));
    }
    return AR::norm(acc);
}

// Line stride in 8-byte words, made odd.
__host__ __device__ constexpr int line_stride(int n) { return n % 2 == 0 ? n + 1 : n; }

// Resident CTAs per SM the register allocation is sized for (what shared memory allows):
// lines with the input window reused and chunks of 16 hold about 3 KB per line.
__host__ __device__ constexpr int line_min_blocks(bool circ, int m, bool alias) {
    return circ ? ((alias && m == 16) ? 7 : 5) : ((alias && m == 16) ? 3 : 2);
}

// Number of per-row tables of a banded line: g a1 a2 b1 b2 pf1 pf2 pb1 pb2.
constexpr int kRowTables = 9;

template <class AR, int Q, int NP, bool SYM, bool CIRC, int M, int NT, bool ALIAS, int STG = 0>
__global__ void __launch_bounds__(NT, line_min_blocks(CIRC, M, ALIAS))
    k_line(const StencilParams cp, const typename AR::IO* __restrict__ f, typename AR::IO* __restrict__ out,
           const LineSet ls, unsigned* __restrict__ status) {
    using V = typename AR::V;
    using IO = typename AR::IO;
    constexpr int H = NP;
    constexpr int S = LineLayout<M, H>::S, W = LineLayout<M, H>::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ns = cp.ns, P = cp.P, L = cp.L;
    const int PW = P * W;                      // one row table (banded)
    // odd line strides: strided staging and stores put consecutive lines on distinct banks
    const int LT = line_stride(P * S), LW = line_stride(PW);
    const int ne = cp.nlo + cp.nhi;            // edge rows (banded)
    V* tab = reinterpret_cast<V*>(smem_raw);   // circulant: phf, phb (M x 2 each); banded: 9 x PW
    V* tile = tab + (CIRC ? 4 * M : kRowTables * PW);  // L lines x (P windows x S), stride LT
    // separate work rows (residual form); otherwise chunk row j's work value overwrites
    // window row j - H, which no later row of the chunk reads
    V* work = tile + (size_t)L * LT;                    // L lines x (P chunks x W), stride LW
    V* edge = work + (ALIAS ? 0 : (size_t)L * LW);      // banded: L x ne edge-row RHS values
    __shared__ int lexp[NT];
    __shared__ long base_in[NT], base_out[NT];

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
    if constexpr (CIRC) {
        for (int i = tid; i < 2 * M; i += nth) {
            tab[i] = AR::coef(cp.phf[i]);
            tab[2 * M + i] = AR::coef(cp.phb[i]);
        }
    } else {
        for (int i = tid; i < ns; i += nth) {
            const int ps = (i / M) * W + (i % M);
#pragma unroll
            for (int k = 0; k < 5; k++) tab[k * PW + ps] = AR::coef(cp.rc[i * 5 + k]);
            tab[5 * PW + ps] = AR::coef(cp.phf[i * 2]);
            tab[6 * PW + ps] = AR::coef(cp.phf[i * 2 + 1]);
            tab[7 * PW + ps] = AR::coef(cp.phb[i * 2]);
            tab[8 * PW + ps] = AR::coef(cp.phb[i * 2 + 1]);
        }
    }
    __syncthreads();

    // ---- A: stage each line scaled by 2^-(e_max - 1023) into the main rows of the windows ----
    auto main_pos = [&](int l, int p) -> int { return l * LT + (p / M) * S + H + (p % M); };
    unsigned bad = 0;
    if constexpr (AR::kScaled) {
        if (ls.fp == 1) {
            const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
            const int U = (ns + 31) >> 5;
            for (int l = warp; l < nl; l += nw) {
                const double* src = f + base_in[l];
                double v[kStageRegs];
                int mx = 0;
    #pragma unroll
                for (int u = 0; u < kStageRegs; u++) {
                    const int p = lane + 32 * u;
                    v[u] = (u < U && p < ns) ? __ldg(src + p) : 0.0;
                    mx = max(mx, bexp(v[u]));
                }
                mx = (int)__reduce_max_sync(0xffffffffu, (unsigned)mx);
                bad |= (unsigned)(mx == 2047);
                if (lane == 0) lexp[l] = mx;
                const SplitK sk = split_consts(mx - 1023);
    #pragma unroll
                for (int u = 0; u < kStageRegs; u++) {
                    const int p = lane + 32 * u;
                    if (u < U && p < ns) tile[main_pos(l, p)] = df_split_line(v[u], sk);
                }
            }
        } else if ((ns + nth / L - 1) / (nth / L) > kStageRegs) {
            // more rows per thread than staging registers: raw FP64 first, split in place
            const int pstep = nth / L;
            const int l = tid % L, q0 = tid / L;
            double* raw = reinterpret_cast<double*>(tile);
            int mx = 0;
            if (l < nl) {
                const double* src = f + base_in[l];
                for (int p0 = q0; p0 < ns; p0 += pstep * kLoadUnroll) {
                    double v[kLoadUnroll];
    #pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + pstep * u;
                        v[u] = p < ns ? __ldg(src + (long)p * ls.fp) : 0.0;
                    }
    #pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + pstep * u;
                        if (p < ns) {
                            raw[main_pos(l, p)] = v[u];
                            mx = max(mx, bexp(v[u]));
                        }
                    }
                }
                atomicMax(&lexp[l], mx);
            }
            __syncthreads();
            if (l < nl) {
                const int k = lexp[l] - 1023;
                bad |= (unsigned)(lexp[l] == 2047);
                const SplitK sk = split_consts(k);
                for (int p = q0; p < ns; p += pstep) {
                    const int ps = main_pos(l, p);
                    tile[ps] = df_split_line(raw[ps], sk);
                }
            }
        } else {
            const int pstep = nth / L;
            const int U = (ns + pstep - 1) / pstep;
            const int l = tid % L, q0 = tid / L;
            double v[kStageRegs];
            int mx = 0;
            if (l < nl) {
                const double* src = f + base_in[l];
    #pragma unroll
                for (int u = 0; u < kStageRegs; u++) {
                    const int p = q0 + pstep * u;
                    v[u] = (u < U && p < ns) ? __ldg(src + (long)p * ls.fp) : 0.0;
                    mx = max(mx, bexp(v[u]));
                }
                atomicMax(&lexp[l], mx);
            }
            __syncthreads();
            if (l < nl) {
                const int k = lexp[l] - 1023;
                bad |= (unsigned)(lexp[l] == 2047);
                const SplitK sk = split_consts(k);
    #pragma unroll
                for (int u = 0; u < kStageRegs; u++) {
                    const int p = q0 + pstep * u;
                    if (u < U && p < ns) tile[main_pos(l, p)] = df_split_line(v[u], sk);
                }
            }
        }
    } else {
        // FP32 in and out: no line scaling, values stored as loaded
        if (ls.fp == 1) {
            const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
            for (int l = warp; l < nl; l += nw) {
                const IO* src = f + base_in[l];
#pragma unroll 4
                for (int p = lane; p < ns; p += 32) tile[main_pos(l, p)] = AR::load(__ldg(src + p), bad);
            }
        } else {
            const int pstep = nth / L;
            const int l = tid % L, q0 = tid / L;
            if (l < nl) {
                const IO* src = f + base_in[l];
#pragma unroll 4
                for (int p = q0; p < ns; p += pstep) tile[main_pos(l, p)] = AR::load(__ldg(src + (long)p * ls.fp), bad);
            }
        }
    }
    __syncthreads();

    const int t = tid % cp.Pp, l = tid / cp.Pp;
    const bool active = (l < nl) && (t < P);
    V* win = tile + (size_t)l * LT + t * S + H;  // row j of the chunk at win[j], -H <= j < M + H
    V* wk = ALIAS ? win - H : work + (size_t)l * LW + t * W;
    const V* rt = tab + t * W;                    // banded: row tables of this chunk, rt[k * PW + j]

    // ---- halo of the window: ring neighbours (periodic) or zeros (non-periodic) ----
    if (active) {
#pragma unroll
        for (int h = 1; h <= H; h++) {
            const int p = t * M - h, q = t * M + M - 1 + h;
            if constexpr (CIRC) {
                win[-h] = tile[main_pos(l, p < 0 ? p + ns : p)];
                win[M - 1 + h] = tile[main_pos(l, q >= ns ? q - ns : q)];
                if constexpr (STG > 0 && AR::kScaled) {
                    if (q == ns && cp.xdup) {
                        const double v = __ldg(f + base_in[l] + (long)ns * ls.fp);
                        bad |= (unsigned)(bexp(v) == 2047);
                        win[M - 1 + h] = df_from_double_shift(v, lexp[l] - 1023);
                    }
                }
            } else {
                win[-h] = p < 0 ? AR::zero() : tile[main_pos(l, p)];
                win[M - 1 + h] = q >= ns ? AR::zero() : tile[main_pos(l, q)];
            }
        }
    }
    // ---- banded: RHS of the edge rows (explicit one-sided closures) ----
    // The double-float path sums them in FP64 from the FP64 input (re-read, in L1/L2 after
    // the staging): a one-sided second-derivative row adds terms ~1/h^2 larger than its
    // result, and the 48-bit split of the input would lose 5 bits of that cancellation.
    if constexpr (!CIRC) {
        for (int it = tid; it < nl * ne; it += nth) {
            const int ll = it / ne, e = it - ll * ne;
            if constexpr (AR::kScaled) {
                // inputs scaled by the line's power of two first (exact), so no product or
                // partial sum of a tiny line falls into the subnormal range
                const double* src = reinterpret_cast<const double*>(f) + base_in[ll];
                const double sc = scalbn(1.0, 1023 - lexp[ll]);
                double acc = 0.0;
#pragma unroll 1
                for (int k = 0; k < cp.tw; k++) {
                    const int idx = __ldg(cp.tidx + e * cp.tw + k);
                    acc = __fma_rn(__ldg(cp.tcd + e * cp.tw + k), __dmul_rn(__ldg(src + (long)idx * ls.fp), sc), acc);
                }
                edge[it] = df_from_double_shift(acc, 0);
            } else {
                V acc = AR::zero();
#pragma unroll 1
                for (int k = 0; k < cp.tw; k++) {
                    const int idx = __ldg(cp.tidx + e * cp.tw + k);
                    acc = AR::add(acc, AR::mul(tile[main_pos(ll, idx)], AR::coef(cp.tc[e * cp.tw + k])));
                }
                edge[it] = AR::norm(acc);
            }
        }
        __syncthreads();
    }

    V cc[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) cc[k] = AR::coef(cp.c[k]);
    const V c0 = AR::coef(cp.c0);
    const V a1 = AR::coef(cp.ca1), a2 = AR::coef(cp.ca2);
    const int Pp = cp.Pp;

    // ---- B: right-hand side and forward recurrence from a zero state ----
    V s1 = AR::zero(), s2 = AR::zero();
    if (active) {
        const int nlo = cp.nlo, ehi = ns - cp.nhi;
#pragma unroll 4
        for (int j = 0; j < M; j++) {
            V y;
            if constexpr (CIRC) {
                const V r = line_stencil<AR, NP, SYM, STG>(win + j, cc, c0);
                y = (Q == 2) ? AR::fms2(r, a1, s1, a2, s2) : AR::fms1(r, a1, s1);
            } else {
                const int i = t * M + j;
                V r;
                if (i < nlo) r = edge[l * ne + i];
                else if (i >= ehi) r = edge[l * ne + nlo + (i - ehi)];
                else r = line_stencil<AR, NP, SYM, STG>(win + j, cc, c0);
                r = AR::mul(r, rt[j]);
                y = (Q == 2) ? AR::fms2(r, rt[PW + j], s1, rt[2 * PW + j], s2) : AR::fms1(r, rt[PW + j], s1);
            }
            wk[j] = y;
            s2 = s1;
            s1 = y;
        }
    }
    // ---- D: log-step scan of the chunk transfers (then the ring wrap, periodic) ----
    for (int k = 0; k < cp.nsteps; k++) {
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_up(s1, dlt, Pp);
        const V o2 = (Q == 2) ? AR::shfl_up(s2, dlt, Pp) : AR::zero();
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
    V i1 = AR::shfl_up(s1, 1, Pp);
    V i2 = (Q == 2) ? AR::shfl_up(s2, 1, Pp) : AR::zero();
    if (t == 0) {
        i1 = AR::zero();
        i2 = AR::zero();
    }
    if constexpr (CIRC) {
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
    // ---- E+F: forward correction and backward recurrence from a zero state ----
    V u1 = AR::zero(), u2 = AR::zero();
    if (active) {
#pragma unroll 4
        for (int j = M - 1; j >= 0; j--) {
            V p1, p2, b1 = a1, b2 = a2;
            if constexpr (CIRC) {
                p1 = tab[2 * j];
                p2 = tab[2 * j + 1];
            } else {
                p1 = rt[5 * PW + j];
                p2 = rt[6 * PW + j];
                b1 = rt[3 * PW + j];
                b2 = rt[4 * PW + j];
            }
            const V y = (Q == 2) ? AR::mac2(wk[j], p1, i1, p2, i2) : AR::mac1(wk[j], p1, i1);
            const V x = (Q == 2) ? AR::fms2(y, b1, u1, b2, u2) : AR::fms1(y, b1, u1);
            wk[j] = x;
            u2 = u1;
            u1 = x;
        }
    }
    // ---- G: reverse scan (then the ring wrap, periodic) ----
    for (int k = 0; k < cp.nsteps; k++) {
        const unsigned dlt = 1u << k;
        const V o1 = AR::shfl_down(u1, dlt, Pp);
        const V o2 = (Q == 2) ? AR::shfl_down(u2, dlt, Pp) : AR::zero();
        if (t + (int)dlt < Pp) {
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
    V j1 = AR::shfl_down(u1, 1, Pp);
    V j2 = (Q == 2) ? AR::shfl_down(u2, 1, Pp) : AR::zero();
    if (t >= P - 1) {
        j1 = AR::zero();
        j2 = AR::zero();
    }
    if constexpr (CIRC) {
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
    // ---- H+I: backward correction, residual form, FP64 assembly (in place) ----
    auto corrected = [&](int j) -> V {
        V q1, q2;
        if constexpr (CIRC) {
            q1 = tab[2 * M + 2 * (M - 1 - j)];
            q2 = tab[2 * M + 2 * (M - 1 - j) + 1];
        } else {
            q1 = rt[7 * PW + j];
            q2 = rt[8 * PW + j];
        }
        return (Q == 2) ? AR::mac2(wk[j], q1, j1, q2, j2) : AR::mac1(wk[j], q1, j1);
    };
    if (active) {
        IO* wio = reinterpret_cast<IO*>(wk);
        if constexpr (AR::kScaled) {
            const int kl = lexp[l] - 1023;
            if (kl >= -800 && kl <= 800) {
                const unsigned kadd = (unsigned)(896 + kl) << 20;
#pragma unroll 4
                for (int j = 0; j < M; j++) {
                    V x = corrected(j);
                    if (!ALIAS && cp.resid) x = df_sub(win[j], x);
                    wio[j] = df_to_double_kadd(x, kadd);
                }
            } else {
#pragma unroll 1
                for (int j = 0; j < M; j++) {
                    V x = corrected(j);
                    if (!ALIAS && cp.resid) x = AR::norm(df_sub(win[j], x));
                    wio[j] = AR::store_scaled(x, kl);
                }
            }
        } else {
#pragma unroll 4
            for (int j = 0; j < M; j++) {
                V x = corrected(j);
                if (!ALIAS && cp.resid) x = AR::sub(win[j], x);
                wio[j] = AR::store(x);
            }
        }
    }
    __syncthreads();

    // ---- J: coalesced stores ----
    const IO* wd = reinterpret_cast<const IO*>(ALIAS ? tile : work);
    auto out_pos = [&](int ll, int p) -> int {
        return ALIAS ? ll * LT + (p / M) * S + (p % M) : ll * LW + (p / M) * W + (p % M);
    };
    if (ls.op == 1) {
        const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
        for (int ll = warp; ll < nl; ll += nw) {
            IO* o = out + base_out[ll];
            for (int p = lane; p < cp.nout; p += 32) o[p] = wd[out_pos(ll, p < ns ? p : p - ns)];
        }
    } else {
        const int ll = tid % L, pstep = nth / L;
        if (ll < nl) {
            IO* o = out + base_out[ll];
            for (int p = tid / L; p < cp.nout; p += pstep) o[(long)p * ls.op] = wd[out_pos(ll, p < ns ? p : p - ns)];
        }
    }
    if (bad) atomicOr(status, 1u);
}

template <class AR, bool CIRC, int NP, int M, bool ALIAS>
size_t line_smem(const StencilParams& c) {
    using Lay = LineLayout<M, NP>;
    const int PW = c.P * Lay::W;
    const size_t tabs = CIRC ? 4 * (size_t)M : kRowTables * (size_t)PW;
    const size_t edges = CIRC ? 0 : (size_t)c.L * (c.nlo + c.nhi);
    const size_t work = ALIAS ? 0 : (size_t)c.L * line_stride(PW);
    return sizeof(typename AR::V) * (tabs + (size_t)c.L * line_stride(c.P * Lay::S) + work + edges);
}

template <class AR, int Q, int NP, bool SYM, bool CIRC, int M, bool ALIAS, int STG = 0>
int launch_line_t(const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                  cudaStream_t s) {
    using IO = typename AR::IO;
    constexpr int NT = CIRC ? kLineThreadsCirc : kLineThreadsBand;
    const long blocks = (ls.nlines + c.L - 1) / c.L;
    const size_t smem = line_smem<AR, CIRC, NP, M, ALIAS>(c);
    auto kern = k_line<AR, Q, NP, SYM, CIRC, M, NT, ALIAS, STG>;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
    }
    kern<<<(unsigned)blocks, NT, smem, s>>>(c, (const IO*)f, (IO*)out, ls, status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

// Dispatch over the instantiated shapes: residual-form cf90 (P4S) with chunks of 16 and
// separate work rows; the others with the input window reused and chunks of 16 or 32.
template <class AR, bool CIRC>
int launch_line_shapes(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                       unsigned* status, cudaStream_t s) {
    const bool m32 = c.M == 32;
    switch (shape) {
        case SHAPE_T2A:
            return m32 ? launch_line_t<AR, 1, 2, false, CIRC, 32, true>(c, f, out, ls, status, s)
                       : launch_line_t<AR, 1, 2, false, CIRC, 16, true>(c, f, out, ls, status, s);
        case SHAPE_T2S:
            return m32 ? launch_line_t<AR, 1, 2, true, CIRC, 32, true>(c, f, out, ls, status, s)
                       : launch_line_t<AR, 1, 2, true, CIRC, 16, true>(c, f, out, ls, status, s);
        case SHAPE_P3A:
            return m32 ? launch_line_t<AR, 2, 3, false, CIRC, 32, true>(c, f, out, ls, status, s)
                       : launch_line_t<AR, 2, 3, false, CIRC, 16, true>(c, f, out, ls, status, s);
        case SHAPE_P3S:
            return m32 ? launch_line_t<AR, 2, 3, true, CIRC, 32, true>(c, f, out, ls, status, s)
                       : launch_line_t<AR, 2, 3, true, CIRC, 16, true>(c, f, out, ls, status, s);
        case SHAPE_P4S: return launch_line_t<AR, 2, 4, true, CIRC, 16, false>(c, f, out, ls, status, s);
        default: return PS_ENOTSUP;
    }
}

int launch_line_circ(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s);
int launch_line_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s);
int launch_line_f32_circ(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                         unsigned* status, cudaStream_t s);
int launch_line_f32_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                         unsigned* status, cudaStream_t s);
// the staggered shapes (double-float, circulant, chunks of 32)
int launch_line_stagg(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                      unsigned* status, cudaStream_t s);

}  // namespace pade
