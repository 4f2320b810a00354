// The chunked scan kernel (the fast path) and its launch templates.
//
// A CTA stages L lines in shared memory; P adjacent lanes per line each own a chunk of M
// rows; the recurrences run twice per chunk around a log-step shuffle scan of the chunk
// transfers.  Arithmetic is double-float (ArDF, FP64 in/out) or FP32 (ArF32).  The
// instantiations are spread over several translation units so they compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "dfmath.cuh"
#include "engine.h"

namespace pade {

// ------------------------------------------------------------------------------------
// arithmetic policies
// ------------------------------------------------------------------------------------
struct ArDF {
    using V = dfv;
    using IO = double;
    // lines are scaled by a power of two so that their maximum is in [1, 2) (exact)
    static constexpr bool kScaled = true;
    static __device__ __forceinline__ V load(double x, unsigned& bad) { return df_from_double(x, bad); }
    static __device__ __forceinline__ double store(V v) { return df_to_double(v); }
    // shift each part on its bits unless the low part could leave the normal FP64 range
    // (lines below ~1e-270), where the sum is formed first and then shifted
    static __device__ __forceinline__ double store_scaled(V v, int k) {
        return k >= -900 ? df_to_double_shift(v, k) : shift_up(df_to_double(v), k);
    }
    static __device__ __forceinline__ V coef(F2 c) { return dfv{c.h, c.l}; }
    static __device__ __forceinline__ V zero() { return df_zero(); }
    static __device__ __forceinline__ V add(V a, V b) { return df_add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return df_sub(a, b); }
    static __device__ __forceinline__ V mul(V a, V c) { return df_mul(a, c); }
    static __device__ __forceinline__ V norm(V a) { return df_norm(a); }
    // base - c1*x1 - c2*x2
    static __device__ __forceinline__ V fms2(V base, V c1, V x1, V c2, V x2) {
        return df_norm(df_sub(df_sub(base, df_mul(x1, c1)), df_mul(x2, c2)));
    }
    static __device__ __forceinline__ V fms1(V base, V c1, V x1) { return df_norm(df_sub(base, df_mul(x1, c1))); }
    // acc + M * v for a 2x2 matrix m (row-major) acting on (v1, v2)
    static __device__ __forceinline__ V mac2(V acc, V m0, V v1, V m1, V v2) {
        return df_norm(df_add(df_add(acc, df_mul(v1, m0)), df_mul(v2, m1)));
    }
    static __device__ __forceinline__ V mac1(V acc, V m0, V v1) { return df_norm(df_add(acc, df_mul(v1, m0))); }
    static __device__ __forceinline__ V shfl_up(V v, unsigned d, int w) { return df_shfl_up(v, d, w); }
    static __device__ __forceinline__ V shfl_down(V v, unsigned d, int w) { return df_shfl_down(v, d, w); }
    static __device__ __forceinline__ V shfl_idx(V v, int s, int w) { return df_shfl_idx(v, s, w); }
};

struct ArF32 {
    using V = float;
    using IO = float;
    static constexpr bool kScaled = false;
    static __device__ __forceinline__ V load(float x, unsigned&) { return x; }
    static __device__ __forceinline__ float store(V v) { return v; }
    static __device__ __forceinline__ float store_scaled(V v, int) { return v; }
    static __device__ __forceinline__ V coef(F2 c) { return c.h; }
    static __device__ __forceinline__ V zero() { return 0.0f; }
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
    static __device__ __forceinline__ V mul(V a, V c) { return a * c; }
    static __device__ __forceinline__ V norm(V a) { return a; }
    static __device__ __forceinline__ V fms2(V base, V c1, V x1, V c2, V x2) {
        return __fmaf_rn(-c2, x2, __fmaf_rn(-c1, x1, base));
    }
    static __device__ __forceinline__ V fms1(V base, V c1, V x1) { return __fmaf_rn(-c1, x1, base); }
    static __device__ __forceinline__ V mac2(V acc, V m0, V v1, V m1, V v2) {
        return __fmaf_rn(m1, v2, __fmaf_rn(m0, v1, acc));
    }
    static __device__ __forceinline__ V mac1(V acc, V m0, V v1) { return __fmaf_rn(m0, v1, acc); }
    static __device__ __forceinline__ V shfl_up(V v, unsigned d, int w) { return __shfl_up_sync(0xffffffffu, v, d, w); }
    static __device__ __forceinline__ V shfl_down(V v, unsigned d, int w) { return __shfl_down_sync(0xffffffffu, v, d, w); }
    static __device__ __forceinline__ V shfl_idx(V v, int s, int w) { return __shfl_sync(0xffffffffu, v, s, w); }
};

// ------------------------------------------------------------------------------------
// k_chunk: the chunked scan engine
// ------------------------------------------------------------------------------------
template <int M>
__device__ __forceinline__ int spos(int p) {
    return p + p / M;
}

// Staging loads keep up to kLoadUnroll loads in flight per thread before converting.
constexpr int kLoadUnroll = 8;
// Largest per-thread share of a line staged in registers by the one-pass scaled load.
constexpr int kStageRegs = 16;

template <class AR, int Q, int M, bool CIRC>
__global__ void __launch_bounds__(256, 3)
    k_chunk(const ChunkParams cp, const typename AR::IO* __restrict__ f, typename AR::IO* __restrict__ out,
            const LineSet ls, unsigned* __restrict__ status) {
    using V = typename AR::V;
    using IO = typename AR::IO;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    long* base_in = reinterpret_cast<long*>(smem_raw);
    long* base_out = base_in + cp.L;
    V* tile = reinterpret_cast<V*>(smem_raw + 16 * cp.L);  // input lines (converted), L x LS
    V* work = tile + (size_t)cp.L * cp.LS;                  // per-row RHS / solution, L x LS
    IO* wio = reinterpret_cast<IO*>(work);                  // same storage, output values

    __shared__ int lexp[256];  // per-line maximum FP64 exponent (scaled double-float path)
    const int tid = threadIdx.x, nth = blockDim.x;
    const long line0 = (long)blockIdx.x * cp.L;
    const int nl = (int)min((long)cp.L, ls.nlines - line0);
    if (AR::kScaled && tid < nl) lexp[tid] = 0;
    if (tid < cp.L) {
        const long lg = line0 + tid;
        const long a = lg % ls.na, b = lg / ls.na;
        base_in[tid] = a * ls.fa + b * ls.fb;
        base_out[tid] = a * ls.oa + b * ls.ob;
    }
    __syncthreads();

    // ---- A: stage the input lines in shared memory, converted once ----
    // Double-float: each line is split as d * 2^-(e_max - 1023), e_max its largest FP64
    // exponent, so the df range (2^-74 .. 2^127) holds relative to the line maximum
    // whatever the input scale.  When a thread's share of a line fits in kStageRegs
    // registers the values are loaded, reduced and split in one pass; longer lines are
    // staged as FP64 first and split in place.
    unsigned bad = 0;
    bool staged = false;
    if constexpr (AR::kScaled) {
        if (ls.fp == 1) {
            const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
            const int U = (cp.m + 31) >> 5;
            if (U <= kStageRegs) {
                staged = true;
                for (int l = warp; l < nl; l += nw) {
                    const IO* src = f + base_in[l];
                    V* dst = tile + l * cp.LS;
                    double v[kStageRegs];
                    int mx = 0;
#pragma unroll
                    for (int u = 0; u < kStageRegs; u++) {
                        const int p = lane + 32 * u;
                        v[u] = (u < U && p < cp.m) ? __ldg(src + p) : 0.0;
                        mx = max(mx, bexp(v[u]));
                    }
                    mx = (int)__reduce_max_sync(0xffffffffu, (unsigned)mx);
                    bad |= (unsigned)(mx == 2047);  // infinity or NaN in the line
                    if (lane == 0) lexp[l] = mx;
                    const SplitK sk = split_consts(mx - 1023);
#pragma unroll
                    for (int u = 0; u < kStageRegs; u++) {
                        const int p = lane + 32 * u;
                        if (u < U && p < cp.m) dst[spos<M>(p)] = df_split_line(v[u], sk);
                    }
                }
            }
        } else {
            const int pstep = nth / cp.L;
            const int U = (cp.m + pstep - 1) / pstep;
            if (U <= kStageRegs) {
                staged = true;
                const int l = tid % cp.L, q0 = tid / cp.L;
                double v[kStageRegs];
                int mx = 0;
                if (l < nl) {
                    const IO* src = f + base_in[l];
#pragma unroll
                    for (int u = 0; u < kStageRegs; u++) {
                        const int p = q0 + pstep * u;
                        v[u] = (u < U && p < cp.m) ? __ldg(src + (long)p * ls.fp) : 0.0;
                        mx = max(mx, bexp(v[u]));
                    }
                    atomicMax(&lexp[l], mx);
                }
                __syncthreads();
                if (l < nl) {
                    const int k = lexp[l] - 1023;
                    bad |= (unsigned)(lexp[l] == 2047);
                    V* dst = tile + l * cp.LS;
                    const SplitK sk = split_consts(k);
#pragma unroll
                    for (int u = 0; u < kStageRegs; u++) {
                        const int p = q0 + pstep * u;
                        if (u < U && p < cp.m) dst[spos<M>(p)] = df_split_line(v[u], sk);
                    }
                }
            }
        }
    }
    if (!staged) {
        if (ls.fp == 1) {
            // contiguous lines: one warp per line, kLoadUnroll loads in flight per lane
            const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
            for (int l = warp; l < nl; l += nw) {
                const IO* src = f + base_in[l];
                V* dst = tile + l * cp.LS;
                int mx = 0;
                for (int p0 = lane; p0 < cp.m; p0 += 32 * kLoadUnroll) {
                    IO v[kLoadUnroll];
#pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + 32 * u;
                        v[u] = p < cp.m ? __ldg(src + p) : (IO)0;
                    }
#pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + 32 * u;
                        if (p < cp.m) {
                            if constexpr (AR::kScaled) {
                                reinterpret_cast<double*>(dst)[spos<M>(p)] = v[u];
                                mx = max(mx, bexp(v[u]));
                            } else {
                                dst[spos<M>(p)] = AR::load(v[u], bad);
                            }
                        }
                    }
                }
                if constexpr (AR::kScaled) {
                    mx = (int)__reduce_max_sync(0xffffffffu, (unsigned)mx);
                    if (lane == 0) lexp[l] = mx;
                }
            }
        } else {
            // strided lines: consecutive threads take consecutive lines (coalesced rows)
            const int l = tid % cp.L, pstep = nth / cp.L;
            if (l < nl) {
                const IO* src = f + base_in[l];
                V* dst = tile + l * cp.LS;
                int mx = 0;
                for (int p0 = tid / cp.L; p0 < cp.m; p0 += pstep * kLoadUnroll) {
                    IO v[kLoadUnroll];
#pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + pstep * u;
                        v[u] = p < cp.m ? __ldg(src + (long)p * ls.fp) : (IO)0;
                    }
#pragma unroll
                    for (int u = 0; u < kLoadUnroll; u++) {
                        const int p = p0 + pstep * u;
                        if (p < cp.m) {
                            if constexpr (AR::kScaled) {
                                reinterpret_cast<double*>(dst)[spos<M>(p)] = v[u];
                                mx = max(mx, bexp(v[u]));
                            } else {
                                dst[spos<M>(p)] = AR::load(v[u], bad);
                            }
                        }
                    }
                }
                if constexpr (AR::kScaled) atomicMax(&lexp[l], mx);
            }
        }
        __syncthreads();
        if constexpr (AR::kScaled) {
            const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
            for (int ll = warp; ll < nl; ll += nw) {
                const int k = lexp[ll] - 1023;
                bad |= (unsigned)(lexp[ll] == 2047);  // infinity or NaN in the line
                V* row = tile + ll * cp.LS;
                const SplitK sk = split_consts(k);
                for (int p = lane; p < cp.m; p += 32) {
                    const int ps = spos<M>(p);
                    row[ps] = df_split_line(reinterpret_cast<const double*>(row)[ps], sk);
                }
            }
        }
    }
    __syncthreads();

    // ---- per-lane chunk: rows r0 .. r1-1 of line l ----
    const int t = tid % cp.Pp, l = tid / cp.Pp;
    const bool active = (l < nl) && (t < cp.P);
    const int ns = cp.ns;
    const int r0 = t * M, r1 = active ? min(ns, r0 + M) : r0;
    const V* line = tile + l * cp.LS;
    V* wl = work + l * cp.LS;
    // non-circulant coefficient tables, staged once per CTA (chunk-padded like the lines)
    V* ctab = work + (size_t)cp.L * cp.LS;  // 9 tables of LSc entries: g a1 a2 b1 b2 pf1 pf2 pb1 pb2
    const int LSc = spos<M>(ns - 1) + 1;
    if constexpr (!CIRC && Q > 0) {
        for (int i = tid; i < ns; i += nth) {
            const int ps = spos<M>(i);
#pragma unroll
            for (int k = 0; k < 5; k++) ctab[k * LSc + ps] = AR::coef(cp.rc[i * 5 + k]);
            ctab[5 * LSc + ps] = AR::coef(cp.phf[i * 2]);
            ctab[6 * LSc + ps] = AR::coef(cp.phf[i * 2 + 1]);
            ctab[7 * LSc + ps] = AR::coef(cp.phb[i * 2]);
            ctab[8 * LSc + ps] = AR::coef(cp.phb[i * 2 + 1]);
        }
        __syncthreads();
    }

    auto rhs_row = [&](int i) -> V {
        V acc = AR::zero();
        if (i < cp.nlo || i >= ns - cp.nhi) {
            const int tr = i < cp.nlo ? i : cp.nlo + (i - (ns - cp.nhi));
#pragma unroll 1
            for (int k = 0; k < cp.tw; k++) {
                const int idx = __ldg(cp.tidx + tr * cp.tw + k);
                acc = AR::add(acc, AR::mul(line[spos<M>(idx)], AR::coef(cp.tc[tr * cp.tw + k])));
            }
        } else {
            if (cp.has_center) acc = AR::mul(line[spos<M>(i + cp.center_off)], AR::coef(cp.center_c));
#pragma unroll 1
            for (int k = 0; k < cp.npair; k++) {
                const V a = line[spos<M>(i + cp.pair_op[k])];
                const V b = line[spos<M>(i + cp.pair_om[k])];
                const V d = cp.pair_sign[k] < 0 ? AR::sub(a, b) : AR::add(a, b);
                acc = AR::add(acc, AR::mul(d, AR::coef(cp.pair_c[k])));
            }
        }
        return AR::norm(acc);
    };

    if constexpr (Q == 0) {
        // explicit operator: the right-hand side is the result
        IO* wlio = reinterpret_cast<IO*>(wl);
        const int kl = AR::kScaled && l < nl ? lexp[l] - 1023 : 0;
#pragma unroll 1
        for (int i = r0; i < r1; i++) {
            V x = rhs_row(i);
            if (cp.resid) x = AR::norm(AR::sub(line[spos<M>(i)], x));
            wlio[spos<M>(i)] = AR::store_scaled(x, kl);
        }
    } else {
        const int Pp = cp.Pp;
        const V ca1 = AR::coef(cp.ca1), ca2 = AR::coef(cp.ca2);
        // ---- B+C: right-hand side and forward recurrence from a zero state ----
        V s1 = AR::zero(), s2 = AR::zero();
#pragma unroll 1
        for (int i = r0; i < r1; i++) {
            V r = rhs_row(i);
            V a1 = ca1, a2 = ca2;
            if constexpr (!CIRC) {
                const int ps = spos<M>(i);
                r = AR::mul(r, ctab[ps]);
                a1 = ctab[LSc + ps];
                a2 = ctab[2 * LSc + ps];
            }
            const V y = (Q == 2) ? AR::fms2(r, a1, s1, a2, s2) : AR::fms1(r, a1, s1);
            wl[spos<M>(i)] = y;
            s2 = s1;
            s1 = y;
        }
        // ---- D: log-step scan of the chunk transfers -> incoming state ----
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
            const V E1 = AR::shfl_idx(s1, cp.P - 1, Pp);
            const V E2 = (Q == 2) ? AR::shfl_idx(s2, cp.P - 1, Pp) : AR::zero();
            if (t < cp.P) {
                const F2* W = cp.fwrap + (size_t)t * 4;
                if constexpr (Q == 2) {
                    const V n1 = AR::mac2(i1, AR::coef(W[0]), E1, AR::coef(W[1]), E2);
                    const V n2 = AR::mac2(i2, AR::coef(W[2]), E1, AR::coef(W[3]), E2);
                    i1 = n1;
                    i2 = n2;
                } else {
                    i1 = AR::mac1(i1, AR::coef(W[0]), E1);
                }
            }
        }
        // ---- E+F: forward correction y = y~ + phi . state, backward recurrence from zero ----
        V u1 = AR::zero(), u2 = AR::zero();
#pragma unroll 1
        for (int i = r1 - 1; i >= r0; i--) {
            const int ps = spos<M>(i);
            V p1, p2, b1 = ca1, b2 = ca2;
            if constexpr (CIRC) {
                const F2* ph = cp.phf + (size_t)(i - r0) * 2;
                p1 = AR::coef(ph[0]);
                p2 = AR::coef(ph[1]);
            } else {
                p1 = ctab[5 * LSc + ps];
                p2 = ctab[6 * LSc + ps];
                b1 = ctab[3 * LSc + ps];
                b2 = ctab[4 * LSc + ps];
            }
            const V y = (Q == 2) ? AR::mac2(wl[ps], p1, i1, p2, i2) : AR::mac1(wl[ps], p1, i1);
            const V x = (Q == 2) ? AR::fms2(y, b1, u1, b2, u2) : AR::fms1(y, b1, u1);
            wl[ps] = x;
            u2 = u1;
            u1 = x;
        }
        // ---- G: reverse scan -> state entering from above ----
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
        if (t >= cp.P - 1) {
            j1 = AR::zero();
            j2 = AR::zero();
        }
        if constexpr (CIRC) {
            const V F1 = AR::shfl_idx(u1, 0, Pp);
            const V F2v = (Q == 2) ? AR::shfl_idx(u2, 0, Pp) : AR::zero();
            if (t < cp.P) {
                const F2* W = cp.bwrap + (size_t)t * 4;
                if constexpr (Q == 2) {
                    const V n1 = AR::mac2(j1, AR::coef(W[0]), F1, AR::coef(W[1]), F2v);
                    const V n2 = AR::mac2(j2, AR::coef(W[2]), F1, AR::coef(W[3]), F2v);
                    j1 = n1;
                    j2 = n2;
                } else {
                    j1 = AR::mac1(j1, AR::coef(W[0]), F1);
                }
            }
        }
        // ---- H+I: backward correction, residual form, FP64 conversion (in place) ----
        IO* wlio = reinterpret_cast<IO*>(wl);
        const int kl = AR::kScaled && l < nl ? lexp[l] - 1023 : 0;
#pragma unroll 2
        for (int i = r0; i < r1; i++) {
            const int ps = spos<M>(i);
            V p1, p2;
            if constexpr (CIRC) {
                const F2* ph = cp.phb + (size_t)(r1 - 1 - i) * 2;
                p1 = AR::coef(ph[0]);
                p2 = AR::coef(ph[1]);
            } else {
                p1 = ctab[7 * LSc + ps];
                p2 = ctab[8 * LSc + ps];
            }
            V x = (Q == 2) ? AR::mac2(wl[ps], p1, j1, p2, j2) : AR::mac1(wl[ps], p1, j1);
            if (cp.resid) x = AR::norm(AR::sub(line[ps], x));
            wlio[ps] = AR::store_scaled(x, kl);
        }
    }
    __syncthreads();

    // ---- J: coalesced stores ----
    if (ls.op == 1) {
        const int warp = tid >> 5, lane = tid & 31, nw = nth >> 5;
        for (int ll = warp; ll < nl; ll += nw) {
            IO* o = out + base_out[ll];
            const IO* src = wio + ll * cp.LS;
            for (int p = lane; p < cp.nout; p += 32) o[p] = src[spos<M>(p < ns ? p : p - ns)];
        }
    } else {
        const int ll = tid % cp.L, pstep = nth / cp.L;
        if (ll < nl) {
            IO* o = out + base_out[ll];
            const IO* src = wio + ll * cp.LS;
            for (int p = tid / cp.L; p < cp.nout; p += pstep) o[(long)p * ls.op] = src[spos<M>(p < ns ? p : p - ns)];
        }
    }
    if (bad) atomicOr(status, 1u);
}

template <class AR, int Q, int M, bool CIRC>
int launch_chunk_t(const ChunkParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                   cudaStream_t s) {
    using IO = typename AR::IO;
    const int threads = c.L * c.Pp;
    const long blocks = (ls.nlines + c.L - 1) / c.L;
    const int LSc = c.ns - 1 + (c.ns - 1) / M + 1;
    const size_t smem = 16 * (size_t)c.L + 2 * sizeof(typename AR::V) * (size_t)c.L * c.LS +
                        ((!CIRC && Q > 0) ? 9 * sizeof(typename AR::V) * (size_t)LSc : 0);
    auto kern = k_chunk<AR, Q, M, CIRC>;
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
    }
    kern<<<(unsigned)blocks, threads, smem, s>>>(c, (const IO*)f, (IO*)out, ls, status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

template <class AR, int M>
int launch_chunk_m(const ChunkPlanHost& h, const ChunkParams& c, const void* f, void* out, const LineSet& ls,
                   unsigned* status, cudaStream_t s) {
    if (h.Q == 0) return launch_chunk_t<AR, 0, M, false>(c, f, out, ls, status, s);
    if (h.Q == 1) return h.circ ? launch_chunk_t<AR, 1, M, true>(c, f, out, ls, status, s)
                                : launch_chunk_t<AR, 1, M, false>(c, f, out, ls, status, s);
    return h.circ ? launch_chunk_t<AR, 2, M, true>(c, f, out, ls, status, s)
                  : launch_chunk_t<AR, 2, M, false>(c, f, out, ls, status, s);
}


// explicit instantiations live in kernels_df16.cu, kernels_df32.cu, kernels_f32.cu
extern template int launch_chunk_m<ArDF, 16>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                             const LineSet&, unsigned*, cudaStream_t);
extern template int launch_chunk_m<ArDF, 32>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                             const LineSet&, unsigned*, cudaStream_t);
extern template int launch_chunk_m<ArF32, 16>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                              const LineSet&, unsigned*, cudaStream_t);
extern template int launch_chunk_m<ArF32, 32>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                              const LineSet&, unsigned*, cudaStream_t);

}  // namespace pade
