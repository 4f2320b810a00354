// Batched FFTs in double-float arithmetic (FP64 in and out, pairs of floats inside).
//
// The FP64 transform of fft.cu keeps GB300's FP64 pipe ~85 % busy at a few per cent of
// the HBM bandwidth (4 n log2 n FP64 operations per line, FP64 issuing at 1/56 of the
// FP32 rate).  This kernel does the same transforms on the FP32 pipes: every complex
// value is (re_hi + re_lo, im_hi + im_lo), butterflies use the error-free TwoSum /
// TwoProduct of dfmath.cuh with a renormalisation per stage, and twiddles are float pairs
// of the correctly rounded values (~48 significant bits; transform error ~log2(n) 2^-47).
//
// Each line is scaled by a power of two before the split so that its largest element is
// in [1, 2): the double-float range (|x| >= 2^-74 for full precision) then holds relative
// to the line maximum and the scaling is exact, done on the exponent bits with integer
// instructions (no FP64 multiply).  Elements below 2^-74 of their line's maximum are
// treated as zero.  Loads are in natural order and the forward transform decimates in
// frequency (bit-reversed result); the fused kinds multiply in that order and transform
// back by decimation in time, so no reordering pass is needed.
//
// Kernels: k_fft_df (any length 2..8192, radix-4 passes through shared memory, the fused z
// kinds), k_fft_df_real (r2c / c2r along x through a half-length complex transform), and
// for 256-point lines the register four-step 16 x 16 (one shared-memory exchange):
// k_fft_df256 (strided complex lines, the y transforms), k_fft_df256_fk (the fused z kinds),
// k_fft_df_c2r_pair256 (two c2r transforms of contiguous x lines as one complex transform).
// PADE_FFT_FOURSTEP=0 (a tuning override) keeps the radix-4 kernels everywhere.
//
// Same modes, kinds and conventions as k_fft (fft.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "dfmath.cuh"
#include "fft.h"
#include "operators.h"

namespace pade {

namespace {

// A complex double-float value, packed for the FP32x2 instructions: the real and imaginary
// parts are the two components of one df2 (h = (re_hi, im_hi), l = (re_lo, im_lo)), so a
// complex sum, difference or real scaling is one packed double-float operation, and a
// twiddle product two packed products and one packed sum.  Every component is rounded as
// the scalar double-float code rounds it (the same operations in the same order), so the
// results are those of the unpacked form.
using cdf = df2;
__device__ __forceinline__ dfv cre(cdf a) { return d2_x(a); }
__device__ __forceinline__ dfv cim(cdf a) { return d2_y(a); }
__device__ __forceinline__ cdf mkc(dfv re, dfv im) { return d2_pack(re, im); }
__device__ __forceinline__ cdf czero() { return d2_zero(); }

// shared memory holds a value as {re_hi, im_hi, re_lo, im_lo}
__device__ __forceinline__ cdf ldc(const float4* s, int idx) { return d2_of(s[idx]); }
__device__ __forceinline__ void stc(float4* s, int idx, cdf c) { s[idx] = d2_f4(c); }

__device__ __forceinline__ cdf cadd(cdf a, cdf b) { return d2_norm(d2_add(a, b)); }
__device__ __forceinline__ cdf csub(cdf a, cdf b) { return d2_norm(d2_sub(a, b)); }

// (im, re): the swap behind the cross terms of a complex product
__device__ __forceinline__ cdf cswap(cdf a) {
    return cdf{make_float2(a.h.y, a.h.x), make_float2(a.l.y, a.l.x)};
}

// a * w (w a twiddle (c_hi, c_lo, s_hi, s_lo)); conj uses c - i s.  With wi the imaginary
// part used: (re, im) * (wr, wr) + (im, re) * (-wi, wi) = (re wr - im wi, im wr + re wi).
__device__ __forceinline__ cdf cmulw(cdf a, float4 w, bool conj) {
    const float sh = conj ? -w.z : w.z, sl = conj ? -w.w : w.w;
    const cdf p1 = d2_mul(a, cdf{make_float2(w.x, w.x), make_float2(w.y, w.y)});
    const cdf p2 = d2_mul(cswap(a), cdf{make_float2(-sh, sh), make_float2(-sl, sl)});
    return d2_norm(d2_add(p1, p2));
}

// -i a (forward), +i a (backward): exact
__device__ __forceinline__ cdf mul_mi(cdf a, bool conj) {
    return conj ? cdf{make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)}
                : cdf{make_float2(a.h.y, -a.h.x), make_float2(a.l.y, -a.l.x)};
}

__device__ __forceinline__ cdf cscale(cdf a, dfv m) { return d2_norm(d2_mul(a, d2_bcast(m))); }

// W^t for t < 3N/4 from the table of t < N/2 (= nh): W^(t + N/2) = -W^t
__device__ __forceinline__ float4 twiddle_ext(const float4* __restrict__ twg, int t, int nh) {
    if (t < nh) return __ldg(&twg[t]);
    const float4 w = __ldg(&twg[t - nh]);
    return make_float4(-w.x, -w.y, -w.z, -w.w);
}

// global elements each thread reads before storing them to shared memory
constexpr int kLoadBatch = 4;

// raises the line maximum emax[l] to m; `warp_line` (uniform over the block) says that the
// 32 lanes of each warp hold points of one line, so one lane updates it for the warp
__device__ __forceinline__ void emax_update(int* emax, int l, int m, bool warp_line) {
    if (warp_line) {
        m = __reduce_max_sync(0xffffffffu, m);
        if ((threadIdx.x & 31) == 0) atomicMax(&emax[l], m);
    } else {
        atomicMax(&emax[l], m);
    }
}

__device__ __forceinline__ int brev(int p, int logn) { return (int)(__brev((unsigned)p) >> (32 - logn)); }

// Bank swizzle of the points of a shared-memory line: q -> q ^ (bits 3..5 of q) ^ (for
// lines of >= 256 points, the two top bits of q).  It is linear over XOR, its own inverse,
// and permutes each aligned group of 8 points, so the butterfly passes (four points h apart),
// bit-reversed reads and contiguous reads each meet few bank conflicts.
struct Swz {
    int sh, m2;
};
__device__ __forceinline__ Swz make_swz(int logn) { return logn >= 8 ? Swz{logn - 2, 3} : Swz{3, 0}; }
__device__ __forceinline__ int swz(int q, Swz z) { return q ^ ((q >> 3) & 7) ^ ((q >> z.sh) & z.m2); }

__device__ __forceinline__ double ksq(double a, double b, double c) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// the multiplier of the fused kinds at wavenumbers (a, b, c); zero_mode: the (0, 0, 0) point
template <int KIND>
__device__ __forceinline__ double fk_mult(double a, double b, double c, bool zero_mode) {
    const double kr = ksq(a, b, c);
    if (KIND == FK_PROJECT) return kr <= 1e-14 ? 0.0 : -(1.0 / kr);
    return zero_mode ? 0.0 : -1.0 / __dadd_rn(kr, 1e-20);
}

// out of line for the unrolled four-step kernel (its tables make this path rare)
template <int KIND>
__device__ __noinline__ double fk_mult_call(double a, double b, double c, bool zero_mode) {
    return fk_mult<KIND>(a, b, c, zero_mode);
}

template <int KIND>
__global__ void k_mult_table(const double* __restrict__ ka, const double* __restrict__ kb,
                             const double* __restrict__ kc, int nxh, int logn, long nlines, double* __restrict__ out) {
    const long total = nlines << logn;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const long lg = e >> logn;
        const int q = (int)(e & ((1 << logn) - 1)), f = brev(q, logn);
        out[e] = fk_mult<KIND>(ka[lg % nxh], kb[lg / nxh], kc[f], lg == 0 && f == 0);
    }
}

// decimation in frequency: natural order -> bit-reversed.  tw holds exp(-2 pi i t / (n 2^tws)),
// so a table made for a longer transform serves with stride 2^tws; it extends to 3/4 of that
// transform's length (W^(t + N/2) = -W^t) for the radix-4 twiddle W^3k.  Line l starts at
// l * lsd (lsd >= 2^logn, padded to spread lines over the banks).  Stages s and s - 1 run as
// one radix-4 pass (four points h = 2^(s-1) apart per thread, twiddles W^k, W^2k, W^3k of the
// block of 4h and the trivial W^h = -i), with a final radix-2 stage when logn is odd.
__device__ __forceinline__ void dif_df(float4* x, int nl, int logn, int lsd, const float4* tw,
                                       bool conj, int tws = 0) {
    const Swz z = make_swz(logn);
    int s = logn - 1;
    for (; s >= 1; s -= 2) {
        const int work4 = nl << (logn - 2);
        const int h = 1 << (s - 1);  // quarter of a block of 2^(s+1)
        const int t1 = logn - 1 - s + tws, t2 = logn - s + tws;
        const int c1 = swz(h, z), c2 = swz(2 * h, z), c3 = swz(3 * h, z);
        for (int e = threadIdx.x; e < work4; e += blockDim.x) {
            const int l = e >> (logn - 2), j = e & ((1 << (logn - 2)) - 1);
            const int k = j & (h - 1);
            // points q0 + r h = q0 ^ (r h) (bits s-1 and s of q0 are clear), swizzled
            const int lb = l * lsd, q0 = swz(((j >> (s - 1)) << (s + 1)) + k, z);
            const int i0 = lb + q0, i1 = lb + (q0 ^ c1), i2 = lb + (q0 ^ c2), i3 = lb + (q0 ^ c3);
            const cdf x0 = ldc(x, i0), x1 = ldc(x, i1), x2 = ldc(x, i2), x3 = ldc(x, i3);
            const cdf s02 = cadd(x0, x2), d02 = csub(x0, x2), s13 = cadd(x1, x3), d13 = csub(x1, x3);
            const cdf c = mul_mi(d13, conj);  // W^h d13, W^h = -i (+i backward)
            cdf y1 = csub(s02, s13), y2 = cadd(d02, c), y3 = csub(d02, c);
            if (s > 1) {  // at s = 1 every k is 0
                y1 = cmulw(y1, tw[k << t2], conj);
                y2 = cmulw(y2, tw[k << t1], conj);
                y3 = cmulw(y3, tw[(3 * k) << t1], conj);
            }
            stc(x, i0, cadd(s02, s13));
            stc(x, i1, y1);
            stc(x, i2, y2);
            stc(x, i3, y3);
        }
        __syncthreads();
    }
    if (s == 0) {  // odd logn: the last stage alone
        const int work = nl << (logn - 1);
        for (int e = threadIdx.x; e < work; e += blockDim.x) {
            const int lb = (e >> (logn - 1)) * lsd, q0 = swz((e & ((1 << (logn - 1)) - 1)) << 1, z);
            const int i0 = lb + q0, i1 = lb + (q0 ^ 1);  // swz(1) = 1
            const cdf a = ldc(x, i0), b = ldc(x, i1);
            stc(x, i0, cadd(a, b));
            stc(x, i1, csub(a, b));
        }
        __syncthreads();
    }
}

// decimation in time: bit-reversed -> natural order; stages s and s + 1 as one radix-4 pass
__device__ __forceinline__ void dit_df(float4* x, int nl, int logn, int lsd, const float4* tw,
                                       bool conj, int tws = 0) {
    const Swz z = make_swz(logn);
    int s = 0;
    for (; s + 1 < logn; s += 2) {
        const int work4 = nl << (logn - 2);
        const int h = 1 << s;  // quarter of a block of 2^(s+2)
        const int t1 = logn - 1 - s + tws, t2 = logn - 2 - s + tws;
        const int c1 = swz(h, z), c2 = swz(2 * h, z), c3 = swz(3 * h, z);
        for (int e = threadIdx.x; e < work4; e += blockDim.x) {
            const int l = e >> (logn - 2), j = e & ((1 << (logn - 2)) - 1);
            const int k = j & (h - 1);
            const int lb = l * lsd, q0 = swz(((j >> s) << (s + 2)) + k, z);
            const int i0 = lb + q0, i1 = lb + (q0 ^ c1), i2 = lb + (q0 ^ c2), i3 = lb + (q0 ^ c3);
            const cdf x0 = ldc(x, i0);
            cdf x1 = ldc(x, i1), x2 = ldc(x, i2), x3 = ldc(x, i3);
            if (s > 0) {  // at s = 0 every k is 0
                x1 = cmulw(x1, tw[k << t1], conj);
                x2 = cmulw(x2, tw[k << t2], conj);
                x3 = cmulw(x3, tw[(3 * k) << t2], conj);
            }
            const cdf s01 = cadd(x0, x1), d01 = csub(x0, x1), s23 = cadd(x2, x3);
            const cdf c = mul_mi(csub(x2, x3), conj);  // W^h (x2 - x3), W^h = -i (+i backward)
            stc(x, i0, cadd(s01, s23));
            stc(x, i2, csub(s01, s23));
            stc(x, i1, cadd(d01, c));
            stc(x, i3, csub(d01, c));
        }
        __syncthreads();
    }
    if (s == logn - 1) {  // odd logn: the last stage alone
        const int half = 1 << s;
        const int work = nl << (logn - 1);
        for (int e = threadIdx.x; e < work; e += blockDim.x) {
            const int l = e >> (logn - 1), k = e & (half - 1);
            const int q0 = swz(k, z), i0 = l * lsd + q0, i1 = l * lsd + (q0 ^ swz(half, z));
            const cdf a = ldc(x, i0);
            cdf b = ldc(x, i1);
            if (s > 0) b = cmulw(b, tw[k << tws], conj);
            stc(x, i0, cadd(a, b));
            stc(x, i1, csub(a, b));
        }
        __syncthreads();
    }
}

// c * 2^k as FP64: d(h) + d(l) with the shift on the exponent bits when |k| <= 800 (exact,
// the same value as shifting the sum), else the checked shift of the sum
__device__ __noinline__ double2 cstore_checked(cdf c, int k) {  // out of line: rare, keeps kernels small
    return make_double2(shift_up(df_to_double(cre(c)), k), shift_up(df_to_double(cim(c)), k));
}
__device__ __forceinline__ double2 cstore(cdf c, int k) {
    if (k >= -800 && k <= 800) {  // both parts scaled on their exponent bits, no range checks
        const unsigned kadd = (unsigned)(896 + k) << 20;
        return make_double2(df_to_double_kadd(cre(c), kadd), df_to_double_kadd(cim(c), kadd));
    }
    return cstore_checked(c, k);
}

template <int IN, int OUT, int KIND>
__global__ void __launch_bounds__(256) k_fft_df(const void* in, void* out, const FftLines ls,
                                                const float4* __restrict__ twg, int logn, int lb, int sign,
                                                int scale_exp, float2 scale_df, int use_scale_df, int oddball,
                                                const FftExtra ex) {
    extern __shared__ __align__(16) float4 smf[];
    double2* smd = reinterpret_cast<double2*>(smf);
    __shared__ int emax[64];
    // per line: input / output offsets, its index a in the first extent, and for the fused
    // kinds its (x, y) wavenumber indices (one division per line, none per element)
    __shared__ long lbin[64], lbout[64];
    __shared__ int la[64], lxi[64], lyj[64];
    __shared__ bool keep_ij[64];  // FK_DEALIAS: the x-y cut-offs of each line
    const int n = 1 << logn, half = n >> 1;
    const int lsd = n + 1;  // shared-memory line stride: lines at one point apart start on distinct banks
    const Swz z = make_swz(logn);  // point p of line l sits at l * lsd + swz(p)
    float4* tw = smf + (size_t)lb * lsd;  // the twiddles W^t, t < 3n/4, staged behind the lines
    for (int t = threadIdx.x; t < half + (half >> 1); t += blockDim.x) tw[t] = twiddle_ext(twg, t, half);
    const long l0 = (long)blockIdx.x * lb;
    const int nl = (int)min((long)lb, ls.nlines - l0);
    const int total = nl << logn;
    const bool pin = ls.fp == 1, pout = ls.op == 1;
    for (int l = threadIdx.x; l < nl; l += blockDim.x) {
        emax[l] = 0;
        const long lg = l0 + l, a = lg % ls.na, b = lg / ls.na;
        lbin[l] = a * ls.fa + b * ls.fb;
        lbout[l] = a * ls.oa + b * ls.ob;
        la[l] = (int)a;
        if (KIND != FK_PLAIN) {
            lxi[l] = (int)(lg % ex.nxh);
            lyj[l] = (int)(lg / ex.nxh);
        }
        if (KIND == FK_DEALIAS) keep_ij[l] = fabs(ex.ka[lxi[l]]) < ex.cut_a && fabs(ex.kb[lyj[l]]) < ex.cut_b;
    }
    __syncthreads();
    // element e = (l, p): e = l n + p on contiguous lines, e = p nl + l on strided lines
    // (consecutive threads on consecutive lines); strided positions advance by (sl, sp)
    const int sl = blockDim.x % nl, sp = blockDim.x / nl;

    // one element (l, p) of the input, with the pre-transform multiplier of its kind applied
    auto fetch = [&](int l, int p) -> double2 {
        const long base = lbin[l];
        double2 v;
        if (IN == IN_COMPLEX) {
            v = reinterpret_cast<const double2*>(in)[base + p * ls.fp];
        } else if (IN == IN_REAL) {
            v = make_double2(reinterpret_cast<const double*>(in)[base + p * ls.fp], 0.0);
        } else {
            const double2* src = reinterpret_cast<const double2*>(in);
            if (p <= half) {
                v = src[base + p * ls.fp];
            } else {
                const double2 c = src[base + (long)(n - p) * ls.fp];
                v = make_double2(c.x, -c.y);
            }
            if (p == 0 || p == half) v.y = 0.0;
            if (oddball && p == half) v.x = 0.0;
        }
        if (KIND == FK_PLAIN && ex.mul == MUL_MASK_AP) {
            const int a = la[l];
            if (!(fabs(ex.ka[a]) < ex.cut_a && fabs(ex.kb[p]) < ex.cut_b)) v = make_double2(0.0, 0.0);
        } else if (KIND == FK_PLAIN && ex.mul != MUL_NONE) {
            const double k = ex.km[ex.mul == MUL_IK_A ? la[l] : p];
            v = make_double2(-k * v.y, k * v.x);
        }
        if (KIND == FK_PROJECT) {
            const long idx = l0 + l + p * ex.plane;
            const double k1 = ex.k1[lxi[l]], k2 = ex.k2[lyj[l]];
            const double2 uu = ex.u[idx], vv = ex.v[idx];
            const double tx = __dadd_rn(__dmul_rn(k1, uu.x), __dmul_rn(k2, vv.x));
            const double ty = __dadd_rn(__dmul_rn(k1, uu.y), __dmul_rn(k2, vv.y));
            v = make_double2(v.x - ty, v.y + tx);
        }
        return v;
    };

    // ---- load (FP64, natural order) and the per-line maximum exponent; kLoadBatch elements
    // per thread are read before any is stored, so their global loads overlap
    int ls_l = threadIdx.x % nl, ls_p = threadIdx.x / nl;
    // strided lines with nl dividing the block: every element of a thread is on its line
    // threadIdx.x % nl, so the thread keeps the maximum and updates emax once
    const bool own_line = !pin && sl == 0;
    int my_max = 0;
    for (int e0 = threadIdx.x; e0 < total; e0 += kLoadBatch * blockDim.x) {
        double2 vb[kLoadBatch];
        int lidx[kLoadBatch], pidx[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; u++) {
            const int e = e0 + u * blockDim.x;
            lidx[u] = pin ? (e >> logn) : ls_l;
            pidx[u] = pin ? (e & (n - 1)) : ls_p;
            if (!pin) {
                ls_l += sl;
                ls_p += sp;
                if (ls_l >= nl) {
                    ls_l -= nl;
                    ls_p++;
                }
            }
            if (e < total) vb[u] = fetch(lidx[u], pidx[u]);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; u++) {
            if (e0 + u * blockDim.x >= total) continue;
            const double2 v = vb[u];
            smd[lidx[u] * lsd + swz(pidx[u], z)] = v;
            const int m = max(bexp(v.x), bexp(v.y));
            if (own_line) {
                my_max = max(my_max, m);
            } else {
                emax_update(emax, lidx[u], m, pin && logn >= 5);
            }
        }
    }
    if (own_line && threadIdx.x < total) atomicMax(&emax[threadIdx.x % nl], my_max);
    __syncthreads();
    // ---- split in place, each line scaled by 2^-(emax - 1023)
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int k = emax[e >> logn] - 1023;
        const int i = e + (e >> logn);
        const double2 v = smd[i];
        stc(smf, i, mkc(df_from_double_shift(v.x, k), df_from_double_shift(v.y, k)));
    }
    __syncthreads();

    if (KIND == FK_PLAIN) {
        dif_df(smf, nl, logn, lsd, tw, sign > 0);
    } else {
        dif_df(smf, nl, logn, lsd, tw, false);
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int l = e >> logn, qs = e & (n - 1);
            const int f = brev(swz(qs, z), logn);  // frequency held at (swizzled) position qs
            const int se = l * lsd + qs;
            const long lg = l0 + l;
            const int i = lxi[l], j = lyj[l];
            if (KIND == FK_DEALIAS) {
                const bool keep = keep_ij[l] && fabs(ex.kc[f]) < ex.cut_c;
                if (!keep) stc(smf, se, czero());
            } else {
                double m;
                if (ex.mtab) {
                    m = ex.mtab[lg * n + swz(qs, z)];
                } else {
                    m = fk_mult<KIND>(ex.ka[i], ex.kb[j], ex.kc[f], lg == 0 && f == 0);
                }
                unsigned bad = 0;
                stc(smf, se, cscale(ldc(smf, se), df_from_double(m, bad)));
            }
        }
        __syncthreads();
        dit_df(smf, nl, logn, lsd, tw, true);
    }

    // ---- store (FP64)
    const int nout = OUT == OUT_HALF ? half + 1 : n;
    const dfv sdf{scale_df.x, scale_df.y};
    int ss_l = threadIdx.x % nl, ss_p = threadIdx.x / nl;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int l = pout ? (e >> logn) : ss_l;
        const int p = pout ? (e & (n - 1)) : ss_p;
        if (!pout) {
            ss_l += sl;
            ss_p += sp;
            if (ss_l >= nl) {
                ss_l -= nl;
                ss_p++;
            }
        }
        if (p >= nout) continue;
        const long lg = l0 + l;
        const long o = lbout[l] + p * ls.op;
        cdf c = ldc(smf, l * lsd + swz(KIND == FK_PLAIN ? brev(p, logn) : p, z));
        if (use_scale_df) c = cscale(c, sdf);
        const int k = emax[l] - 1023 + scale_exp;
        const double2 v = cstore(c, k);
        if (OUT == OUT_REAL) {
            reinterpret_cast<double*>(out)[o] = v.x;
        } else {
            reinterpret_cast<double2*>(out)[o] = v;
        }
        if (KIND == FK_DEALIAS && ex.edge_copy && p == 0) reinterpret_cast<double2*>(out)[o + (long)n * ls.op] = v;
        if (KIND == FK_PROJECT) {
            const long idx = lg + p * ex.plane;
            const double k1 = ex.k1[lxi[l]], k2 = ex.k2[lyj[l]];
            double2 uu = ex.u[idx], vv = ex.v[idx];
            uu = make_double2(uu.x + k1 * v.y, uu.y - k1 * v.x);
            vv = make_double2(vv.x + k2 * v.y, vv.y - k2 * v.x);
            ex.u[idx] = uu;
            ex.v[idx] = vv;
        }
    }
}

__device__ __forceinline__ cdf cconj(cdf a) { return cdf{make_float2(a.h.x, -a.h.y), make_float2(a.l.x, -a.l.y)}; }
__device__ __forceinline__ cdf chalf(cdf a) {
    const float2 half = make_float2(0.5f, 0.5f);
    return cdf{__fmul2_rn(a.h, half), __fmul2_rn(a.l, half)};
}

// Real transforms along x lines (fp == 1) of N = 2^logN points through one complex transform
// of M = N/2 points (the classical even/odd packing):
//   r2c: z[j] = x[2j] + i x[2j+1], Z = FFT_M(z), and for k = 0..M
//        X[k] = ((Z[k] + conj Z[M-k]) - i W^k (Z[k] - conj Z[M-k])) / 2,   W = exp(-2 pi i / N)
//   c2r: Z'[k] = (X[k] + conj X[M-k]) + i conj(W^k) (X[k] - conj X[M-k]), k = 0..M-1,
//        w = unnormalised backward FFT_M(Z'), x[2j] = Re w[j], x[2j+1] = Im w[j]
// (the imaginary parts of X[0] and X[M] are ignored, as FFTW's c2r does; oddball zeroes X[M]).
// km (c2r only, may be null): X[k] is first multiplied by i km[k], k = 0..M (the x derivative
// of the spectrum, ahead of the dropped imaginary parts as when the product is stored).
template <bool R2C>
__global__ void __launch_bounds__(256) k_fft_df_real(const void* in, void* out, const FftLines ls,
                                                     const float4* __restrict__ twg, int logN, int lb, int scale_exp,
                                                     float2 scale_df, int use_scale_df, int oddball,
                                                     const double* __restrict__ km) {
    extern __shared__ __align__(16) float4 smf[];
    double2* smd = reinterpret_cast<double2*>(smf);
    __shared__ int emax[64];
    __shared__ float4 xlast[64];  // c2r: X[M] of each line (split)
    __shared__ double2 xlast_raw[64];
    __shared__ long lbin[64], lbout[64];  // per-line input / output offsets
    const int logM = logN - 1, M = 1 << logM;
    const Swz z = make_swz(logM);  // point j of line l sits at (l << logM) + swz(j)
    float4* tw = smf + ((size_t)lb << logM);  // the twiddles W_N^t, t < 3N/4, staged behind the lines
    for (int t = threadIdx.x; t < M + (M >> 1); t += blockDim.x) tw[t] = twiddle_ext(twg, t, M);
    const long l0 = (long)blockIdx.x * lb;
    const int nl = (int)min((long)lb, ls.nlines - l0);
    const int total = nl << logM;
    for (int l = threadIdx.x; l < nl; l += blockDim.x) {
        emax[l] = 0;
        const long lg = l0 + l, a = lg % ls.na, b = lg / ls.na;
        lbin[l] = a * ls.fa + b * ls.fb;
        lbout[l] = a * ls.oa + b * ls.ob;
    }
    __syncthreads();
    for (int e0 = threadIdx.x; e0 < total; e0 += kLoadBatch * blockDim.x) {
        double2 vb[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; u++) {
            const int e = e0 + u * blockDim.x;
            if (e >= total) continue;
            const int l = e >> logM, j = e & (M - 1);
            const long base = lbin[l];
            if (R2C) {
                vb[u] = *reinterpret_cast<const double2*>(reinterpret_cast<const double*>(in) + base + 2 * j);
            } else {
                double2 v = reinterpret_cast<const double2*>(in)[base + j];
                if (km) v = make_double2(-km[j] * v.y, km[j] * v.x);  // i k(j) X[j]
                if (j == 0) v.y = 0.0;
                vb[u] = v;
            }
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; u++) {
            const int e = e0 + u * blockDim.x;
            if (e >= total) continue;
            smd[(e & ~(M - 1)) + swz(e & (M - 1), z)] = vb[u];
            emax_update(emax, e >> logM, max(bexp(vb[u].x), bexp(vb[u].y)), logM >= 5);
        }
    }
    if (!R2C) {
        for (int l = threadIdx.x; l < nl; l += blockDim.x) {
            double2 v = reinterpret_cast<const double2*>(in)[lbin[l] + M];
            if (km) v = make_double2(-km[M] * v.y, km[M] * v.x);
            v.y = 0.0;
            if (oddball) v.x = 0.0;
            xlast_raw[l] = v;
            atomicMax(&emax[l], bexp(v.x));
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int k = emax[e >> logM] - 1023;
        const double2 v = smd[e];
        stc(smf, e, mkc(df_from_double_shift(v.x, k), df_from_double_shift(v.y, k)));
    }
    if (!R2C) {
        for (int l = threadIdx.x; l < nl; l += blockDim.x) {
            const int k = emax[l] - 1023;
            const double2 v = xlast_raw[l];
            stc(xlast, l, mkc(df_from_double_shift(v.x, k), df_from_double_shift(v.y, k)));
        }
    }
    __syncthreads();
    const dfv sdf{scale_df.x, scale_df.y};
    if (R2C) {
        dif_df(smf, nl, logM, M, tw, false, 1);  // Z in bit-reversed order
        for (int e = threadIdx.x; e < total + nl; e += blockDim.x) {
            int l, k;
            if (e < total) {
                l = e >> logM;
                k = e & (M - 1);
            } else {
                l = e - total;
                k = M;
            }
            const int ka = k & (M - 1), kb = (M - k) & (M - 1);
            const cdf za = ldc(smf, (l << logM) + swz(brev(ka, logM), z));
            const cdf zb = cconj(ldc(smf, (l << logM) + swz(brev(kb, logM), z)));
            const cdf sm = cadd(za, zb), df = csub(za, zb);
            cdf t;
            if (k < M) {
                t = cmulw(df, tw[k], false);
            } else {
                t = d2_neg(df);  // W^M = -1
            }
            // X = (sm - i t) / 2, -i t = (t.i, -t.r)
            cdf X = chalf(cadd(sm, mul_mi(t, false)));
            if (use_scale_df) X = cscale(X, sdf);
            reinterpret_cast<double2*>(out)[lbout[l] + k] = cstore(X, emax[l] - 1023 + scale_exp);
        }
    } else {
        // pairs (k, M-k) for k = 0 .. M/2 - 1, in place; X[M] of k = 0 comes from xlast
        const int half = M >> 1;
        for (int e = threadIdx.x; e < (nl << (logM - 1)); e += blockDim.x) {
            const int l = e >> (logM - 1), k = e & (half - 1);
            const int k2 = M - k;
            const int ik = (l << logM) + swz(k, z), ik2 = (l << logM) + swz(k2 & (M - 1), z);
            const cdf xk = ldc(smf, ik);
            const cdf xk2 = k == 0 ? ldc(xlast, l) : ldc(smf, ik2);
            // Z'[k] = (xk + conj xk2) + i conj(W^k) (xk - conj xk2)
            {
                const cdf c2 = cconj(xk2);
                const cdf sm = cadd(xk, c2);
                cdf d = csub(xk, c2);
                if (k > 0) d = cmulw(d, tw[k], true);
                stc(smf, ik, cadd(sm, mul_mi(d, true)));  // sm + i d
            }
            if (k > 0) {  // Z'[k2], k2 = M - k in (M/2, M)
                const cdf c1 = cconj(xk);
                const cdf sm = cadd(xk2, c1);
                const cdf d = cmulw(csub(xk2, c1), tw[k2], true);
                stc(smf, ik2, cadd(sm, mul_mi(d, true)));
            }
        }
        // k = M/2 pairs with itself: conj(W^(M/2)) = i
        for (int l = threadIdx.x; l < nl; l += blockDim.x) {
            const int ih = (l << logM) + swz(half, z);
            const cdf x = ldc(smf, ih);
            const cdf c = cconj(x);
            const cdf sm = cadd(x, c);
            cdf d = csub(x, c);
            d = mul_mi(d, true);  // i * d
            stc(smf, ih, cadd(sm, mul_mi(d, true)));
        }
        __syncthreads();
        dif_df(smf, nl, logM, M, tw, true, 1);  // backward, bit-reversed
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int l = e >> logM, j = e & (M - 1);
            cdf w = ldc(smf, (l << logM) + swz(brev(j, logM), z));
            if (use_scale_df) w = cscale(w, sdf);
            *reinterpret_cast<double2*>(reinterpret_cast<double*>(out) + lbout[l] + 2 * j) =
                cstore(w, emax[l] - 1023 + scale_exp);
        }
    }
}

// ---- 256-point complex transforms of strided lines in registers (the y transforms) ----
// Four-step form n = 16 x 16: thread (l, j) of a CTA of 16 lines loads x[16 p1 + j],
// p1 = 0..15, runs a 16-point DFT over p1 in registers, multiplies by W256^(j k1), and
// exchanges through shared memory once; thread (l, k1) then runs the 16-point DFT over j and
// stores X[k1 + 16 k2].  Each 16-point DFT is radix-4 x radix-4 (W16^(q r) between), so per
// point one shared-memory store and load replace the four passes of k_fft_df.

// y0..y3 = the 4-point DFT of x0..x3 (W4 = -i forward, +i backward)
__device__ __forceinline__ void radix4(const cdf& x0, const cdf& x1, const cdf& x2, const cdf& x3, bool inv, cdf& y0,
                                       cdf& y1, cdf& y2, cdf& y3) {
    const cdf s02 = cadd(x0, x2), d02 = csub(x0, x2), s13 = cadd(x1, x3);
    const cdf c = mul_mi(csub(x1, x3), inv);
    y0 = cadd(s02, s13);
    y1 = cadd(d02, c);
    y2 = csub(s02, s13);
    y3 = csub(d02, c);
}

// in place: a[k] = sum_m a[m] W16^(m k); tw is the 256-point table (W16^e = tw[16 e])
__device__ __forceinline__ void dft16(cdf (&a)[16], bool inv, const float4* tw) {
    cdf b[16];  // b[4 q + r]: the 4-point DFT over m of a[q + 4 m], times W16^(q r)
#pragma unroll
    for (int q = 0; q < 4; q++) radix4(a[q], a[q + 4], a[q + 8], a[q + 12], inv, b[4 * q], b[4 * q + 1], b[4 * q + 2], b[4 * q + 3]);
#pragma unroll
    for (int q = 1; q < 4; q++)
#pragma unroll
        for (int r = 1; r < 4; r++) {
            const int e = q * r;
            b[4 * q + r] = e == 4 ? mul_mi(b[4 * q + r], inv) : cmulw(b[4 * q + r], tw[16 * e], inv);
        }
#pragma unroll
    for (int r = 0; r < 4; r++) radix4(b[r], b[4 + r], b[8 + r], b[12 + r], inv, a[r], a[r + 4], a[r + 8], a[r + 12]);
}

template <int MUL>  // the load-time multiplier (FftMul), one instantiation each: smaller code
__global__ void __launch_bounds__(256, 2) k_fft_df256(const void* in, void* out, const FftLines ls,
                                                       const float4* __restrict__ twg, int sign, int scale_exp,
                                                       float2 scale_df, int use_scale_df, const FftExtra ex) {
    constexpr int LSD = 257;  // shared line stride (float4): consecutive lines on distinct banks
    extern __shared__ __align__(16) float4 smf[];
    float4* tw = smf + 16 * LSD;  // W256^t, t < 256
    __shared__ int emax[16];
    __shared__ long lbin[16], lbout[16];
    __shared__ int la[16];
    __shared__ bool keep_a[16], keep_p[256];  // MUL_MASK_AP: the two cut-offs, once per line / position
    __shared__ dfv kdf[256];  // MUL_IK_P: km per position, MUL_IK_A: per line, as double-float
    const bool inv = sign > 0;
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
        tw[t] = twiddle_ext(twg, t, 128);
        if (MUL == MUL_MASK_AP) keep_p[t] = fabs(ex.kb[t]) < ex.cut_b;
        if (MUL == MUL_IK_P) {
            unsigned bad = 0;
            kdf[t] = df_from_double(ex.km[t], bad);
        }
    }
    const long l0 = (long)blockIdx.x * 16;
    const int nl = (int)min(16L, ls.nlines - l0);
    if (threadIdx.x < nl) {
        const long lg = l0 + threadIdx.x, a = lg % ls.na, b = lg / ls.na;
        emax[threadIdx.x] = 0;
        lbin[threadIdx.x] = a * ls.fa + b * ls.fb;
        lbout[threadIdx.x] = a * ls.oa + b * ls.ob;
        la[threadIdx.x] = (int)a;
        if (MUL == MUL_MASK_AP) keep_a[threadIdx.x] = fabs(ex.ka[a]) < ex.cut_a;
        if (MUL == MUL_IK_A) {
            unsigned bad = 0;
            kdf[threadIdx.x] = df_from_double(ex.km[a], bad);
        }
    }
    __syncthreads();
    const int l = threadIdx.x & 15, j = threadIdx.x >> 4;
    const bool act = l < nl;
    // ---- load x[16 p1 + j] (FP64) with the load-time multiplier, and the line maximum
    double2 v[16];
    int mx = 0;
    if (act) {
        const double2* src = reinterpret_cast<const double2*>(in) + lbin[l];
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) v[p1] = src[(long)(16 * p1 + j) * ls.fp];
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) {
            const int p = 16 * p1 + j;
            if (MUL == MUL_MASK_AP) {
                if (!(keep_a[l] && keep_p[p])) v[p1] = make_double2(0.0, 0.0);
            }
            mx = max(mx, max(bexp(v[p1].x), bexp(v[p1].y)));
        }
        atomicMax(&emax[l], mx);
    }
    __syncthreads();
    const int ke = emax[l] - 1023;
    cdf a[16];
#pragma unroll
    for (int p1 = 0; p1 < 16; p1++) {
        a[p1] = mkc(df_from_double_shift(v[p1].x, ke), df_from_double_shift(v[p1].y, ke));
        if (MUL == MUL_IK_A || MUL == MUL_IK_P) {  // i k x in double-float (the FP64 products ran on the FP64 pipe)
            const dfv k = kdf[MUL == MUL_IK_A ? l : 16 * p1 + j];
            a[p1] = mul_mi(cscale(a[p1], k), true);
        }
    }
    // ---- DFT over p1, twiddles and exchange; then the DFT over j.  One copy of the DFT code
    // serves both stages (a loop that is not unrolled): the unrolled kernel outgrew the
    // instruction cache.
#pragma unroll 1
    for (int stage = 0; stage < 2; stage++) {
        dft16(a, inv, tw);
        if (stage == 1) break;
#pragma unroll
        for (int k1 = 1; k1 < 16; k1++) a[k1] = cmulw(a[k1], tw[j * k1], inv);
#pragma unroll
        for (int k1 = 0; k1 < 16; k1++) stc(smf, l * LSD + 16 * k1 + j, a[k1]);
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 16; jj++) a[jj] = ldc(smf, l * LSD + 16 * j + jj);  // this thread: k1 = j
    }
    // ---- store X[k1 + 16 k2]
    if (act) {
        const dfv sdf{scale_df.x, scale_df.y};
        const int ks = ke + scale_exp;
        double2* dst = reinterpret_cast<double2*>(out) + lbout[l];
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++) {
            cdf c = a[k2];
            if (use_scale_df) c = cscale(c, sdf);
            dst[(long)(j + 16 * k2) * ls.op] = cstore(c, ks);
        }
    }
}

// The fused z kinds on strided 256-point lines, four-step: forward (16 x 16 in registers, one
// exchange), the kind's multiplier at natural frequency f = j + 16 k2 (thread (line, j) then
// holds X[j + 16 k2], which is exactly the input layout of the backward four-step), backward,
// store; the same loads, multipliers and stores as k_fft_df's fused kinds.
template <int KIND>
__global__ void __launch_bounds__(256, 2) k_fft_df256_fk(const void* in, void* out, const FftLines ls,
                                                          const float4* __restrict__ twg, int scale_exp,
                                                          float2 scale_df, int use_scale_df, const FftExtra ex) {
    constexpr int LSD = 257;
    extern __shared__ __align__(16) float4 smf[];
    float4* tw = smf + 16 * LSD;  // W256^t, t < 256
    __shared__ int emax[16];
    __shared__ long lbin[16], lbout[16];
    __shared__ int lxi[16], lyj[16];
    __shared__ bool keep_ij[16];  // FK_DEALIAS: the x-y cut-offs of each line
    for (int t = threadIdx.x; t < 256; t += blockDim.x) tw[t] = twiddle_ext(twg, t, 128);
    const long l0 = (long)blockIdx.x * 16;
    const int nl = (int)min(16L, ls.nlines - l0);
    if (threadIdx.x < nl) {
        const long lg = l0 + threadIdx.x, a = lg % ls.na, b = lg / ls.na;
        emax[threadIdx.x] = 0;
        lbin[threadIdx.x] = a * ls.fa + b * ls.fb;
        lbout[threadIdx.x] = a * ls.oa + b * ls.ob;
        lxi[threadIdx.x] = (int)(lg % ex.nxh);
        lyj[threadIdx.x] = (int)(lg / ex.nxh);
        if (KIND == FK_DEALIAS)
            keep_ij[threadIdx.x] = fabs(ex.ka[lxi[threadIdx.x]]) < ex.cut_a && fabs(ex.kb[lyj[threadIdx.x]]) < ex.cut_b;
    }
    __syncthreads();
    const int l = threadIdx.x & 15, j = threadIdx.x >> 4;
    const bool act = l < nl;
    const long lg = l0 + l;
    // ---- load x[16 p1 + j] (the projection adds i (k1 uhat + k2 vhat) to dw/dz)
    double2 v[16];
    int mx = 0;
    if (act) {
        const double2* src = reinterpret_cast<const double2*>(in) + lbin[l];
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) v[p1] = src[(long)(16 * p1 + j) * ls.fp];
        if (KIND == FK_PROJECT) {
            const double k1 = ex.k1[lxi[l]], k2 = ex.k2[lyj[l]];
#pragma unroll
            for (int p1 = 0; p1 < 16; p1++) {
                const long idx = lg + (long)(16 * p1 + j) * ex.plane;
                const double2 uu = ex.u[idx], vv = ex.v[idx];
                const double tx = __dadd_rn(__dmul_rn(k1, uu.x), __dmul_rn(k2, vv.x));
                const double ty = __dadd_rn(__dmul_rn(k1, uu.y), __dmul_rn(k2, vv.y));
                v[p1] = make_double2(v[p1].x - ty, v[p1].y + tx);
            }
        }
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) mx = max(mx, max(bexp(v[p1].x), bexp(v[p1].y)));
        atomicMax(&emax[l], mx);
    }
    __syncthreads();
    const int ke = emax[l] - 1023;
    cdf a[16];
#pragma unroll
    for (int p1 = 0; p1 < 16; p1++) a[p1] = mkc(df_from_double_shift(v[p1].x, ke), df_from_double_shift(v[p1].y, ke));
    // ---- forward (stages 0, 1), multiplier, backward (stages 2, 3): one copy of the DFT code
#pragma unroll 1
    for (int st = 0; st < 4; st++) {
        const bool inv = st >= 2;
        dft16(a, inv, tw);
        if (st == 3) break;
        if (st == 1) {  // a[k2] = X[j + 16 k2]; lines past the end have no table entries
#pragma unroll
            for (int k2 = 0; k2 < 16 && act; k2++) {
                const int f = j + 16 * k2;
                if (KIND == FK_DEALIAS) {
                    if (!(keep_ij[l] && fabs(ex.kc[f]) < ex.cut_c)) a[k2] = czero();
                } else {
                    const double m = ex.mtab ? ex.mtab[lg * 256 + brev(f, 8)]
                                             : fk_mult_call<KIND>(ex.ka[lxi[l]], ex.kb[lyj[l]], ex.kc[f],
                                                                  lg == 0 && f == 0);
                    unsigned bad = 0;
                    a[k2] = cscale(a[k2], df_from_double(m, bad));
                }
            }
            continue;
        }
#pragma unroll
        for (int k1 = 1; k1 < 16; k1++) a[k1] = cmulw(a[k1], tw[j * k1], inv);
        if (st == 2) __syncthreads();  // the first exchange's reads are done
#pragma unroll
        for (int k1 = 0; k1 < 16; k1++) stc(smf, l * LSD + 16 * k1 + j, a[k1]);
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 16; jj++) a[jj] = ldc(smf, l * LSD + 16 * j + jj);
    }
    // ---- store x[j + 16 k2] (the projection also updates uhat and vhat)
    if (act) {
        const dfv sdf{scale_df.x, scale_df.y};
        const int ks = ke + scale_exp;
        double2* dst = reinterpret_cast<double2*>(out) + lbout[l];
        const double k1 = KIND == FK_PROJECT ? ex.k1[lxi[l]] : 0.0, k2 = KIND == FK_PROJECT ? ex.k2[lyj[l]] : 0.0;
#pragma unroll
        for (int k2i = 0; k2i < 16; k2i++) {
            const int p = j + 16 * k2i;
            cdf c = a[k2i];
            if (use_scale_df) c = cscale(c, sdf);
            const double2 r = cstore(c, ks);
            dst[(long)p * ls.op] = r;
            if (KIND == FK_DEALIAS && ex.edge_copy && p == 0) dst[256L * ls.op] = r;
            if (KIND == FK_PROJECT) {
                const long idx = lg + (long)p * ex.plane;
                double2 uu = ex.u[idx], vv = ex.v[idx];
                uu = make_double2(uu.x + k1 * r.y, uu.y - k1 * r.x);
                vv = make_double2(vv.x + k2 * r.y, vv.y - k2 * r.x);
                ex.u[idx] = uu;
                ex.v[idx] = vv;
            }
        }
    }
}

// Two real fields from two half spectra along x (N = 256; the second one given, or i km X,
// the x derivative of the first): both outputs are real, so the two c2r transforms run as one
// complex inverse transform of length N,
//   Z[q] = X'[q] + i Y'[q],  Z[N - q] = conj X'[q] + i conj Y'[q],
// (X', Y': the imaginary parts at q = 0 and N/2 dropped, as c2r does), out1 = Re z,
// out2 = Im z.  The complex transform is the four-step 16 x 16 of k_fft_df256 with thread
// (line, j) on consecutive points of a contiguous line (coalesced loads and stores).
__device__ __noinline__ double dstore_checked(dfv a, int k) { return shift_up(df_to_double(a), k); }
__device__ __forceinline__ double dstore(dfv a, int k) {
    if (k >= -800 && k <= 800) return df_to_double_kadd(a, (unsigned)(896 + k) << 20);
    return dstore_checked(a, k);  // out of line: rare, keeps the kernel small
}
// X split at line scale 2^k (the rare path of the derivative pair, out of line)
__device__ __noinline__ cdf split_at(double2 x, int k) {
    return mkc(df_from_double_shift(x.x, k), df_from_double_shift(x.y, k));
}

template <bool DERIV>  // Y = i km X (DERIV) or the second half spectrum in2
__global__ void __launch_bounds__(256, 2) k_fft_df_c2r_pair256(const double2* __restrict__ in, const double2* __restrict__ in2,
                                                                double* __restrict__ out1, double* __restrict__ out2,
                                                                const FftLines ls, const float4* __restrict__ twg,
                                                                const double* __restrict__ km, int scale_exp,
                                                                float2 scale_df, int use_scale_df) {
    constexpr int LSD = 16 * 17 + 1;  // rows of 17 (the exchange's reads then hit distinct banks)
    extern __shared__ __align__(16) float4 smf[];
    float4* tw = smf + 16 * LSD;  // W256^t, t < 256
    // each of the two fields is scaled by its own line maximum (emax1 / emax2) before the
    // packing, so either keeps its full relative precision whatever the other's magnitude
    __shared__ int emax1[16], emax2[16];
    __shared__ long lbin[16], lbout[16];
    __shared__ dfv kdf[129];
    __shared__ int kexp[129];  // DERIV: an exponent bound of km[q] (-2000 for 0)
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
        tw[t] = twiddle_ext(twg, t, 128);
        if (DERIV && t <= 128) {
            unsigned bad = 0;
            kdf[t] = df_from_double(km[t], bad);
            kexp[t] = km[t] == 0.0 ? -2000 : bexp(km[t]) - 1022;
        }
    }
    const long l0 = (long)blockIdx.x * 16;
    const int nl = (int)min(16L, ls.nlines - l0);
    if (threadIdx.x < nl) {
        const long lg = l0 + threadIdx.x, a = lg % ls.na, b = lg / ls.na;
        emax1[threadIdx.x] = 0;
        emax2[threadIdx.x] = 0;
        lbin[threadIdx.x] = a * ls.fa + b * ls.fb;
        lbout[threadIdx.x] = a * ls.oa + b * ls.ob;
    }
    __syncthreads();
    const int l = threadIdx.x >> 4, j = threadIdx.x & 15;
    const bool act = l < nl;
    // ---- load X[q] for the points q' = 16 p1 + j (q = q' up to N/2, else N - q')
    // (two inputs: the maximum first, then the values are read again after the barrier, so
    // that the 32 raw values need not stay in registers)
    double2 v[16];
    int mx = 0, my = 0;
    if (act) {
        const double2* src = in + lbin[l];
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) {
            const int qp = 16 * p1 + j, q = qp <= 128 ? qp : 256 - qp;
            v[p1] = src[q];
            const int bx = max(bexp(v[p1].x), bexp(v[p1].y));
            mx = max(mx, bx);
            if (DERIV && bx > 0) my = max(my, bx + kexp[q]);  // |k X| < 2^(that - 1023)
        }
        if (!DERIV) {
            const double2* src2 = in2 + lbin[l];
#pragma unroll
            for (int p1 = 0; p1 < 16; p1++) {
                const int qp = 16 * p1 + j;
                const double2 w = src2[qp <= 128 ? qp : 256 - qp];
                my = max(my, max(bexp(w.x), bexp(w.y)));
            }
        }
        atomicMax(&emax1[l], mx);
        atomicMax(&emax2[l], min(max(my, 0), 2046));
    }
    __syncthreads();
    const int ke = emax1[l] - 1023, ke2 = emax2[l] - 1023;
    // DERIV: i k X formed from X at the first scale, then moved to the second by 2^(ke - ke2)
    const int dsh = ke - ke2;
    const bool sh_ok = dsh >= -126 && dsh <= 127;
    const float shf = sh_ok ? __uint_as_float((unsigned)(dsh + 127) << 23) : 1.0f;
    cdf a[16];
#pragma unroll
    for (int p1 = 0; p1 < 16; p1++) {
        const int qp = 16 * p1 + j, q = qp <= 128 ? qp : 256 - qp;
        const bool edge = q == 0 || q == 128;
        const dfv xr = df_from_double_shift(v[p1].x, ke), xi0 = df_from_double_shift(v[p1].y, ke);
        const dfv xi = edge ? df_zero() : xi0;
        dfv yr, yi;
        if (DERIV) {
            const dfv k = kdf[q];
            dfv xr2 = xr, xi2 = xi0;
            if (sh_ok) {
                xr2 = dfv{xr.h * shf, xr.l * shf};
                xi2 = dfv{xi0.h * shf, xi0.l * shf};
            } else {
                const cdf x2 = split_at(v[p1], ke2);
                xr2 = cre(x2);
                xi2 = cim(x2);
            }
            yr = df_neg(df_norm(df_mul(xi2, k)));           // Re(i k X) (from the stored X)
            yi = edge ? df_zero() : df_norm(df_mul(xr2, k));  // Im(i k X)
        } else {
            const double2 w = act ? in2[lbin[l] + q] : make_double2(0.0, 0.0);
            yr = df_from_double_shift(w.x, ke2);
            yi = edge ? df_zero() : df_from_double_shift(w.y, ke2);
        }
        a[p1] = qp <= 128 ? mkc(df_norm(df_sub(xr, yi)), df_norm(df_add(xi, yr)))
                          : mkc(df_norm(df_add(xr, yi)), df_norm(df_sub(yr, xi)));
    }
    // ---- backward four-step (one copy of the DFT code for both stages)
#pragma unroll 1
    for (int stage = 0; stage < 2; stage++) {
        dft16(a, true, tw);
        if (stage == 1) break;
#pragma unroll
        for (int k1 = 1; k1 < 16; k1++) a[k1] = cmulw(a[k1], tw[j * k1], true);
#pragma unroll
        for (int k1 = 0; k1 < 16; k1++) stc(smf, l * LSD + 17 * k1 + j, a[k1]);
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 16; jj++) a[jj] = ldc(smf, l * LSD + 17 * j + jj);  // this thread: k1 = j
    }
    // ---- store z[j + 16 k2]: real part to out1, imaginary part to out2
    if (act) {
        const dfv sdf{scale_df.x, scale_df.y};
        const int ks = ke + scale_exp, ks2 = ke2 + scale_exp;
        double* d1 = out1 + lbout[l];
        double* d2 = out2 + lbout[l];
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++) {
            cdf c = a[k2];
            if (use_scale_df) c = cscale(c, sdf);
            const long o = (long)(j + 16 * k2) * ls.op;
            d1[o] = dstore(cre(c), ks);
            d2[o] = dstore(cim(c), ks2);
        }
    }
}

// Two real fields along x (N = 256) to their half spectra with one complex transform:
// z = x1 2^-e1 + i x2 2^-e2 (each field scaled by its own line maximum), Z = FFT(z), and for
// k = 0..N/2: X1 = (Z[k] + conj Z[N-k]) / 2, X2 = -i (Z[k] - conj Z[N-k]) / 2, each stored
// with its own exponent.  The transform is the register four-step 16 x 16.
__global__ void __launch_bounds__(256, 2) k_fft_df_r2c_pair256(const double* __restrict__ in1,
                                                                const double* __restrict__ in2,
                                                                double2* __restrict__ out1, double2* __restrict__ out2,
                                                                const FftLines ls, const float4* __restrict__ twg,
                                                                int scale_exp, float2 scale_df, int use_scale_df) {
    constexpr int LSD = 16 * 17 + 1;
    extern __shared__ __align__(16) float4 smf[];
    float4* tw = smf + 16 * LSD;  // W256^t, t < 256
    __shared__ int emax1[16], emax2[16];
    __shared__ long lbin[16], lbout[16];
    for (int t = threadIdx.x; t < 256; t += blockDim.x) tw[t] = twiddle_ext(twg, t, 128);
    const long l0 = (long)blockIdx.x * 16;
    const int nl = (int)min(16L, ls.nlines - l0);
    if (threadIdx.x < nl) {
        const long lg = l0 + threadIdx.x, a = lg % ls.na, b = lg / ls.na;
        emax1[threadIdx.x] = 0;
        emax2[threadIdx.x] = 0;
        lbin[threadIdx.x] = a * ls.fa + b * ls.fb;
        lbout[threadIdx.x] = a * ls.oa + b * ls.ob;
    }
    __syncthreads();
    const int l = threadIdx.x >> 4, j = threadIdx.x & 15;
    const bool act = l < nl;
    double2 v[16];  // (x1, x2) at point 16 p1 + j
    if (act) {
        int m1 = 0, m2 = 0;
#pragma unroll
        for (int p1 = 0; p1 < 16; p1++) {
            const long o = lbin[l] + 16 * p1 + j;
            v[p1] = make_double2(in1[o], in2[o]);
            m1 = max(m1, bexp(v[p1].x));
            m2 = max(m2, bexp(v[p1].y));
        }
        atomicMax(&emax1[l], m1);
        atomicMax(&emax2[l], m2);
    }
    __syncthreads();
    const int ke1 = emax1[l] - 1023, ke2 = emax2[l] - 1023;
    cdf a[16];
#pragma unroll
    for (int p1 = 0; p1 < 16; p1++) a[p1] = mkc(df_from_double_shift(v[p1].x, ke1), df_from_double_shift(v[p1].y, ke2));
#pragma unroll 1
    for (int stage = 0; stage < 2; stage++) {
        dft16(a, false, tw);
        if (stage == 1) break;
#pragma unroll
        for (int k1 = 1; k1 < 16; k1++) a[k1] = cmulw(a[k1], tw[j * k1], false);
#pragma unroll
        for (int k1 = 0; k1 < 16; k1++) stc(smf, l * LSD + 17 * k1 + j, a[k1]);
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 16; jj++) a[jj] = ldc(smf, l * LSD + 17 * j + jj);  // this thread: k1 = j
    }
    // ---- Z in natural order, then the two half spectra
    __syncthreads();  // the exchange's reads are done
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) stc(smf, l * LSD + j + 16 * k2, a[k2]);
    __syncthreads();
    if (act) {
        const dfv sdf{scale_df.x, scale_df.y};
        const int ks1 = ke1 + scale_exp, ks2 = ke2 + scale_exp;
        for (int k = j; k <= 128; k += 16) {
            const cdf zk = ldc(smf, l * LSD + k), zn = ldc(smf, l * LSD + ((256 - k) & 255));
            // X1 = (zk + conj zn) / 2, X2 = -i (zk - conj zn) / 2
            const cdf czn = cconj(zn);
            cdf x1 = chalf(cadd(zk, czn));
            cdf x2 = chalf(mul_mi(csub(zk, czn), false));
            if (use_scale_df) {
                x1 = cscale(x1, sdf);
                x2 = cscale(x2, sdf);
            }
            out1[lbout[l] + (long)k * ls.op] = cstore(x1, ks1);
            out2[lbout[l] + (long)k * ls.op] = cstore(x2, ks2);
        }
    }
}

std::mutex g_twdf_mu;
std::map<std::pair<int, int>, float4*> g_twdf;  // (device, n) -> df exp(-2 pi i t / n), t < n/2

void split_ld(long double x, float& h, float& l) {
    h = (float)x;
    l = (float)(x - (long double)h);
}

int twiddles_df(int n, const float4** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PS_ECUDA;
    std::lock_guard<std::mutex> lock(g_twdf_mu);
    auto it = g_twdf.find({dev, n});
    if (it != g_twdf.end()) {
        *out = it->second;
        return PS_OK;
    }
    std::vector<float4> h(std::max(1, n / 2));
    for (int t = 0; t < n / 2; t++) {
        const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
        float ch, cl, sh, sl;
        split_ld(cosl(ang), ch, cl);
        split_ld(sinl(ang), sh, sl);
        h[t] = make_float4(ch, cl, sh, sl);
    }
    float4* d = nullptr;
    if (cudaMalloc(&d, sizeof(float4) * h.size()) != cudaSuccess) {
        cudaGetLastError();
        return PS_ENOMEM;
    }
    if (cudaMemcpy(d, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return PS_ECUDA;
    }
    g_twdf[{dev, n}] = d;
    *out = d;
    return PS_OK;
}

template <int I, int O, int K>
int launch_df_t(const void* in, void* out, const FftLines& ls, const float4* tw, int logn, int lb, int sign,
                int sexp, float2 sdf, int use_sdf, int oddball, const FftExtra& ex, cudaStream_t s) {
    // lines padded by one point, then the 3n/4 twiddles
    const size_t smem = sizeof(float4) * ((size_t)lb * (size_t)((1 << logn) + 1) + (size_t)(3 << logn) / 4);
    auto kern = k_fft_df<I, O, K>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PS_ECUDA;
    const long blocks = (ls.nlines + lb - 1) / lb;
    if (blocks > 0x7fffffffL) return PS_ENOTSUP;
    kern<<<(unsigned)blocks, 256, smem, s>>>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use_sdf, oddball, ex);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

}  // namespace

int fft_df_mult_table(int kind, const double* ka, const double* kb, const double* kc, int nxh, int ny, int nz,
                      double** out, cudaStream_t s) {
    *out = nullptr;
    int logn = 0;
    while ((1 << logn) < nz) logn++;
    if ((1 << logn) != nz || (kind != FK_PROJECT && kind != FK_POISSON3D)) return PS_EINVAL;
    const long nlines = (long)nxh * ny;
    if (cudaMalloc(reinterpret_cast<void**>(out), sizeof(double) * (size_t)(nlines << logn)) != cudaSuccess) {
        *out = nullptr;
        cudaGetLastError();
        return PS_ENOMEM;
    }
    const unsigned g = 152 * 8;
    if (kind == FK_PROJECT) {
        k_mult_table<FK_PROJECT><<<g, 256, 0, s>>>(ka, kb, kc, nxh, logn, nlines, *out);
    } else {
        k_mult_table<FK_POISSON3D><<<g, 256, 0, s>>>(ka, kb, kc, nxh, logn, nlines, *out);
    }
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

// the four-step 256-point kernel unless PADE_FFT_FOURSTEP=0 (a tuning override: k_fft_df instead)
bool fourstep_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("PADE_FFT_FOURSTEP");
        return !(e && e[0] == '0');
    }();
    return on;
}

int fft_r2c_pair_df(const double* in1, const double* in2, void* out1, void* out2, const FftLines& ls, int n,
                    double scale, cudaStream_t s) {
    if (n != 256 || ls.fp != 1 || ls.op != 1 || !fourstep_enabled()) return PS_ENOTSUP;
    if (ls.nlines <= 0) return PS_OK;
    const float4* tw = nullptr;
    int rc = twiddles_df(n, &tw);
    if (rc != PS_OK) return rc;
    int e2 = 0;
    const double mant = std::frexp(scale, &e2);
    int sexp = 0, use = 0;
    float2 sdf = make_float2(1.0f, 0.0f);
    if (mant == 0.5) {
        sexp = e2 - 1;
    } else {
        use = 1;
        sdf.x = (float)scale;
        sdf.y = (float)(scale - (double)sdf.x);
    }
    const size_t smem = sizeof(float4) * ((16 * 17 + 1) * 16 + 256);
    if (cudaFuncSetAttribute(k_fft_df_r2c_pair256, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return PS_ECUDA;
    const long blocks = (ls.nlines + 15) / 16;
    if (blocks > 0x7fffffffL) return PS_ENOTSUP;
    k_fft_df_r2c_pair256<<<(unsigned)blocks, 256, smem, s>>>(in1, in2, static_cast<double2*>(out1),
                                                             static_cast<double2*>(out2), ls, tw, sexp, sdf, use);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

int fft_c2r_pair_df(const void* in, const void* in2, double* out1, double* out2, const FftLines& ls, int n,
                    double scale, const double* km, cudaStream_t s) {
    if (n != 256 || ls.fp != 1 || ls.op != 1 || (!km && !in2) || !fourstep_enabled()) return PS_ENOTSUP;
    if (ls.nlines <= 0) return PS_OK;
    const float4* tw = nullptr;
    int rc = twiddles_df(n, &tw);
    if (rc != PS_OK) return rc;
    int e2 = 0;
    const double mant = std::frexp(scale, &e2);
    int sexp = 0, use = 0;
    float2 sdf = make_float2(1.0f, 0.0f);
    if (mant == 0.5) {
        sexp = e2 - 1;
    } else {
        use = 1;
        sdf.x = (float)scale;
        sdf.y = (float)(scale - (double)sdf.x);
    }
    const size_t smem = sizeof(float4) * ((16 * 17 + 1) * 16 + 256);
    auto kern = in2 ? k_fft_df_c2r_pair256<false> : k_fft_df_c2r_pair256<true>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PS_ECUDA;
    const long blocks = (ls.nlines + 15) / 16;
    if (blocks > 0x7fffffffL) return PS_ENOTSUP;
    kern<<<(unsigned)blocks, 256, smem, s>>>(static_cast<const double2*>(in), static_cast<const double2*>(in2), out1,
                                             out2, ls, tw, km, sexp, sdf, use);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

int fft_launch_df(int in_mode, int out_mode, int kind, int logn, int sign, double scale, int oddball, const void* in,
                  void* out, const FftLines& ls, const FftExtra& ex, cudaStream_t s) {
    const int n = 1 << logn;
    const float4* tw = nullptr;
    const int rc = twiddles_df(n, &tw);
    if (rc != PS_OK) return rc;
    const int lb = std::max(1, std::min(64, 4096 >> logn));
    // scale = 2^sexp exactly when its mantissa is 1/2; otherwise a df multiplier
    int e2 = 0;
    const double mant = std::frexp(scale, &e2);
    int sexp = 0, use = 0;
    float2 sdf = make_float2(1.0f, 0.0f);
    if (mant == 0.5) {
        sexp = e2 - 1;
    } else {
        use = 1;
        sdf.x = (float)scale;
        sdf.y = (float)(scale - (double)sdf.x);
    }
    if (kind != FK_PLAIN && logn == 8 && ls.fp != 1 && ls.op != 1 && fourstep_enabled()) {
        const size_t smem = sizeof(float4) * (16 * 257 + 256);
        auto kern = kind == FK_PROJECT ? k_fft_df256_fk<FK_PROJECT>
                    : kind == FK_POISSON3D ? k_fft_df256_fk<FK_POISSON3D>
                                           : k_fft_df256_fk<FK_DEALIAS>;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
        const long blocks = (ls.nlines + 15) / 16;
        if (blocks > 0x7fffffffL) return PS_ENOTSUP;
        kern<<<(unsigned)blocks, 256, smem, s>>>(in, out, ls, tw, sexp, sdf, use, ex);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    if (kind == FK_PROJECT)
        return launch_df_t<IN_COMPLEX, OUT_COMPLEX, FK_PROJECT>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, 0, ex, s);
    if (kind == FK_POISSON3D)
        return launch_df_t<IN_COMPLEX, OUT_COMPLEX, FK_POISSON3D>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, 0, ex,
                                                                  s);
    if (kind == FK_DEALIAS)
        return launch_df_t<IN_COMPLEX, OUT_COMPLEX, FK_DEALIAS>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, 0, ex, s);
    if (in_mode == IN_COMPLEX && out_mode == OUT_COMPLEX && logn == 8 && ls.fp != 1 && ls.op != 1 && fourstep_enabled()) {
        // strided 256-point lines (the y transforms): the register-resident four-step kernel
        const size_t smem = sizeof(float4) * (16 * 257 + 256);
        auto kern = ex.mul == MUL_MASK_AP ? k_fft_df256<MUL_MASK_AP>
                    : ex.mul == MUL_IK_A  ? k_fft_df256<MUL_IK_A>
                    : ex.mul == MUL_IK_P  ? k_fft_df256<MUL_IK_P>
                                          : k_fft_df256<MUL_NONE>;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
        const long blocks = (ls.nlines + 15) / 16;
        if (blocks > 0x7fffffffL) return PS_ENOTSUP;
        kern<<<(unsigned)blocks, 256, smem, s>>>(in, out, ls, tw, sign, sexp, sdf, use, ex);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    if (in_mode == IN_COMPLEX && out_mode == OUT_COMPLEX)
        return launch_df_t<IN_COMPLEX, OUT_COMPLEX, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, 0, ex, s);
    // 16-byte pair loads (r2c input) / stores (c2r output) need aligned real lines
    const bool aligned = in_mode == IN_REAL
                             ? ((reinterpret_cast<uintptr_t>(in) & 15) == 0 && ls.fa % 2 == 0 && ls.fb % 2 == 0)
                             : ((reinterpret_cast<uintptr_t>(out) & 15) == 0 && ls.oa % 2 == 0 && ls.ob % 2 == 0);
    const bool xreal = ls.fp == 1 && ls.op == 1 && logn >= 3 && aligned &&
                       (ex.mul == MUL_NONE || (in_mode == IN_HALF && ex.mul == MUL_IK_P));
    if (xreal && ((in_mode == IN_REAL && out_mode == OUT_HALF) || (in_mode == IN_HALF && out_mode == OUT_REAL))) {
        // half-length complex transform; lb lines of M = n/2 points per CTA
        const int lbr = std::max(1, std::min(64, 4096 >> (logn - 1)));
        const size_t smem = sizeof(float4) * (((size_t)lbr << (logn - 1)) + (size_t)(3 << logn) / 4);
        const bool r2c = in_mode == IN_REAL;
        auto kern = r2c ? k_fft_df_real<true> : k_fft_df_real<false>;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return PS_ECUDA;
        const long blocks = (ls.nlines + lbr - 1) / lbr;
        kern<<<(unsigned)blocks, 256, smem, s>>>(in, out, ls, tw, logn, lbr, sexp, sdf, use, oddball,
                                                 ex.mul == MUL_IK_P ? ex.km : nullptr);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    if (ex.mul != MUL_NONE) return PS_ENOTSUP;  // on real / half lines only the real kernel has one
    if (in_mode == IN_REAL && out_mode == OUT_HALF)
        return launch_df_t<IN_REAL, OUT_HALF, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, 0, ex, s);
    if (in_mode == IN_HALF && out_mode == OUT_REAL)
        return launch_df_t<IN_HALF, OUT_REAL, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, sexp, sdf, use, oddball, ex, s);
    return PS_EINVAL;
}

}  // namespace pade
