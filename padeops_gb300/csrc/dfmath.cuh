// Double-float ("df") arithmetic on the FP32 pipes.
//
// A df value is an unevaluated sum h + l of two floats.  GB300 runs FP64 (and the
// FP64<->FP32 conversions) at 1/56 of the FP32 rate, so the FP64 operator path keeps its
// arithmetic in df: inputs are split with integer instructions, sums and products use
// the classical error-free transformations (Knuth's TwoSum, FMA-based TwoProduct), and
// results go back to FP64 with integer instructions plus one FP64 add.  All float
// operations use the _rn intrinsics so the compiler cannot contract them into FMAs,
// which would break the error-free transformations.
#pragma once
#include <cuda_runtime.h>

namespace pade {

struct dfv {
    float h, l;
};

// Split an FP64 value into (hi, lo): hi keeps the leading 24 significant bits
// (truncated), lo the remaining 29 bits rounded to float.  Exact to 2^-47 relative.
// Full precision needs the biased FP64 exponent in [949, 1150] (|d| in [2^-74, 2^127));
// other non-zero values set `bad` and are flushed.  The kernels scale each line into
// range first (df_from_double_shift), so only infinities and NaNs reach that case.
__device__ __forceinline__ dfv df_from_double(double d, unsigned& bad) {
    const unsigned lo32 = (unsigned)__double2loint(d);
    const unsigned hi32 = (unsigned)__double2hiint(d);
    const unsigned ex = hi32 & 0x7FF00000u;
    const unsigned sign = hi32 & 0x80000000u;
    const bool ok = (ex - (949u << 20)) <= ((1150u - 949u) << 20);
    const bool zero = ((hi32 & 0x7FFFFFFFu) | lo32) == 0u;
    bad |= (unsigned)(!ok && !zero);
    const unsigned hb = (((hi32 - (896u << 20)) << 3) & 0x7FFFFFF8u) | (lo32 >> 29) | sign;
    const float lf = __uint2float_rn(lo32 & 0x1FFFFFFFu);
    const unsigned sb = (ex - (948u << 20)) << 3;
    float lo = __fmul_rn(lf, __uint_as_float(sb));
    lo = __uint_as_float(__float_as_uint(lo) ^ sign);
    dfv r;
    r.h = ok ? __uint_as_float(hb) : 0.0f;
    r.l = ok ? lo : 0.0f;
    return r;
}

// Exact float -> double with integer instructions (zero and subnormal floats map to 0).
__device__ __forceinline__ double float_bits_to_double(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7FFFFFFFu;
    const unsigned sg = b & 0x80000000u;
    const bool z = mag < 0x00800000u;
    const unsigned hi = z ? sg : (((mag >> 3) + (896u << 20)) | sg);
    const unsigned lo = z ? 0u : (b << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// (h + l) rounded once to FP64: two exact conversions and one FP64 add.
__device__ __forceinline__ double df_to_double(dfv a) {
    return __dadd_rn(float_bits_to_double(a.h), float_bits_to_double(a.l));
}

// Per-line power-of-two scaling keeps the df range relative to a line's maximum: values
// are split as d * 2^-k and reassembled as r * 2^k, both on the exponent bits.
// Biased FP64 exponent of d (0 for zero and subnormals, 2047 for inf/NaN).
__device__ __forceinline__ int bexp(double d) { return (__double2hiint(d) >> 20) & 0x7FF; }

// d * 2^-k split into a df value: df_from_double with the exponent lowered by k on the
// bits; zero for zero/subnormal input and when the shifted value is below 2^-74.
__device__ __forceinline__ dfv df_from_double_shift(double d, int k) {
    const unsigned lo32 = (unsigned)__double2loint(d);
    const unsigned h0 = (unsigned)__double2hiint(d);
    const int e2 = (int)((h0 >> 20) & 0x7FFu) - k;
    const bool ok = (h0 & 0x7FF00000u) != 0u && e2 >= 949 && e2 <= 1149;
    const unsigned sign = h0 & 0x80000000u;
    const unsigned hi32 = (h0 & 0x800FFFFFu) | ((unsigned)(e2 & 0x7FF) << 20);
    const unsigned ex = hi32 & 0x7FF00000u;
    const unsigned hb = (((hi32 - (896u << 20)) << 3) & 0x7FFFFFF8u) | (lo32 >> 29) | sign;
    const float lf = __uint2float_rn(lo32 & 0x1FFFFFFFu);
    const unsigned sb = (ex - (948u << 20)) << 3;
    float lo = __fmul_rn(lf, __uint_as_float(sb));
    lo = __uint_as_float(__float_as_uint(lo) ^ sign);
    return dfv{ok ? __uint_as_float(hb) : 0.0f, ok ? lo : 0.0f};
}

// The split of df_from_double_shift for values already scaled below 2 (a line's maximum in
// [1, 2) after the shift by k): about half the instructions.  The FP64 exponent's low 9 bits
// and the top 23 mantissa bits are shifted together into the FP32 layout and rebased by one
// integer add (the shifted exponent e - k - 896 lies in [53, 127], so the 9-bit field cannot
// carry); values below 2^-74 of the maximum (and zeros) give zero.  Per-line constants:
struct SplitK {
    unsigned kb, kc, thr;
};

__device__ __forceinline__ SplitK split_consts(int k) {
    SplitK s;
    s.kb = (unsigned)(-(k + 896)) << 23;
    s.kc = (unsigned)(-(k + 948)) << 23;
    s.thr = (unsigned)max(949 + k, 1) << 20;
    return s;
}

__device__ __forceinline__ dfv df_split_line(double d, const SplitK& s) {
    const unsigned lo32 = (unsigned)__double2loint(d);
    const unsigned hi32 = (unsigned)__double2hiint(d);
    const unsigned sign = hi32 & 0x80000000u;
    // mantissa top 23 bits below the low 8 exponent bits: (hi32 << 3) | (lo32 >> 29)
    const unsigned t = __funnelshift_l(lo32, hi32, 3);
    const unsigned hb = (t + s.kb) | sign;  // exponent e - k - 896 in [53, 127] fits the field
    const float lf = __uint2float_rn(lo32 & 0x1FFFFFFFu);
    const unsigned sb = ((t & 0xFF800000u) + s.kc) | sign;  // 2^(e - k - 1075), signed
    const float lo = __fmul_rn(lf, __uint_as_float(sb));
    const bool ok = (hi32 & 0x7FF00000u) >= s.thr;
    return dfv{ok ? __uint_as_float(hb) : 0.0f, ok ? lo : 0.0f};
}

// float x * 2^k as an exact double (x normal; zero, subnormal x and results below the
// normal FP64 range give 0, results above it infinity)
__device__ __forceinline__ double float_bits_to_double_shift(float x, int k) {
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7FFFFFFFu;
    const unsigned sg = b & 0x80000000u;
    const int e2 = (int)(mag >> 23) + 896 + k;  // FP64 biased exponent of the result
    const bool z = mag < 0x00800000u || e2 <= 0;
    const bool inf = !z && e2 >= 2047;           // beyond the FP64 range: infinity
    const unsigned hi = z ? sg : (inf ? (sg | 0x7FF00000u) : ((((mag >> 3) & 0x000FFFFFu) | ((unsigned)e2 << 20)) | sg));
    const unsigned lo = (z || inf) ? 0u : (b << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// (h + l) * 2^k rounded once to FP64
__device__ __forceinline__ double df_to_double_shift(dfv a, int k) {
    return __dadd_rn(float_bits_to_double_shift(a.h, k), float_bits_to_double_shift(a.l, k));
}

// float x * 2^k as an exact double when -800 <= k <= 800 (every normal float then lands
// in the normal FP64 range, so no range checks); zero and subnormal x give 0.
// kadd = (896 + k) << 20, the FP32-to-FP64 exponent rebias plus the shift.
__device__ __forceinline__ double float_bits_to_double_kadd(float x, unsigned kadd) {
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7FFFFFFFu;
    const unsigned sg = b & 0x80000000u;
    const bool z = mag < 0x00800000u;
    const unsigned hi = z ? sg : (((mag >> 3) + kadd) | sg);
    return __hiloint2double((int)hi, z ? 0 : (int)(b << 29));
}

// (h + l) * 2^k rounded once to FP64, for -800 <= k <= 800
__device__ __forceinline__ double df_to_double_kadd(dfv a, unsigned kadd) {
    return __dadd_rn(float_bits_to_double_kadd(a.h, kadd), float_bits_to_double_kadd(a.l, kadd));
}

// r * 2^k on the exponent bits (flushes below the normal range)
__device__ __forceinline__ double shift_up(double r, int k) {
    const unsigned lo = (unsigned)__double2loint(r);
    unsigned hi = (unsigned)__double2hiint(r);
    const int ex = (int)((hi >> 20) & 0x7FFu);
    if (ex == 0) return 0.0;
    int e2 = ex + k;
    if (e2 <= 0) return 0.0;
    if (e2 >= 2047) return __hiloint2double((int)((hi & 0x80000000u) | 0x7FF00000u), 0);
    hi = (hi & 0x800FFFFFu) | ((unsigned)e2 << 20);
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ dfv df_zero() { return dfv{0.0f, 0.0f}; }

// a + b, high parts by TwoSum (exact), low parts by one rounded add; not renormalised
__device__ __forceinline__ dfv df_add(dfv a, dfv b) {
    const float s = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return dfv{s, __fadd_rn(e, __fadd_rn(a.l, b.l))};
}

__device__ __forceinline__ dfv df_neg(dfv a) { return dfv{-a.h, -a.l}; }
__device__ __forceinline__ dfv df_sub(dfv a, dfv b) { return df_add(a, df_neg(b)); }

// FastTwoSum renormalisation (|h| >= |l| holds for every value this code produces)
__device__ __forceinline__ dfv df_norm(dfv a) {
    const float s = __fadd_rn(a.h, a.l);
    return dfv{s, __fsub_rn(a.l, __fsub_rn(s, a.h))};
}

// a * c (TwoProduct of the high parts, cross terms in FP32); not renormalised
__device__ __forceinline__ dfv df_mul(dfv a, dfv c) {
    const float ph = __fmul_rn(a.h, c.h);
    float pe = __fmaf_rn(a.h, c.h, -ph);
    pe = __fmaf_rn(a.h, c.l, pe);
    pe = __fmaf_rn(a.l, c.h, pe);
    return dfv{ph, pe};
}

__device__ __forceinline__ dfv df_shfl_up(dfv v, unsigned d, int w) {
    return dfv{__shfl_up_sync(0xffffffffu, v.h, d, w), __shfl_up_sync(0xffffffffu, v.l, d, w)};
}
__device__ __forceinline__ dfv df_shfl_down(dfv v, unsigned d, int w) {
    return dfv{__shfl_down_sync(0xffffffffu, v.h, d, w), __shfl_down_sync(0xffffffffu, v.l, d, w)};
}
__device__ __forceinline__ dfv df_shfl_idx(dfv v, int src, int w) {
    return dfv{__shfl_sync(0xffffffffu, v.h, src, w), __shfl_sync(0xffffffffu, v.l, src, w)};
}

// Two double-float values in packed form for the FP32x2 instructions (add/mul/fma.rn.f32x2,
// each component rounded as the scalar instruction, so every error-free transformation
// stays exact): h = the two high parts, l = the two low parts.
struct df2 {
    float2 h, l;
};

__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __fadd2_rn(a, f2neg(b)); }

__device__ __forceinline__ df2 d2_zero() { return df2{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
__device__ __forceinline__ df2 d2_of(float4 v) { return df2{make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 d2_f4(df2 a) { return make_float4(a.h.x, a.h.y, a.l.x, a.l.y); }
// a coefficient broadcast to both components ({h, h, l, l} in shared memory)
__device__ __forceinline__ df2 d2_bcast(dfv c) { return df2{make_float2(c.h, c.h), make_float2(c.l, c.l)}; }
__device__ __forceinline__ dfv d2_x(df2 a) { return dfv{a.h.x, a.l.x}; }
__device__ __forceinline__ dfv d2_y(df2 a) { return dfv{a.h.y, a.l.y}; }
__device__ __forceinline__ df2 d2_pack(dfv x, dfv y) { return df2{make_float2(x.h, y.h), make_float2(x.l, y.l)}; }
__device__ __forceinline__ dfv d2c_scalar(float4 c) { return dfv{c.x, c.z}; }

// df_add, df_norm and df_mul above, componentwise
__device__ __forceinline__ df2 d2_add(df2 a, df2 b) {
    const float2 s = f2add(a.h, b.h);
    const float2 bb = f2sub(s, a.h);
    const float2 e = f2add(f2sub(a.h, f2sub(s, bb)), f2sub(b.h, bb));
    return df2{s, f2add(e, f2add(a.l, b.l))};
}
__device__ __forceinline__ df2 d2_neg(df2 a) { return df2{f2neg(a.h), f2neg(a.l)}; }
__device__ __forceinline__ df2 d2_sub(df2 a, df2 b) { return d2_add(a, d2_neg(b)); }
__device__ __forceinline__ df2 d2_norm(df2 a) {
    const float2 s = f2add(a.h, a.l);
    return df2{s, f2sub(a.l, f2sub(s, a.h))};
}
__device__ __forceinline__ df2 d2_mul(df2 a, df2 c) {
    const float2 ph = __fmul2_rn(a.h, c.h);
    float2 pe = __ffma2_rn(a.h, c.h, f2neg(ph));
    pe = __ffma2_rn(a.h, c.l, pe);
    pe = __ffma2_rn(a.l, c.h, pe);
    return df2{ph, pe};
}
// base - c1 x1 - c2 x2 and acc + m0 v1 + m1 v2 (ArDF::fms2 / mac2, componentwise)
__device__ __forceinline__ df2 d2_fms2(df2 base, df2 c1, df2 x1, df2 c2, df2 x2) {
    return d2_norm(d2_sub(d2_sub(base, d2_mul(x1, c1)), d2_mul(x2, c2)));
}
__device__ __forceinline__ df2 d2_fms1(df2 base, df2 c1, df2 x1) { return d2_norm(d2_sub(base, d2_mul(x1, c1))); }
__device__ __forceinline__ df2 d2_mac2(df2 acc, df2 m0, df2 v1, df2 m1, df2 v2) {
    return d2_norm(d2_add(d2_add(acc, d2_mul(v1, m0)), d2_mul(v2, m1)));
}
__device__ __forceinline__ df2 d2_mac1(df2 acc, df2 m0, df2 v1) { return d2_norm(d2_add(acc, d2_mul(v1, m0))); }

}  // namespace pade
