// Batched FP64 FFTs for the spectral layer and the periodic Poisson solves.
//
// k_fft transforms lines of n = 2^m complex points along any strided direction of a 3-D
// array.  A CTA stages lb lines in shared memory, loads them in bit-reversed order and
// runs the m radix-2 decimation-in-time stages in place (natural-order result).  Loads
// and stores put consecutive threads on consecutive points when a line is contiguous
// (x lines) and on consecutive lines otherwise (y and z lines, whose neighbours are
// adjacent in memory), so global accesses coalesce in both cases.
//
// Conventions follow FFTW, which the reference calls: forward = exp(-2 pi i jk/n),
// backward = exp(+2 pi i jk/n), both unnormalised; callers pass the scale.  Input
// modes: complex, real (r2c along x), half spectrum (n/2+1 entries expanded by Hermitian
// symmetry, for c2r; the imaginary parts of the mean and Nyquist entries are ignored
// like FFTW's c2r does).  Output modes: all n entries, the first n/2+1 (r2c), or the
// real part (c2r).
//
// Two fused kinds keep a line in shared memory from load to store:
//  * FK_PROJECT, the z part of PadePoisson's periodic projection (PadePoisson.F90:
//    386-432): load f = dwdz + i (k1 uhat + k2 vhat), forward transform, multiply by
//    -1/(k1^2 + k2^2 + k3mod^2) (0 where that is <= 1e-14, PadePoisson.F90:100-111),
//    backward transform (decimation in frequency, so no reordering pass), scale by 1/nz,
//    store the pressure and update uhat -= i k1 p, vhat -= i k2 p in the same pass.
//  * FK_POISSON3D, the z part of PoissonPeriodic (PoissonPeriodic.F90:89-111):
//    forward, multiply by -1/(kx^2 + ky^2 + kz^2 + 1e-20) with the zero mode set to 0,
//    backward.
//  * FK_DEALIAS, spectral%dealias / dealias_edgeField for periodic z (spectral.F90:
//    314-363, mask 777-811): forward, multiply by the 0/1 mask, backward times 1/nz; for
//    an edge field the first plane is copied to plane nz+1.
// FK_PLAIN can multiply by i*k on load (the mtimes_ik1/ik2 pass before an inverse
// transform, spectral.F90:235-310), with the reference's two products per point.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "fft.h"
#include "operators.h"

namespace pade {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int brev(int p, int logn) { return (int)(__brev((unsigned)p) >> (32 - logn)); }

// |k|^2 in the reference's evaluation order, (a^2 + b^2) + c^2, without contraction
__device__ __forceinline__ double ksq(double a, double b, double c) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// radix-2 decimation-in-time stages, bit-reversed input -> natural order
__device__ __forceinline__ void dit(double2* x, int nl, int logn, const double2* __restrict__ tw, bool conj) {
    const int half = 1 << (logn - 1);
    const int work = nl << (logn - 1);
    for (int s = 0; s < logn; s++) {
        for (int e = threadIdx.x; e < work; e += blockDim.x) {
            const int l = e >> (logn - 1), j = e & (half - 1);
            const int k = j & ((1 << s) - 1);
            const int i0 = (l << logn) + ((j >> s) << (s + 1)) + k;
            const int i1 = i0 + (1 << s);
            double2 w = __ldg(&tw[k << (logn - 1 - s)]);
            if (conj) w.y = -w.y;
            const double2 a = x[i0];
            const double2 b = cmul(x[i1], w);
            x[i0] = make_double2(a.x + b.x, a.y + b.y);
            x[i1] = make_double2(a.x - b.x, a.y - b.y);
        }
        __syncthreads();
    }
}

// radix-2 decimation-in-frequency stages, natural input -> bit-reversed order
__device__ __forceinline__ void dif(double2* x, int nl, int logn, const double2* __restrict__ tw, bool conj) {
    const int half = 1 << (logn - 1);
    const int work = nl << (logn - 1);
    for (int s = logn - 1; s >= 0; s--) {
        for (int e = threadIdx.x; e < work; e += blockDim.x) {
            const int l = e >> (logn - 1), j = e & (half - 1);
            const int k = j & ((1 << s) - 1);
            const int i0 = (l << logn) + ((j >> s) << (s + 1)) + k;
            const int i1 = i0 + (1 << s);
            double2 w = __ldg(&tw[k << (logn - 1 - s)]);
            if (conj) w.y = -w.y;
            const double2 a = x[i0];
            const double2 b = x[i1];
            x[i0] = make_double2(a.x + b.x, a.y + b.y);
            x[i1] = cmul(make_double2(a.x - b.x, a.y - b.y), w);
        }
        __syncthreads();
    }
}

// in and out may be the same array (in-place transforms): every CTA reads its own lines
// completely before a barrier and writes them after it.
template <int IN, int OUT, int KIND>
__global__ void __launch_bounds__(256) k_fft(const void* in, void* out, const FftLines ls,
                                             const double2* __restrict__ tw, int logn, int lb, int sign,
                                             double scale, int oddball, const FftExtra ex) {
    extern __shared__ __align__(16) double2 sm[];
    const int n = 1 << logn, half = n >> 1;
    const long l0 = (long)blockIdx.x * lb;
    const int nl = (int)min((long)lb, ls.nlines - l0);
    const int total = nl << logn;
    const bool pin = ls.fp == 1, pout = ls.op == 1;  // contiguous lines: points fastest

    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int l = pin ? (e >> logn) : (e % nl);
        const int p = pin ? (e & (n - 1)) : (e / nl);
        const long lg = l0 + l, a = lg % ls.na, b = lg / ls.na;
        const long base = a * ls.fa + b * ls.fb;
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
            if (!(fabs(ex.ka[a]) < ex.cut_a && fabs(ex.kb[p]) < ex.cut_b)) v = make_double2(0.0, 0.0);
        } else if (KIND == FK_PLAIN && ex.mul != MUL_NONE) {
            const double k = ex.km[ex.mul == MUL_IK_A ? a : p];
            v = make_double2(-k * v.y, k * v.x);
        }
        if (KIND == FK_PROJECT) {
            // f2d = dwdz + i (k1 uhat + k2 vhat), PadePoisson.F90:391-407
            const long idx = lg + p * ex.plane;
            const double k1 = ex.k1[lg % ex.nxh], k2 = ex.k2[lg / ex.nxh];
            const double2 uu = ex.u[idx], vv = ex.v[idx];
            const double tx = __dadd_rn(__dmul_rn(k1, uu.x), __dmul_rn(k2, vv.x));
            const double ty = __dadd_rn(__dmul_rn(k1, uu.y), __dmul_rn(k2, vv.y));
            v = make_double2(v.x - ty, v.y + tx);
        }
        sm[(l << logn) + brev(p, logn)] = v;
    }
    __syncthreads();

    if (KIND == FK_PLAIN) {
        dit(sm, nl, logn, tw, sign > 0);
    } else {
        dit(sm, nl, logn, tw, false);
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int l = e >> logn, p = e & (n - 1);
            const long lg = l0 + l;
            const long i = lg % ex.nxh, j = lg / ex.nxh;
            const double kr = KIND == FK_DEALIAS ? 0.0 : ksq(ex.ka[i], ex.kb[j], ex.kc[p]);
            double m;
            if (KIND == FK_PROJECT) {
                m = kr <= 1e-14 ? 0.0 : -(1.0 / kr);
            } else if (KIND == FK_DEALIAS) {
                m = (fabs(ex.ka[i]) < ex.cut_a && fabs(ex.kb[j]) < ex.cut_b && fabs(ex.kc[p]) < ex.cut_c) ? 1.0 : 0.0;
            } else {
                m = -1.0 / __dadd_rn(kr, 1e-20);
                if (lg == 0 && p == 0) m = 0.0;
            }
            const double2 v = sm[e];
            sm[e] = make_double2(v.x * m, v.y * m);
        }
        __syncthreads();
        dif(sm, nl, logn, tw, true);
    }

    const int nout = OUT == OUT_HALF ? half + 1 : n;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int l = pout ? (e >> logn) : (e % nl);
        const int p = pout ? (e & (n - 1)) : (e / nl);
        if (p >= nout) continue;
        const long lg = l0 + l, a = lg % ls.na, b = lg / ls.na;
        const long o = a * ls.oa + b * ls.ob + p * ls.op;
        double2 v = sm[(l << logn) + (KIND == FK_PLAIN ? p : brev(p, logn))];
        v = make_double2(v.x * scale, v.y * scale);
        if (OUT == OUT_REAL) {
            reinterpret_cast<double*>(out)[o] = v.x;
        } else {
            reinterpret_cast<double2*>(out)[o] = v;
        }
        if (KIND == FK_DEALIAS && ex.edge_copy && p == 0) reinterpret_cast<double2*>(out)[o + (long)n * ls.op] = v;
        if (KIND == FK_PROJECT) {
            // uhat -= i k1 p ; vhat -= i k2 p  (PadePoisson.F90:422-430)
            const long idx = lg + p * ex.plane;
            const double k1 = ex.k1[lg % ex.nxh], k2 = ex.k2[lg / ex.nxh];
            double2 uu = ex.u[idx], vv = ex.v[idx];
            uu = make_double2(uu.x + k1 * v.y, uu.y - k1 * v.x);
            vv = make_double2(vv.x + k2 * v.y, vv.y - k2 * v.x);
            ex.u[idx] = uu;
            ex.v[idx] = vv;
        }
    }
}

std::atomic<int> g_arith{FFT_ARITH_DF};

std::mutex g_tw_mu;
std::map<std::pair<int, int>, double2*> g_tw;  // (device, n) -> exp(-2 pi i t / n), t < n/2

int twiddles(int n, const double2** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PS_ECUDA;
    std::lock_guard<std::mutex> lock(g_tw_mu);
    auto it = g_tw.find({dev, n});
    if (it != g_tw.end()) {
        *out = it->second;
        return PS_OK;
    }
    std::vector<double2> h(std::max(1, n / 2));
    for (int t = 0; t < n / 2; t++) {
        const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
        h[t] = make_double2((double)cosl(ang), (double)sinl(ang));
    }
    double2* d = nullptr;
    if (cudaMalloc(&d, sizeof(double2) * h.size()) != cudaSuccess) {
        cudaGetLastError();
        return PS_ENOMEM;
    }
    if (cudaMemcpy(d, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return PS_ECUDA;
    }
    g_tw[{dev, n}] = d;
    *out = d;
    return PS_OK;
}

int log2_exact(int n) {
    int l = 0;
    while ((1 << l) < n && l < 30) l++;
    return (1 << l) == n ? l : -1;
}

template <int I, int O, int K>
int launch_t(const void* in, void* out, const FftLines& ls, const double2* tw, int logn, int lb, int sign,
             double scale, int oddball, const FftExtra& ex, cudaStream_t s) {
    const size_t smem = sizeof(double2) * ((size_t)lb << logn);
    auto kern = k_fft<I, O, K>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PS_ECUDA;
    const long blocks = (ls.nlines + lb - 1) / lb;
    if (blocks > 0x7fffffffL) return PS_ENOTSUP;
    kern<<<(unsigned)blocks, 256, smem, s>>>(in, out, ls, tw, logn, lb, sign, scale, oddball, ex);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

}  // namespace

FftLines fft_lines(int dir, long n1, long n2, long n3, long in_len, long out_len) {
    FftLines s{};
    if (dir == 1) {
        s.nlines = n2 * n3; s.na = s.nlines;
        s.fa = in_len; s.fb = 0; s.fp = 1;
        s.oa = out_len; s.ob = 0; s.op = 1;
    } else if (dir == 2) {
        s.nlines = n1 * n3; s.na = n1;
        s.fa = 1; s.fb = n1 * in_len; s.fp = n1;
        s.oa = 1; s.ob = n1 * out_len; s.op = n1;
    } else {
        s.nlines = n1 * n2; s.na = s.nlines;
        s.fa = 1; s.fb = 0; s.fp = n1 * n2;
        s.oa = 1; s.ob = 0; s.op = n1 * n2;
    }
    return s;
}

int fft_c2r_pair(const void* in, const void* in2, double* out1, double* out2, const FftLines& ls, int n, double scale,
                 const double* km, cudaStream_t s) {
    if (g_arith.load() != FFT_ARITH_DF) return PS_ENOTSUP;
    return fft_c2r_pair_df(in, in2, out1, out2, ls, n, scale, km, s);
}

int fft_r2c_pair(const double* in1, const double* in2, void* out1, void* out2, const FftLines& ls, int n,
                 double scale, cudaStream_t s) {
    if (g_arith.load() != FFT_ARITH_DF) return PS_ENOTSUP;
    return fft_r2c_pair_df(in1, in2, out1, out2, ls, n, scale, s);
}

void fft_set_arith(int a) { g_arith.store(a == FFT_ARITH_FP64 ? FFT_ARITH_FP64 : FFT_ARITH_DF); }
int fft_get_arith() { return g_arith.load(); }

int fft_launch(int in_mode, int out_mode, int kind, int n, int sign, double scale, int oddball, const void* in,
               void* out, const FftLines& ls, const FftExtra& ex, cudaStream_t s) {
    const int logn = log2_exact(n);
    if (logn < 1 || logn > 13) return PS_ENOTSUP;
    if (ls.nlines <= 0) return PS_OK;
    // a multiplier on load is defined for complex lines; on half-spectrum lines only i k(p)
    // (MUL_IK_P, applied to the stored half and extended Hermitian), in the double-float path
    if (ex.mul != MUL_NONE && in_mode != IN_COMPLEX &&
        !(in_mode == IN_HALF && ex.mul == MUL_IK_P && g_arith.load() == FFT_ARITH_DF))
        return PS_ENOTSUP;
    if (g_arith.load() == FFT_ARITH_DF)
        return fft_launch_df(in_mode, out_mode, kind, logn, sign, scale, oddball, in, out, ls, ex, s);
    const double2* tw = nullptr;
    const int rc = twiddles(n, &tw);
    if (rc != PS_OK) return rc;
    const int lb = std::max(1, std::min(64, 4096 >> logn));
    if (kind == FK_PROJECT)
        return launch_t<IN_COMPLEX, OUT_COMPLEX, FK_PROJECT>(in, out, ls, tw, logn, lb, sign, scale, 0, ex, s);
    if (kind == FK_POISSON3D)
        return launch_t<IN_COMPLEX, OUT_COMPLEX, FK_POISSON3D>(in, out, ls, tw, logn, lb, sign, scale, 0, ex, s);
    if (kind == FK_DEALIAS)
        return launch_t<IN_COMPLEX, OUT_COMPLEX, FK_DEALIAS>(in, out, ls, tw, logn, lb, sign, scale, 0, ex, s);
    if (in_mode == IN_COMPLEX && out_mode == OUT_COMPLEX)
        return launch_t<IN_COMPLEX, OUT_COMPLEX, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, scale, 0, ex, s);
    if (in_mode == IN_REAL && out_mode == OUT_HALF)
        return launch_t<IN_REAL, OUT_HALF, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, scale, 0, ex, s);
    if (in_mode == IN_HALF && out_mode == OUT_REAL)
        return launch_t<IN_HALF, OUT_REAL, FK_PLAIN>(in, out, ls, tw, logn, lb, sign, scale, oddball, ex, s);
    return PS_EINVAL;
}

}  // namespace pade
