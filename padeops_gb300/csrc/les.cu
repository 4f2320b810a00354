// LES time step of the incompressible solver (igrid), periodic in z, on one GPU.
//
// Restates src/incompressible/igrid.F90 for the configuration PeriodicInZ, Fourier x/y,
// staggered CD06 z (Pade6stagg periodic), rotational advection, TVD-RK3, molecular
// viscosity 1/Re, and the Smagorinsky model with the standard (planar-averaged) dynamic
// procedure; no stratification, Coriolis, forcing, turbines, fringe or wall model:
//   TVD_RK3            igrid.F90:1105-1174     compute_deltaT        1374-1403
//   populate_rhs       1793-1912               addNonLinearTerm_Rot  1497-1570
//   addViscousTerm     1914-1959               project_and_prep      1961-1991
//   dealiasFields      1020-1037               interp_PrimitiveVars  1423-1463
//   compute_duidxj     2553-2684               init sequence         625-648
//   getTauSGS/getRHS_SGS            sgsmod_igrid.F90:157-265
//   Smagorinsky kernel, Sij, nu interpolation   smagorinsky.F90, eddyViscosity.F90
//   DoStandardDynamicProcedure      standardDynamicProcedure.F90:74-244
// The slip-wall BC codes of the periodic configuration select d2dz2_C2C for the viscous
// z term of u and v (igrid.F90:2651-2658).  The test filter is spectral%InitTestFilter's
// x-y sharp cutoff at (2/3)(pi/dx)/deltaRatio (spectral.F90:1333-1367); the reference
// itself stops there for periodic-z problems (GracefulExit 1233).
//
// Every step is a fixed sequence of kernels on one stream with the time step held in
// device memory, so steps without a divergence check (which reads a maximum on the host)
// can be replayed from a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "dfmath.cuh"
#include "fft.h"
#include "operators.h"
#include "spectral_internal.h"

using namespace pade;

namespace {

enum { OP_DDZ_E2C = 0, OP_DDZ_C2E = 1, OP_D2_C2C = 4, OP_D2_E2E = 5, OP_I_E2C = 6, OP_I_C2E = 7 };

#define GRID_STRIDE(e, n) \
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (n); e += (long)gridDim.x * blockDim.x)

// non-contracting FP64 arithmetic: the reference evaluates each product and sum separately
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// Sij from duidxj (eddyViscosity.F90:1-21); d holds 9 arrays at stride n
__device__ __forceinline__ double sij(const double* const* d, int idx, long e) {
    switch (idx) {
        case 0: return d[0][e];
        case 1: return 0.5 * add(d[1][e], d[3][e]);
        case 2: return 0.5 * add(d[2][e], d[6][e]);
        case 3: return d[4][e];
        case 4: return 0.5 * add(d[5][e], d[7][e]);
        default: return d[8][e];
    }
}

struct Ptr9 {
    const double* p[9];
};

// ---- double-float forms of the pointwise kernels whose FP64 work exceeds their HBM traffic
// (|S|, the Germano products, the RK and RHS updates).  GB300 issues FP64 at about 2 lanes
// per SM cycle, so these ran at the FP64 rate; here each FP64 input is split into a df value
// with integer instructions (48 significant bits; magnitudes below 2^-74 count as zero, far
// below any field of the step), the arithmetic runs on the FP32 pipes and each result is
// rounded once to FP64 (one FP64 add).  The results agree with the FP64 operation order to
// ~1e-14 relative.
__device__ __forceinline__ dfv dsp(double x) {
    unsigned b = 0;
    return df_from_double(x, b);
}
__device__ __forceinline__ double dfo(dfv a) { return df_to_double(df_norm(a)); }
__device__ __forceinline__ dfv dmul(dfv a, dfv b) { return df_norm(df_mul(a, b)); }
__device__ __forceinline__ dfv dscale(dfv a, float p2) { return dfv{a.h * p2, a.l * p2}; }  // p2 a power of two
// an FP64 constant as df (its leading 48 bits)
__device__ __forceinline__ dfv dconst(double c) { return dsp(c); }

// sqrt of a non-negative df value: the FP32 root refined by one Newton (Heron) step with an
// exact residual (TwoProduct by FMA): relative error ~2^-47
__device__ __forceinline__ dfv df_sqrt(dfv x) {
    if (!(x.h > 0.0f)) return df_zero();
    const float r = __fsqrt_rn(x.h);
    const float p = __fmul_rn(r, r);
    const float e = __fmaf_rn(r, r, -p);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(x.h, p), e), x.l);
    const float c = __fdiv_rn(d, __fadd_rn(r, r));
    return df_norm(dfv{r, c});
}

// sqrt(2 Sij Sij) of six Sij values (df), smagorinsky.F90:39-67
__device__ __forceinline__ dfv df_smag(dfv s1, dfv s2, dfv s3, dfv s4, dfv s5, dfv s6) {
    dfv s = df_mul(s1, s1);
    s = df_add(s, dscale(df_mul(s2, s2), 2.0f));
    s = df_add(s, dscale(df_mul(s3, s3), 2.0f));
    s = df_add(s, df_mul(s4, s4));
    s = df_add(s, dscale(df_mul(s5, s5), 2.0f));
    s = df_add(s, df_mul(s6, s6));
    return df_sqrt(dscale(df_norm(s), 2.0f));
}

// ---- addNonLinearTerm_Rot products (igrid.F90:1530-1557)
__global__ void k_nl_c(Ptr9 dC, const double* __restrict__ u, const double* __restrict__ v, double* __restrict__ a,
                       double* __restrict__ b, long n) {
    GRID_STRIDE(e, n) {
        const double dudy = dC.p[1][e], dvdx = dC.p[3][e];
        a[e] = mul(sub(dvdx, dudy), v[e]);
        b[e] = mul(sub(dudy, dvdx), u[e]);
    }
}

__global__ void k_nl_e(Ptr9 dE, const double* __restrict__ w, const double* __restrict__ uE,
                       const double* __restrict__ vE, double* __restrict__ a, double* __restrict__ b,
                       double* __restrict__ c, long n) {
    GRID_STRIDE(e, n) {
        const double dudz = dE.p[2][e], dvdz = dE.p[5][e], dwdx = dE.p[6][e], dwdy = dE.p[7][e];
        a[e] = mul(sub(dwdx, dudz), w[e]);
        b[e] = mul(sub(dwdy, dvdz), w[e]);
        c[e] = add(mul(sub(dudz, dwdx), uE[e]), mul(sub(dvdz, dwdy), vE[e]));
    }
}

// rhs = rhs + f1  [+ (1/Re)(-kabs_sq fhat + d2)]  (igrid.F90:1537-1538, 1924-1930), double-float
__global__ void k_rhs_finish(double2* __restrict__ rhs, const double2* __restrict__ f1,
                             const double2* __restrict__ fhat, const double2* __restrict__ d2,
                             const double* __restrict__ k1, const double* __restrict__ k2, long nxh, long nxy,
                             double oneByRe, int viscous, long n) {
    const dfv re = dconst(oneByRe);
    GRID_STRIDE(e, n) {
        const double2 r0 = rhs[e];
        dfv rx = dsp(r0.x), ry = dsp(r0.y);
        if (f1) {
            const double2 a = f1[e];
            rx = df_add(rx, dsp(a.x));
            ry = df_add(ry, dsp(a.y));
        }
        if (viscous) {
            const long q = e % nxy;
            const dfv ka = dsp(k1[q % nxh]), kb = dsp(k2[q / nxh]);
            const dfv ks = df_norm(df_add(df_mul(ka, ka), df_mul(kb, kb)));
            const double2 fh = fhat[e], dd = d2[e];
            const dfv tx = df_norm(df_sub(dsp(dd.x), df_mul(ks, dsp(fh.x))));
            const dfv ty = df_norm(df_sub(dsp(dd.y), df_mul(ks, dsp(fh.y))));
            rx = df_add(df_norm(rx), df_mul(re, tx));
            ry = df_add(df_norm(ry), df_mul(re, ty));
        }
        rhs[e] = make_double2(dfo(rx), dfo(ry));
    }
}

// |S| at cell centres (get_smagorinsky_kernel) in double-float; optional copy for the
// dynamic procedure
__global__ void k_nu_kernel(Ptr9 dC, double* __restrict__ nu, double* __restrict__ dsgs, long n) {
    GRID_STRIDE(e, n) {
        const dfv g0 = dsp(dC.p[0][e]), g4 = dsp(dC.p[4][e]), g8 = dsp(dC.p[8][e]);
        // Sij off-diagonal = 0.5 (a + b): 2 Sij^2 = 0.5 (a + b)^2
        const dfv a = df_add(dsp(dC.p[1][e]), dsp(dC.p[3][e]));
        const dfv b = df_add(dsp(dC.p[2][e]), dsp(dC.p[6][e]));
        const dfv c = df_add(dsp(dC.p[5][e]), dsp(dC.p[7][e]));
        dfv s = df_mul(g0, g0);
        s = df_add(s, dscale(df_mul(a, a), 0.5f));
        s = df_add(s, dscale(df_mul(b, b), 0.5f));
        s = df_add(s, df_mul(g4, g4));
        s = df_add(s, dscale(df_mul(c, c), 0.5f));
        s = df_add(s, df_mul(g8, g8));
        const double v = dfo(df_sqrt(dscale(df_norm(s), 2.0f)));
        nu[e] = v;
        if (dsgs) dsgs[e] = v;
    }
}

// sigma model kernel (sigma.F90:30-95): singular values of the velocity gradient from the
// invariants of G = g^T g; FP64 in the reference's operation order
__global__ void k_sigma_kernel(Ptr9 d, double* __restrict__ nu, long n) {
    GRID_STRIDE(e, n) {
        const double d1 = d.p[0][e], d2 = d.p[1][e], d3 = d.p[2][e], d4 = d.p[3][e], d5 = d.p[4][e],
                     d6 = d.p[5][e], d7 = d.p[6][e], d8 = d.p[7][e], d9 = d.p[8][e];
        const double G11 = add(add(mul(d1, d1), mul(d4, d4)), mul(d7, d7));
        const double G12 = add(add(mul(d1, d2), mul(d4, d5)), mul(d7, d8));
        const double G13 = add(add(mul(d1, d3), mul(d4, d6)), mul(d7, d9));
        const double G22 = add(add(mul(d2, d2), mul(d5, d5)), mul(d8, d8));
        const double G23 = add(add(mul(d2, d3), mul(d5, d6)), mul(d8, d9));
        const double G33 = add(add(mul(d3, d3), mul(d6, d6)), mul(d9, d9));
        const double I1 = add(add(G11, G22), G33);
        const double I1sq = mul(I1, I1), I1cu = mul(I1sq, I1);
        double I2 = sub(sub(-mul(G11, G11), mul(G22, G22)), mul(G33, G33));
        I2 = sub(sub(I2, mul(mul(2.0, G12), G12)), mul(mul(2.0, G13), G13));
        I2 = sub(I2, mul(mul(2.0, G23), G23));
        I2 = add(I2, I1sq);
        I2 = mul(0.5, I2);
        double I3 = mul(G11, sub(mul(G22, G33), mul(G23, G23)));
        I3 = add(I3, mul(G12, sub(mul(G13, G23), mul(G12, G33))));
        I3 = add(I3, mul(G13, sub(mul(G12, G23), mul(G22, G13))));
        double a1 = sub(I1sq / 9.0, I2 / 3.0);
        a1 = fmax(a1, 0.0);
        const double a2 = add(sub(I1cu / 27.0, mul(I1, I2) / 6.0), I3 / 2.0);
        const double a1s = sqrt(a1);
        double t = mul(a1, a1s);
        t = a2 / add(t, 1e-13);
        t = fmin(t, 1.0);
        t = fmax(t, -1.0);
        t = acos(t);
        const double a3 = mul(1.0 / 3.0, t);
        const double third = I1 / 3.0;
        double s1sq = add(third, mul(mul(2.0, a1s), cos(a3)));
        s1sq = fmax(s1sq, 0.0);
        const double s1 = sqrt(s1sq);
        const double pi3 = 3.14159265358979323846 / 3.0;
        double s2 = mul(mul(-2.0, a1s), cos(add(pi3, a3)));
        s2 = sqrt(fmax(add(s2, third), 0.0));
        double s3 = mul(mul(-2.0, a1s), cos(sub(pi3, a3)));
        s3 = sqrt(fmax(add(s3, third), 0.0));
        nu[e] = mul(mul(s3, sub(s1, s2)), sub(s2, s3)) / add(s1sq, 1e-15);
    }
}

// AMD model kernel (AMD.F90:23-72), with S_ij from the same gradients
__global__ void k_amd_kernel(Ptr9 d, double cx, double cy, double cz, double* __restrict__ nu, long n) {
    GRID_STRIDE(e, n) {
        double g[9];
#pragma unroll
        for (int i = 0; i < 9; i++) g[i] = d.p[i][e];
        const double S[6] = {sij(d.p, 0, e), sij(d.p, 1, e), sij(d.p, 2, e),
                             sij(d.p, 3, e), sij(d.p, 4, e), sij(d.p, 5, e)};
        // row r of the scaled gradient: (g[3r] cx, g[3r+1] cy, g[3r+2] cz)
        auto dot = [&](int r, int q) {
            return add(add(mul(mul(g[3 * r], cx), mul(g[3 * q], cx)), mul(mul(g[3 * r + 1], cy), mul(g[3 * q + 1], cy))),
                       mul(mul(g[3 * r + 2], cz), mul(g[3 * q + 2], cz)));
        };
        double num = mul(dot(0, 0), S[0]);
        num = add(num, mul(dot(1, 1), S[3]));
        num = add(num, mul(dot(2, 2), S[5]));
        num = add(num, mul(mul(2.0, dot(0, 1)), S[1]));
        num = add(num, mul(mul(2.0, dot(0, 2)), S[2]));
        num = add(num, mul(mul(2.0, dot(1, 2)), S[4]));
        double den = mul(g[0], g[0]);
#pragma unroll
        for (int i = 1; i < 9; i++) den = add(den, mul(g[i], g[i]));
        nu[e] = fmax(-num / add(den, 1e-32), 0.0);
    }
}

// |S| of six arrays
__global__ void k_smag6(const double* s0, const double* s1, const double* s2, const double* s3, const double* s4,
                        const double* s5, double* __restrict__ out, long n) {
    GRID_STRIDE(e, n) {
        out[e] = dfo(df_smag(dsp(s0[e]), dsp(s1[e]), dsp(s2[e]), dsp(s3[e]), dsp(s4[e]), dsp(s5[e])));
    }
}

// out = [scale *] Sij(idx)
__global__ void k_sij(Ptr9 d, int idx, const double* __restrict__ scale, double* __restrict__ out, long n) {
    GRID_STRIDE(e, n) {
        const double s = sij(d.p, idx, e);
        out[e] = scale ? mul(scale[e], s) : s;
    }
}

// M = filt - dr2 * Df * Sf  (standardDynamicProcedure.F90:102-106)
__global__ void k_mij(const double* __restrict__ filt, const double* __restrict__ df, const double* __restrict__ sf,
                      double dr2, double* __restrict__ m, long n) {
    GRID_STRIDE(e, n) { m[e] = sub(filt[e], mul(mul(dr2, df[e]), sf[e])); }
}

__global__ void k_prod(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out, long n) {
    GRID_STRIDE(e, n) { out[e] = mul(a[e], b[e]); }
}

// L = filt - a * b  (standardDynamicProcedure.F90:112-136)
__global__ void k_lij(const double* __restrict__ filt, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ l, long n) {
    GRID_STRIDE(e, n) { l[e] = sub(filt[e], mul(a[e], b[e])); }
}

struct Ptr6 {
    const double* p[6];
};

// scalar dynamic procedure (standardDynamicProcedure.F90:57-63): num = R . P, den = R . R
__global__ void k_num_den3(const double* __restrict__ r0, const double* __restrict__ r1,
                           const double* __restrict__ r2, const double* __restrict__ p0,
                           const double* __restrict__ p1, const double* __restrict__ p2, double* __restrict__ num,
                           double* __restrict__ den, long n) {
    GRID_STRIDE(e, n) {
        const double a = r0[e], b = r1[e], c = r2[e];
        num[e] = add(add(mul(a, p0[e]), mul(b, p1[e])), mul(c, p2[e]));
        den[e] = add(add(mul(a, a), mul(b, b)), mul(c, c));
    }
}

// kappa = beta(z) Dsgs (beta per z plane) or nu / Pr (getQjSGS, sgsmod_igrid.F90:318-326)
__global__ void k_kappa(const double* __restrict__ a, const double* __restrict__ beta, double pr_inv, long plane,
                        double* __restrict__ kappa, long n) {
    GRID_STRIDE(e, n) { kappa[e] = beta ? mul(a[e], beta[e / plane]) : mul(a[e], pr_inv); }
}

// q = -kappa dT  (sgsmod_igrid.F90:330-332)
__global__ void k_negmul(const double* __restrict__ kappa, const double* __restrict__ g, double* __restrict__ q,
                         long n) {
    GRID_STRIDE(e, n) { q[e] = -mul(kappa[e], g[e]); }
}

// numerator / denominator of the Germano identity (standardDynamicProcedure.F90:139-154) in
// double-float: Lij Mij and Mij Mij with the off-diagonal products (1, 2, 4) counted twice
__global__ void k_num_den(Ptr6 L, Ptr6 M, double* __restrict__ num, double* __restrict__ den, long n) {
    GRID_STRIDE(e, n) {
        dfv a = df_zero(), b = df_zero();
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const dfv m = dsp(M.p[i][e]);
            dfv lm = df_mul(dsp(L.p[i][e]), m), mm = df_mul(m, m);
            if (i == 1 || i == 2 || i == 4) {
                lm = dscale(lm, 2.0f);
                mm = dscale(mm, 2.0f);
            }
            a = df_add(a, lm);
            b = df_add(b, mm);
        }
        num[e] = dfo(a);
        den[e] = dfo(dscale(df_norm(b), 2.0f));
    }
}

// per-plane sums of two arrays (b == nullptr: of a and of ones): grid (chunks, nz);
// partials [nz][chunks][2]
constexpr int kPlaneChunks = 16;
__global__ void k_plane_sums(const double* __restrict__ a, const double* __restrict__ b, long plane,
                             double* __restrict__ part) {
    __shared__ double sa[8], sb[8];
    const int k = blockIdx.y;
    const double* pa = a + (long)k * plane;
    const double* pb = b + (long)k * plane;
    double x = 0.0, y = 0.0;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < plane; e += (long)gridDim.x * blockDim.x) {
        x += pa[e];
        y += b ? pb[e] : 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = x;
        sb[threadIdx.x >> 5] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tx = 0.0, ty = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            tx += sa[w];
            ty += sb[w];
        }
        part[((long)k * gridDim.x + blockIdx.x) * 2] = tx;
        part[((long)k * gridDim.x + blockIdx.x) * 2 + 1] = ty;
    }
}

// lambda(z) = max(<num> , 0) / (<den> + 1e-18)  (planarAverage_and_TakeRatio, 221-244)
__global__ void k_lambda(const double* __restrict__ part, int chunks, double meanfact, int nz,
                         double* __restrict__ lambda) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    double x = 0.0, y = 0.0;
    for (int c = 0; c < chunks; c++) {
        x += part[((long)k * chunks + c) * 2];
        y += part[((long)k * chunks + c) * 2 + 1];
    }
    const double nm = fmax(mul(x, meanfact), 0.0);
    lambda[k] = nm / add(mul(y, meanfact), 1e-18);
}

// the learned closure's judge: relative error of the closure's plane-averaged coefficient
// lamL against the dynamic procedure's lambda, and the switch that sends every point to the
// fallback while it exceeds tol (> 0)
// The judge: relative difference of the closure's plane-averaged coefficient lamL(z) and the
// dynamic procedure's lambda(z), max_z |lamL - lambda| / max(max_z |lambda|, max_z |lamL|)
// (0 when both vanish, 1 when only one does); above tol every point takes lambda(z) until
// the next judge step.
__global__ void k_judge(const double* __restrict__ lambda, const double* __restrict__ lamL, int nz, double tol,
                        double* __restrict__ err, int* __restrict__ all) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double dm = 0.0, lm = 0.0;
    for (int k = 0; k < nz; k++) {
        dm = fmax(dm, fabs(lamL[k] - lambda[k]));
        lm = fmax(lm, fmax(fabs(lambda[k]), fabs(lamL[k])));
    }
    const double e = lm > 0.0 ? dm / lm : 0.0;
    *err = e;
    *all = (tol > 0.0 && e > tol) ? 1 : 0;
}

// nu *= lambda(z) (dynamic) or cmodel_global
__global__ void k_scale_nu(double* __restrict__ nu, const double* __restrict__ lambda, double c, long plane,
                           long n) {
    GRID_STRIDE(e, n) { nu[e] = lambda ? mul(lambda[e / plane], nu[e]) : mul(c, nu[e]); }
}

// learned closure, plane-averaged form: a = Cs^2 Delta^2 from the closure's FP32 output
__global__ void k_cs2_delta2(const float* __restrict__ cs2, double d2, double* __restrict__ a, long n) {
    GRID_STRIDE(e, n) { a[e] = mul((double)cs2[e], d2); }
}

__global__ void k_clip_neg(double* __restrict__ x, long n) {
    GRID_STRIDE(e, n) {
        if (x[e] < 0.0) x[e] = 0.0;
    }
}

// tau = -2 nu Sij(idx)  (sgsmod_igrid.F90:188-193), in double-float like the kernels above:
// its two FP64 operations per value had kept it at 106 us per 256^3 launch against ~80 us
// of HBM traffic
__global__ void k_tau(Ptr9 d, int idx, const double* __restrict__ nu, double* __restrict__ out, long n) {
    // off-diagonal: 2 nu * (0.5 (a + b)) is nu * (a + b) exactly (power-of-two scalings)
    const int ia = idx == 1 ? 1 : (idx == 2 ? 2 : 5), ib = idx == 1 ? 3 : (idx == 2 ? 6 : 7);
    if (idx == 1 || idx == 2 || idx == 4) {
        GRID_STRIDE(e, n) {
            const dfv s = df_norm(df_add(dsp(d.p[ia][e]), dsp(d.p[ib][e])));
            out[e] = -dfo(df_mul(dsp(nu[e]), s));
        }
    } else {
        const int id = idx == 0 ? 0 : (idx == 3 ? 4 : 8);
        GRID_STRIDE(e, n) { out[e] = -dfo(df_mul(dscale(dsp(nu[e]), 2.0f), dsp(d.p[id][e]))); }
    }
}

// a -= i k(a) X ; b -= i k(b) X  (mtimes_ik then subtraction, sgsmod_igrid.F90:213-260);
// which: 1 = k1 (x index), 2 = k2 (y index)
__global__ void k_sub_ik(double2* __restrict__ a, int wa, double2* __restrict__ b, int wb,
                         const double2* __restrict__ X, const double* __restrict__ k1,
                         const double* __restrict__ k2, long nxh, long nxy, long n) {
    GRID_STRIDE(e, n) {
        const long q = e % nxy;
        const double2 x = X[e];
        if (a) {
            const double k = wa == 1 ? k1[q % nxh] : k2[q / nxh];
            const double2 r = a[e];
            a[e] = make_double2(sub(r.x, -mul(k, x.y)), sub(r.y, mul(k, x.x)));
        }
        if (b) {
            const double k = wb == 1 ? k1[q % nxh] : k2[q / nxh];
            const double2 r = b[e];
            b[e] = make_double2(sub(r.x, -mul(k, x.y)), sub(r.y, mul(k, x.x)));
        }
    }
}

__global__ void k_csub2(double2* __restrict__ y, const double2* __restrict__ x, long n) {
    GRID_STRIDE(e, n) {
        const double2 a = y[e], b = x[e];
        y[e] = make_double2(sub(a.x, b.x), sub(a.y, b.y));
    }
}

// TVD-RK3 stage updates (igrid.F90:1128-1164), double-float; dt read from device memory
__global__ void k_rk(int stage, double2* __restrict__ u0, double2* __restrict__ u1, const double2* __restrict__ r,
                     const double* __restrict__ dtp, long n) {
    const double dt = *dtp;
    // stage weights (1, 1), (3/4, 1/4), (1/3, 2/3) and the dt factor, in double-float
    const dfv c0 = dconst(stage == 2 ? 3.0 / 4.0 : 1.0 / 3.0), c1 = dconst(stage == 2 ? 1.0 / 4.0 : 2.0 / 3.0);
    const dfv c2 = dmul(dconst(stage == 1 ? 1.0 : (stage == 2 ? 1.0 / 4.0 : 2.0 / 3.0)), dsp(dt));
    GRID_STRIDE(e, n) {
        const double2 a = u0[e], rr = r[e];
        const dfv ax = dsp(a.x), ay = dsp(a.y);
        if (stage == 1) {
            u1[e] = make_double2(dfo(df_add(ax, df_mul(c2, dsp(rr.x)))), dfo(df_add(ay, df_mul(c2, dsp(rr.y)))));
        } else {
            const double2 b = u1[e];
            const dfv tx = df_add(df_norm(df_add(df_mul(c0, ax), df_mul(c1, dsp(b.x)))), df_mul(c2, dsp(rr.x)));
            const dfv ty = df_add(df_norm(df_add(df_mul(c0, ay), df_mul(c1, dsp(b.y)))), df_mul(c2, dsp(rr.y)));
            const double2 o = make_double2(dfo(tx), dfo(ty));
            if (stage == 2) u1[e] = o;
            else u0[e] = o;
        }
    }
}

// CFL time-step partials: max(|u/dx| + |v/dy| + |wC/dz|)  (igrid.F90:1384-1393)
__global__ void k_cfl_partial(const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, double rdx, double rdy, double rdz, long n,
                              double* __restrict__ part) {
    __shared__ double s[8];
    double m = 0.0;
    GRID_STRIDE(e, n) {
        double a = fabs(mul(rdx, u[e]));
        a = add(a, fabs(mul(rdy, v[e])));
        a = add(a, fabs(mul(rdz, w[e])));
        m = fmax(m, a);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t = fmax(t, s[i]);
        part[blockIdx.x] = t;
    }
}

__global__ void k_cfl_final(const double* __restrict__ part, int np, double cfl, double tvisc, int viscous,
                            double* __restrict__ dt) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = 0.0;
    for (int i = 0; i < np; i++) m = fmax(m, part[i]);
    double d = cfl / m;
    if (viscous) d = fmin(d, tvisc);
    *dt = d;
}

__global__ void k_set(double* __restrict__ p, double v) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *p = v;
}

// wrapup_timestep: tsim = tsim + dt (igrid.F90:2074)
__global__ void k_advance(double* __restrict__ tsim, const double* __restrict__ dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *tsim = *tsim + *dt;
}

constexpr int kCflBlocks = 152 * 4;

}  // namespace

struct pade_les_s {
    pade_les_params prm{};
    int nx = 0, ny = 0, nz = 0, nxh = 0;
    double dx = 0, dy = 0, dz = 0;
    long NC = 0, NE = 0, SC = 0, SE = 0, plane = 0, splane = 0;
    pade_spectral spC = nullptr, spE = nullptr;
    pade_poisson po = nullptr;
    pade_op stagg = nullptr;
    double* d_k3 = nullptr;  // spectral k3 (oddball sign flipped) for the dealias mask
    double cut_x = 0, cut_y = 0, cut_z = 0, tf_x = 0, tf_y = 0;
    double cmodel_global = 0, meanfact = 0, tvisc = 0;
    double camd_x = 0, camd_y = 0, camd_z = 0;
    // spectral state and stage copies
    double2 *uhat = nullptr, *vhat = nullptr, *what = nullptr;
    double2 *uhat1 = nullptr, *vhat1 = nullptr, *what1 = nullptr;
    double2 *urhs = nullptr, *vrhs = nullptr, *wrhs = nullptr;
    double2 *whatC = nullptr, *uEhat = nullptr, *vEhat = nullptr;
    double2 *d2u = nullptr, *d2v = nullptr, *d2w = nullptr;
    double2 *tC1 = nullptr, *tE1 = nullptr;
    // second stream of the RHS and its scratch (the v / w chains and every other tau chain)
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double2 *tC1b = nullptr, *tE1b = nullptr;
    double *rC1b = nullptr, *rE1b = nullptr;
    double2 *uhat_cur = nullptr, *vhat_cur = nullptr, *what_cur = nullptr;  // fields project_and_prep acts on
    // physical fields
    double *u = nullptr, *v = nullptr, *wC = nullptr, *w = nullptr, *uE = nullptr, *vE = nullptr;
    double* dC[9] = {nullptr};
    double* dE[9] = {nullptr};
    double *rC1 = nullptr, *rC2 = nullptr, *rE1 = nullptr, *rE2 = nullptr, *rE3 = nullptr;
    double *nuC = nullptr, *nuE = nullptr, *div = nullptr;
    // dynamic procedure
    double *Sf[6] = {nullptr}, *M[6] = {nullptr}, *Lm[6] = {nullptr}, *uf[3] = {nullptr};
    double *Df = nullptr, *Dsgs = nullptr, *lambda = nullptr, *part = nullptr, *lamL = nullptr;
    double* betaT = nullptr;  // the scalar dynamic procedure's Beta(z) (pade_les_scalar_sgs)
    double *d_dt = nullptr, *d_tsim = nullptr, *cflpart = nullptr;
    std::vector<void*> allocs;
    int step = 0, mstep = 0;
    bool newTimeStep = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;
    pade_mlp mlp = nullptr;
    double deltaLES = 0;
    // learned closure: fallback switch, fallback count, judge error
    int* fball = nullptr;
    unsigned long long* fbcount = nullptr;
    double* judge_err = nullptr;
};

namespace {

int al(pade_les h, void* p, size_t bytes) {
    void** pp = static_cast<void**>(p);
    int rc = dalloc(pp, bytes);
    if (rc == PS_OK) h->allocs.push_back(*pp);
    return rc;
}

int zop(pade_les h, int op, int cplx, const void* in, void* out, cudaStream_t s) {
    return pade_apply(h->stagg, op, 3, cplx, in, out, cplx ? h->nxh : h->nx, h->ny, 0, 0, PADE_PATH_DF, s);
}

#define CK(x)                        \
    do {                             \
        const int rc_ = (x);         \
        if (rc_ != PS_OK) return rc_; \
    } while (0)
#define KCHECK() CK(cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA)

Ptr9 p9(double* const* a) {
    Ptr9 r;
    for (int i = 0; i < 9; i++) r.p[i] = a[i];
    return r;
}

// spectral test filter of a real C field (TestFilter_Real_to_Real): fft, cutoff, ifft
int test_filter(pade_les h, const double* in, double* out, cudaStream_t s) {
    CK(spectral_fft(h->spC, in, h->tC1, s));
    return spectral_ifft_masked(h->spC, h->tC1, out, h->tf_x, h->tf_y, s);
}

int dealias(pade_les h, double2* f, int edge, cudaStream_t s) {
    FftExtra ex{};
    ex.ka = h->spC->d_k1;
    ex.kb = h->spC->d_k2;
    ex.kc = h->d_k3;
    ex.nxh = h->nxh;
    ex.plane = h->splane;
    ex.cut_a = h->cut_x;
    ex.cut_b = h->cut_y;
    ex.cut_c = h->cut_z;
    ex.edge_copy = edge;
    FftLines lz = fft_lines(3, h->nxh, h->ny, h->nz, h->nz, h->nz);
    return fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_DEALIAS, h->nz, -1, 1.0 / (double)h->nz, 0, f, f, lz, ex, s);
}

// the y and z gradients (the x gradients come with the fields from prep_physical), two
// inverse transforms per call (their x passes paired in one launch); tC1b / tE1b are free here
int compute_duidxj(pade_les h, cudaStream_t s) {
    pade_spectral C = h->spC, E = h->spE;
    // d/dy of u and v
    CK(spectral_ifft_two(C, h->uhat_cur, MUL_IK_P, h->vhat_cur, MUL_IK_P, h->dC[1], h->dC[4], C->work, h->tC1b, s));
    CK(spectral_ifft_two(E, h->uEhat, MUL_IK_P, h->vEhat, MUL_IK_P, h->dE[1], h->dE[4], E->work, h->tE1b, s));
    // dw/dy with dw/dz (dw/dz at C, then at E; the scratch transforms in place)
    CK(zop(h, OP_DDZ_E2C, 1, h->what_cur, h->tC1, s));
    CK(zop(h, OP_I_C2E, 1, h->tC1, h->tE1, s));
    CK(spectral_ifft_two(C, h->whatC, MUL_IK_P, h->tC1, MUL_NONE, h->dC[7], h->dC[8], C->work, h->tC1, s));
    CK(spectral_ifft_two(E, h->what_cur, MUL_IK_P, h->tE1, MUL_NONE, h->dE[7], h->dE[8], E->work, h->tE1, s));
    if (!h->prm.isInviscid) CK(zop(h, OP_D2_E2E, 1, h->what_cur, h->d2w, s));
    // du/dz with dv/dz, at E and at C
    CK(zop(h, OP_DDZ_C2E, 1, h->uhat_cur, h->tE1, s));
    CK(zop(h, OP_DDZ_C2E, 1, h->vhat_cur, h->tE1b, s));
    if (!h->prm.isInviscid) {
        CK(zop(h, OP_D2_C2C, 1, h->uhat_cur, h->d2u, s));
        CK(zop(h, OP_D2_C2C, 1, h->vhat_cur, h->d2v, s));
    }
    CK(zop(h, OP_I_E2C, 1, h->tE1, h->tC1, s));
    CK(zop(h, OP_I_E2C, 1, h->tE1b, h->tC1b, s));
    CK(spectral_ifft_two(E, h->tE1, MUL_NONE, h->tE1b, MUL_NONE, h->dE[2], h->dE[5], h->tE1, h->tE1b, s));
    return spectral_ifft_two(C, h->tC1, MUL_NONE, h->tC1b, MUL_NONE, h->dC[2], h->dC[5], h->tC1, h->tC1b, s);
}

// physical fields and their x gradients (one y transform per pair), then the other gradients
int prep_physical(pade_les h, cudaStream_t s) {
    CK(spectral_ifft_pair(h->spC, h->uhat_cur, h->u, h->dC[0], s));
    CK(spectral_ifft_pair(h->spC, h->vhat_cur, h->v, h->dC[3], s));
    CK(spectral_ifft_pair(h->spE, h->what_cur, h->w, h->dE[6], s));
    CK(zop(h, OP_I_E2C, 1, h->what_cur, h->whatC, s));
    CK(spectral_ifft_pair(h->spC, h->whatC, h->wC, h->dC[6], s));
    CK(zop(h, OP_I_C2E, 1, h->uhat_cur, h->uEhat, s));
    CK(spectral_ifft_pair(h->spE, h->uEhat, h->uE, h->dE[0], s));
    CK(zop(h, OP_I_C2E, 1, h->vhat_cur, h->vEhat, s));
    CK(spectral_ifft_pair(h->spE, h->vEhat, h->vE, h->dE[3], s));
    return compute_duidxj(h, s);
}

int project_and_prep(pade_les h, cudaStream_t s) {
    CK(dealias(h, h->uhat_cur, 0, s));
    CK(dealias(h, h->vhat_cur, 0, s));
    CK(dealias(h, h->what_cur, 1, s));
    CK(pade_poisson_projection(h->po, h->uhat_cur, h->vhat_cur, h->what_cur, s));
    if (h->prm.t_DivergenceCheck > 0 && h->step % h->prm.t_DivergenceCheck == 0) {
        double m = 0;
        CK(pade_poisson_divergence_check(h->po, h->uhat_cur, h->vhat_cur, h->what_cur, h->div, 1, &m, s));
    }
    return prep_physical(h, s);
}

int dynamic_procedure(pade_les h, cudaStream_t s) {
    const long n = h->NC;
    const unsigned g = grid_for(n);
    const Ptr9 dC = p9(h->dC);
    for (int i = 0; i < 6; i++) {
        k_sij<<<g, 256, 0, s>>>(dC, i, nullptr, h->rC1, n);
        KCHECK();
        CK(test_filter(h, h->rC1, h->Sf[i], s));
    }
    k_smag6<<<g, 256, 0, s>>>(h->Sf[0], h->Sf[1], h->Sf[2], h->Sf[3], h->Sf[4], h->Sf[5], h->Df, n);
    KCHECK();
    const double dr2 = h->prm.deltaRatio * h->prm.deltaRatio;
    for (int i = 0; i < 6; i++) {
        k_sij<<<g, 256, 0, s>>>(dC, i, h->Dsgs, h->rC1, n);
        KCHECK();
        CK(test_filter(h, h->rC1, h->rC2, s));
        k_mij<<<g, 256, 0, s>>>(h->rC2, h->Df, h->Sf[i], dr2, h->M[i], n);
        KCHECK();
    }
    CK(spectral_ifft_masked(h->spC, h->uhat_cur, h->uf[0], h->tf_x, h->tf_y, s));
    CK(spectral_ifft_masked(h->spC, h->vhat_cur, h->uf[1], h->tf_x, h->tf_y, s));
    CK(spectral_ifft_masked(h->spC, h->whatC, h->uf[2], h->tf_x, h->tf_y, s));
    const double* U[3] = {h->u, h->v, h->wC};
    const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; q++) {
        k_prod<<<g, 256, 0, s>>>(U[pi[q]], U[pj[q]], h->rC1, n);
        KCHECK();
        CK(test_filter(h, h->rC1, h->rC2, s));
        k_lij<<<g, 256, 0, s>>>(h->rC2, h->uf[pi[q]], h->uf[pj[q]], h->Lm[q], n);
        KCHECK();
    }
    Ptr6 L, M;
    for (int i = 0; i < 6; i++) {
        L.p[i] = h->Lm[i];
        M.p[i] = h->M[i];
    }
    k_num_den<<<g, 256, 0, s>>>(L, M, h->rC1, h->rC2, n);
    KCHECK();
    dim3 grid(kPlaneChunks, h->nz);
    k_plane_sums<<<grid, 256, 0, s>>>(h->rC1, h->rC2, h->plane, h->part);
    KCHECK();
    k_lambda<<<(h->nz + 127) / 128, 128, 0, s>>>(h->part, kPlaneChunks, h->meanfact, h->nz, h->lambda);
    KCHECK();
    return PS_OK;
}

// b waits for the work enqueued so far on a (event slot e)
// the learned closure's fallback: the last judged lambda(z) (initially (Csgs Delta)^2), every
// point while the judge's switch is on
MlpFallback fallback(pade_les h) { return MlpFallback{h->lambda, h->plane, h->fball, h->fbcount}; }

int after(pade_les h, int e, cudaStream_t a, cudaStream_t b) {
    if (cudaEventRecord(h->ev[e], a) != cudaSuccess) return PS_ECUDA;
    return cudaStreamWaitEvent(b, h->ev[e], 0) == cudaSuccess ? PS_OK : PS_ECUDA;
}

// Whether the eddy viscosity is pointwise in the gradients and needs no scratch, so that it
// can run beside the nonlinear terms: every model but the plane-averaged learned one.
bool nu_pointwise(pade_les h) { return !(h->prm.learnedSGS && h->prm.learnedPlaneAvg); }

// nuC (and Dsgs, the dynamic procedure's |S|) of the pointwise models
int sgs_nu_pointwise(pade_les h, cudaStream_t s) {
    const long n = h->NC;
    const unsigned g = grid_for(n);
    const Ptr9 dC = p9(h->dC);
    if (h->prm.learnedSGS) {
        if (!h->mlp) return PS_EINVAL;
        const double* grads[9];
        for (int i = 0; i < 9; i++) grads[i] = h->dC[i];
        return mlp_infer_nu_fb(h->mlp, grads, n, h->deltaLES, 1.0 / h->prm.Re, h->nuC, nullptr, fallback(h), s);
    }
    const bool dyn = h->prm.dynamic != 0;
    if (h->prm.SGSModelID == 1) {
        k_sigma_kernel<<<g, 256, 0, s>>>(dC, h->nuC, n);
    } else if (h->prm.SGSModelID == 2) {
        k_amd_kernel<<<g, 256, 0, s>>>(dC, h->camd_x, h->camd_y, h->camd_z, h->nuC, n);
    } else {
        k_nu_kernel<<<g, 256, 0, s>>>(dC, h->nuC, (dyn && h->newTimeStep) ? h->Dsgs : nullptr, n);
    }
    KCHECK();
    return PS_OK;
}

// the closure's plane-averaged Cs^2 Delta^2 into lamL from Cs^2 (FP32) in cs2
int closure_plane_average(pade_les h, const float* cs2, cudaStream_t s) {
    const long n = h->NC;
    const unsigned g = grid_for(n);
    k_cs2_delta2<<<g, 256, 0, s>>>(cs2, h->deltaLES * h->deltaLES, h->rC2, n);
    KCHECK();
    dim3 grid(kPlaneChunks, h->nz);
    k_plane_sums<<<grid, 256, 0, s>>>(h->rC2, nullptr, h->plane, h->part);
    KCHECK();
    k_lambda<<<(h->nz + 127) / 128, 128, 0, s>>>(h->part, kPlaneChunks, h->meanfact, h->nz, h->lamL);
    KCHECK();
    return PS_OK;
}

// the rest of the eddy viscosity (dynamic procedure, plane averages, model constant) and
// its interpolation to the edges
int sgs_nu_rest(pade_les h, cudaStream_t s) {
    const long n = h->NC, nE = h->NE;
    const unsigned g = grid_for(n), gE = grid_for(nE);
    const Ptr9 dC = p9(h->dC);
    const bool learned = h->prm.learnedSGS != 0;
    const bool dyn = h->prm.dynamic != 0 && !learned;
    if (learned) {
        if (!h->mlp) return PS_EINVAL;
        const double* grads[9];
        for (int i = 0; i < 9; i++) grads[i] = h->dC[i];
        float* cs2 = reinterpret_cast<float*>(h->rC1);
        // the judge: the dynamic procedure's lambda(z) (then the fallback coefficient) against
        // the closure's plane average on the same fields (standardDynamicProcedure.F90:74-244)
        if (h->newTimeStep && h->prm.JudgeFreq > 0 && h->mstep % h->prm.JudgeFreq == 0) {
            k_nu_kernel<<<g, 256, 0, s>>>(dC, h->rC2, h->Dsgs, n);
            KCHECK();
            CK(dynamic_procedure(h, s));
            MlpFallback fb = fallback(h);
            fb.count = nullptr;  // the judge's own evaluation is not counted
            CK(mlp_infer_nu_fb(h->mlp, grads, n, h->deltaLES, 1.0 / h->prm.Re, h->rC2, cs2, fb, s));
            CK(closure_plane_average(h, cs2, s));
            k_judge<<<1, 32, 0, s>>>(h->lambda, h->lamL, h->nz, h->prm.JudgeTol, h->judge_err, h->fball);
            KCHECK();
        }
        if (h->prm.learnedPlaneAvg) {
            // nu = <Cs^2 Delta^2>_xy |S|: the closure's coefficient through the dynamic
            // procedure's plane average (Cs^2 as FP32 in the rC1 scratch)
            CK(mlp_infer_nu_fb(h->mlp, grads, n, h->deltaLES, 1.0 / h->prm.Re, h->nuC, cs2, fallback(h), s));
            CK(closure_plane_average(h, cs2, s));
            k_nu_kernel<<<g, 256, 0, s>>>(dC, h->nuC, nullptr, n);
            KCHECK();
            k_scale_nu<<<g, 256, 0, s>>>(h->nuC, h->lamL, 0.0, h->plane, n);
            KCHECK();
        }
    } else {
        if (dyn && h->newTimeStep && h->mstep % std::max(1, h->prm.DynProcFreq) == 0) CK(dynamic_procedure(h, s));
        k_scale_nu<<<g, 256, 0, s>>>(h->nuC, dyn ? h->lambda : nullptr, h->cmodel_global, h->plane, n);
        KCHECK();
    }
    CK(zop(h, OP_I_C2E, 0, h->nuC, h->nuE, s));
    if (!dyn) {
        k_clip_neg<<<gE, 256, 0, s>>>(h->nuE, nE);
        KCHECK();
    }
    if (h->newTimeStep) h->mstep++;
    return PS_OK;
}

// The divergence of tau into the right-hand sides: six chains (tau component, its x-y
// transform, the z operator where one applies, then the subtraction from the RHS).  Chains
// alternate between two streams with their own scratch, so one chain's FP64-bound tau and
// subtraction kernels run beside the other's transforms; the subtractions keep the
// sequential order (each waits for the previous one), so the sums are those of one stream.
int sgs_tau_rhs(pade_les h, cudaStream_t s) {
    const long n = h->NC, nE = h->NE;
    const unsigned g = grid_for(n), gE = grid_for(nE), gs = grid_for(h->SC), gsE = grid_for(h->SE);
    const Ptr9 dC = p9(h->dC), dE = p9(h->dE);
    const double* k1 = h->spC->d_k1;
    const double* k2 = h->spC->d_k2;
    const long nxh = h->nxh, nxy = h->splane;
    struct Scr {
        double *rC, *rE;
        double2 *tC, *tE;
        cudaStream_t st;
    };
    const Scr A{h->rC1, h->rE1, h->tC1, h->tE1, s}, B{h->rC1b, h->rE1b, h->tC1b, h->tE1b, h->s2};
    CK(after(h, 0, s, h->s2));  // nuC / nuE are ready
    for (int c = 0; c < 6; c++) {
        const Scr& X = (c % 2 == 0) ? A : B;
        const cudaStream_t t = X.st;
        // tau component, transform, z operator
        if (c < 4) {
            static const int idx[4] = {0, 3, 5, 1};  // tau11, tau22, tau33, tau12
            k_tau<<<g, 256, 0, t>>>(dC, idx[c], h->nuC, X.rC, n);
            KCHECK();
            CK(spectral_fft(h->spC, X.rC, X.tC, t));
            if (c == 2) CK(zop(h, OP_DDZ_C2E, 1, X.tC, X.tE, t));
        } else {
            k_tau<<<gE, 256, 0, t>>>(dE, c == 4 ? 2 : 4, h->nuE, X.rE, nE);  // tau13, tau23 (edges)
            KCHECK();
            CK(spectral_fft(h->spE, X.rE, X.tE, t));
            CK(zop(h, OP_DDZ_E2C, 1, X.tE, X.tC, t));
        }
        // the subtractions, after the previous chain's
        if (c > 0) CK(after(h, 3, (c % 2 == 0) ? B.st : A.st, t));
        switch (c) {
            case 0: k_sub_ik<<<gs, 256, 0, t>>>(h->urhs, 1, nullptr, 0, X.tC, k1, k2, nxh, nxy, h->SC); break;
            case 1: k_sub_ik<<<gs, 256, 0, t>>>(h->vrhs, 2, nullptr, 0, X.tC, k1, k2, nxh, nxy, h->SC); break;
            case 2: k_csub2<<<gsE, 256, 0, t>>>(h->wrhs, X.tE, h->SE); break;
            case 3: k_sub_ik<<<gs, 256, 0, t>>>(h->vrhs, 1, h->urhs, 2, X.tC, k1, k2, nxh, nxy, h->SC); break;
            default:
                k_csub2<<<gs, 256, 0, t>>>(c == 4 ? h->urhs : h->vrhs, X.tC, h->SC);
                KCHECK();
                k_sub_ik<<<gsE, 256, 0, t>>>(h->wrhs, c == 4 ? 1 : 2, nullptr, 0, X.tE, k1, k2, nxh, nxy, h->SE);
                break;
        }
        KCHECK();
    }
    return after(h, 2, h->s2, s);  // join
}

// RHS of one stage (addNonLinearTerm_Rot, addViscousTerm, getRHS_SGS; igrid.F90:1497-1571,
// 1793-1951).  The u chain runs on s, the v and w chains on the second stream with their
// own scratch (the u and v products transformed in pairs, one per grid and stream), and the
// pointwise eddy viscosity beside them.
int populate_rhs(pade_les h, cudaStream_t s) {
    const long n = h->NC, nE = h->NE;
    const unsigned g = grid_for(n), gE = grid_for(nE), gs = grid_for(h->SC), gsE = grid_for(h->SE);
    const Ptr9 dC = p9(h->dC), dE = p9(h->dE);
    const int visc = h->prm.isInviscid ? 0 : 1;
    const double r = 1.0 / h->prm.Re;
    const double* k1 = h->spC->d_k1;
    const double* k2 = h->spC->d_k2;
    const cudaStream_t s2 = h->s2;
    const bool early = h->prm.useSGS && nu_pointwise(h);
    CK(after(h, 0, s, s2));  // fork
    if (early) CK(sgs_nu_pointwise(h, s2));
    k_nl_c<<<g, 256, 0, s>>>(dC, h->u, h->v, h->rC1, h->rC2, n);
    KCHECK();
    k_nl_e<<<gE, 256, 0, s>>>(dE, h->w, h->uE, h->vE, h->rE1, h->rE2, h->rE3, nE);
    KCHECK();
    CK(after(h, 1, s, s2));  // the products are ready
    // the edge-grid products of u and v transformed as a pair (second stream), then w there;
    // the cell-grid pair on s; each stream then waits for the other's pair
    CK(spectral_fft_two(h->spE, h->rE1, h->rE2, h->tE1, h->tE1b, s2));
    if (cudaEventRecord(h->ev[4], s2) != cudaSuccess) return PS_ECUDA;  // the edge-grid pair is done
    CK(spectral_fft(h->spE, h->rE3, h->wrhs, s2));
    if (visc) {
        k_rhs_finish<<<gsE, 256, 0, s2>>>(h->wrhs, nullptr, h->what_cur, h->d2w, k1, k2, h->nxh, h->splane, r, 1,
                                           h->SE);
        KCHECK();
    }
    CK(spectral_fft_two(h->spC, h->rC1, h->rC2, h->tC1, h->tC1b, s));
    CK(after(h, 5, s, s2));
    // v (second stream, scratch tC1b / tE1b)
    CK(zop(h, OP_I_E2C, 1, h->tE1b, h->vrhs, s2));
    k_rhs_finish<<<gs, 256, 0, s2>>>(h->vrhs, h->tC1b, h->vhat_cur, h->d2v, k1, k2, h->nxh, h->splane, r, visc, h->SC);
    KCHECK();
    // u
    if (cudaStreamWaitEvent(s, h->ev[4], 0) != cudaSuccess) return PS_ECUDA;
    CK(zop(h, OP_I_E2C, 1, h->tE1, h->urhs, s));
    k_rhs_finish<<<gs, 256, 0, s>>>(h->urhs, h->tC1, h->uhat_cur, h->d2u, k1, k2, h->nxh, h->splane, r, visc, h->SC);
    KCHECK();
    CK(after(h, 2, s2, s));  // join
    if (!h->prm.useSGS) return PS_OK;
    CK(sgs_nu_rest(h, s));
    return sgs_tau_rhs(h, s);
}

int compute_dt(pade_les h, cudaStream_t s) {
    if (!(h->prm.CFL > 0)) {
        k_set<<<1, 1, 0, s>>>(h->d_dt, h->prm.dt);
        KCHECK();
        return PS_OK;
    }
    k_cfl_partial<<<kCflBlocks, 256, 0, s>>>(h->u, h->v, h->wC, 1.0 / h->dx, 1.0 / h->dy, 1.0 / h->dz, h->NC,
                                              h->cflpart);
    KCHECK();
    k_cfl_final<<<1, 1, 0, s>>>(h->cflpart, kCflBlocks, h->prm.CFL, h->tvisc, h->prm.isInviscid ? 0 : 1, h->d_dt);
    KCHECK();
    return PS_OK;
}

int rk_stage(pade_les h, int stage, cudaStream_t s) {
    const unsigned gs = grid_for(h->SC), gsE = grid_for(h->SE);
    k_rk<<<gs, 256, 0, s>>>(stage, h->uhat, h->uhat1, h->urhs, h->d_dt, h->SC);
    k_rk<<<gs, 256, 0, s>>>(stage, h->vhat, h->vhat1, h->vrhs, h->d_dt, h->SC);
    k_rk<<<gsE, 256, 0, s>>>(stage, h->what, h->what1, h->wrhs, h->d_dt, h->SE);
    KCHECK();
    return PS_OK;
}

void set_cur(pade_les h, bool stagecopy) {
    h->uhat_cur = stagecopy ? h->uhat1 : h->uhat;
    h->vhat_cur = stagecopy ? h->vhat1 : h->vhat;
    h->what_cur = stagecopy ? h->what1 : h->what;
}

// one TVD-RK3 step (igrid.F90:1105-1174) enqueued on s
int enqueue_step(pade_les h, cudaStream_t s) {
    CK(compute_dt(h, s));
    set_cur(h, false);
    CK(populate_rhs(h, s));
    h->newTimeStep = false;
    CK(rk_stage(h, 1, s));
    set_cur(h, true);
    CK(project_and_prep(h, s));
    CK(populate_rhs(h, s));
    CK(rk_stage(h, 2, s));
    set_cur(h, true);
    CK(project_and_prep(h, s));
    CK(populate_rhs(h, s));
    CK(rk_stage(h, 3, s));
    set_cur(h, false);
    CK(project_and_prep(h, s));
    k_advance<<<1, 1, 0, s>>>(h->d_tsim, h->d_dt);
    KCHECK();
    return PS_OK;
}

}  // namespace

extern "C" {

int pade_les_init(pade_les* out, const pade_les_params* p) {
    if (!out || !p) return PS_EINVAL;
    *out = nullptr;
    if (p->nx < 4 || p->ny < 4 || p->nz < 6 || !(p->Lx > 0) || !(p->Ly > 0) || !(p->Lz > 0)) return PS_EINVAL;
    if (!(p->isInviscid) && !(p->Re > 0)) return PS_EINVAL;
    if (!(p->CFL > 0) && !(p->dt > 0)) return PS_EINVAL;
    if (p->useSGS && (p->dynamic || p->learnedSGS) && !(p->deltaRatio > 0)) return PS_EINVAL;
    if (p->SGSModelID < 0 || p->SGSModelID > 2) return PS_EINVAL;
    if (p->useSGS && p->SGSModelID != 0 && (p->dynamic || p->learnedSGS)) return PS_ENOTSUP;
    if (p->useSGS && p->learnedSGS && !(p->Re > 0)) return PS_EINVAL;  // features use the molecular 1/Re
    for (int n : {p->nx, p->ny, p->nz})
        if (n > 8192 || (n & (n - 1)) != 0) return PS_ENOTSUP;
    auto* h = new pade_les_s();
    h->prm = *p;
    h->nx = p->nx;
    h->ny = p->ny;
    h->nz = p->nz;
    h->nxh = p->nx / 2 + 1;
    h->dx = p->Lx / p->nx;
    h->dy = p->Ly / p->ny;
    h->dz = p->Lz / p->nz;
    h->plane = (long)h->nx * h->ny;
    h->splane = (long)h->nxh * h->ny;
    h->NC = h->plane * h->nz;
    h->NE = h->plane * (h->nz + 1);
    h->SC = h->splane * h->nz;
    h->SE = h->splane * (h->nz + 1);
    const double pi = 3.141592653589793238462643383279502884;
    const double dfact = p->dealiasFact > 0 ? p->dealiasFact : 2.0 / 3.0;
    h->cut_x = dfact * pi / h->dx;
    h->cut_y = dfact * pi / h->dy;
    h->cut_z = dfact * pi / h->dz;
    h->tf_x = ((2.0 / 3.0) * pi / h->dx) / p->deltaRatio;
    h->tf_y = ((2.0 / 3.0) * pi / h->dy) / p->deltaRatio;
    const double deltaLES = std::pow(1.5 * h->dx * 1.5 * h->dy * 1.5 * h->dz, 1.0 / 3.0);
    h->deltaLES = deltaLES;
    h->cmodel_global = (p->Csgs * deltaLES) * (p->Csgs * deltaLES);
    if (p->SGSModelID == 2) {  // AMD.F90:1-14: anisotropic constants, cd06 Poincare constant in z
        h->camd_x = p->Csgs * h->dx * std::sqrt(1.0 / 12.0);
        h->camd_y = p->Csgs * h->dy * std::sqrt(1.0 / 12.0);
        h->camd_z = p->Csgs * h->dz * (1.0 / std::sqrt(10.0));
        h->cmodel_global = 1.0;
    }
    h->meanfact = 1.0 / ((double)h->nx * (double)h->ny);
    const double mn = std::min(h->dx, std::min(h->dy, h->dz));
    h->tvisc = p->CFL * p->Re * (mn * mn);
    int rc = pade_spectral_init(&h->spC, h->nx, h->ny, h->nz, h->dx, h->dy, 0);
    if (rc == PS_OK) rc = pade_spectral_init(&h->spE, h->nx, h->ny, h->nz + 1, h->dx, h->dy, 0);
    if (rc == PS_OK) rc = pade_poisson_periodic_init(&h->po, h->spC, h->dx, h->dy, h->dz);
    if (rc == PS_OK) rc = pade_cd06stagg_init_periodic(&h->stagg, h->nz, h->dz);
    if (rc == PS_OK && cudaStreamCreateWithFlags(&h->s2, cudaStreamNonBlocking) != cudaSuccess) rc = PS_ECUDA;
    for (int i = 0; i < 6 && rc == PS_OK; i++)
        if (cudaEventCreateWithFlags(&h->ev[i], cudaEventDisableTiming) != cudaSuccess) rc = PS_ECUDA;
    if (rc == PS_OK) {
        std::vector<double> k3 = wavenums(h->nz, h->dz);
        k3[h->nz / 2] = -k3[h->nz / 2];
        rc = upload(&h->d_k3, k3);
        if (rc == PS_OK) h->allocs.push_back(h->d_k3);
    }
    const size_t c16 = sizeof(double2), r8 = sizeof(double);
    double2** cC[] = {&h->uhat, &h->vhat, &h->uhat1, &h->vhat1, &h->urhs, &h->vrhs, &h->whatC, &h->d2u, &h->d2v,
                      &h->tC1, &h->tC1b};
    double2** cE[] = {&h->what, &h->what1, &h->wrhs, &h->uEhat, &h->vEhat, &h->d2w, &h->tE1, &h->tE1b};
    for (auto pp : cC)
        if (rc == PS_OK) rc = al(h, pp, c16 * h->SC);
    for (auto pp : cE)
        if (rc == PS_OK) rc = al(h, pp, c16 * h->SE);
    double** rCl[] = {&h->u, &h->v, &h->wC, &h->rC1, &h->rC2, &h->nuC, &h->div, &h->rC1b};
    double** rEl[] = {&h->w, &h->uE, &h->vE, &h->rE1, &h->rE2, &h->rE3, &h->nuE, &h->rE1b};
    for (auto pp : rCl)
        if (rc == PS_OK) rc = al(h, pp, r8 * h->NC);
    for (auto pp : rEl)
        if (rc == PS_OK) rc = al(h, pp, r8 * h->NE);
    for (int i = 0; i < 9 && rc == PS_OK; i++) rc = al(h, &h->dC[i], r8 * h->NC);
    for (int i = 0; i < 9 && rc == PS_OK; i++) rc = al(h, &h->dE[i], r8 * h->NE);
    if (p->useSGS && (p->dynamic || (p->learnedSGS && p->JudgeFreq > 0))) {
        for (int i = 0; i < 6 && rc == PS_OK; i++) rc = al(h, &h->Sf[i], r8 * h->NC);
        for (int i = 0; i < 6 && rc == PS_OK; i++) rc = al(h, &h->M[i], r8 * h->NC);
        for (int i = 0; i < 6 && rc == PS_OK; i++) rc = al(h, &h->Lm[i], r8 * h->NC);
        for (int i = 0; i < 3 && rc == PS_OK; i++) rc = al(h, &h->uf[i], r8 * h->NC);
        if (rc == PS_OK) rc = al(h, &h->Df, r8 * h->NC);
        if (rc == PS_OK) rc = al(h, &h->Dsgs, r8 * h->NC);
        if (rc == PS_OK) rc = al(h, &h->part, r8 * 2 * kPlaneChunks * h->nz);
    }
    if (p->useSGS && p->learnedSGS) {
        if (!h->part && rc == PS_OK) rc = al(h, &h->part, r8 * 2 * kPlaneChunks * h->nz);
        if (rc == PS_OK) rc = al(h, &h->lamL, r8 * h->nz);
        if (rc == PS_OK) rc = al(h, &h->fball, sizeof(int));
        if (rc == PS_OK) rc = al(h, &h->fbcount, sizeof(unsigned long long));
        if (rc == PS_OK) rc = al(h, &h->judge_err, r8);
        if (rc == PS_OK && (cudaMemset(h->fball, 0, sizeof(int)) != cudaSuccess ||
                            cudaMemset(h->fbcount, 0, sizeof(unsigned long long)) != cudaSuccess ||
                            cudaMemset(h->lamL, 0, r8 * h->nz) != cudaSuccess))
            rc = PS_ECUDA;
        if (rc == PS_OK) {
            const double m1 = -1.0;  // no judge step yet
            if (cudaMemcpy(h->judge_err, &m1, r8, cudaMemcpyHostToDevice) != cudaSuccess) rc = PS_ECUDA;
        }
    }
    if (rc == PS_OK) rc = al(h, &h->lambda, r8 * h->nz);
    if (rc == PS_OK) rc = al(h, &h->d_dt, r8);
    if (rc == PS_OK) rc = al(h, &h->d_tsim, r8);
    if (rc == PS_OK) rc = al(h, &h->cflpart, r8 * kCflBlocks);
    if (rc == PS_OK && cudaMemset(h->lambda, 0, r8 * h->nz) != cudaSuccess) rc = PS_ECUDA;
    if (rc == PS_OK && p->useSGS && p->learnedSGS) {
        // the closure's fallback before any judge step: the constant Smagorinsky coefficient
        const std::vector<double> c(h->nz, h->cmodel_global);
        if (cudaMemcpy(h->lambda, c.data(), r8 * h->nz, cudaMemcpyHostToDevice) != cudaSuccess) rc = PS_ECUDA;
    }
    if (rc == PS_OK && cudaMemset(h->d_tsim, 0, r8) != cudaSuccess) rc = PS_ECUDA;
    if (rc == PS_OK && cudaMemset(h->d_dt, 0, r8) != cudaSuccess) rc = PS_ECUDA;
    if (rc != PS_OK) {
        pade_les_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_les_destroy(pade_les h) {
    if (!h) return PS_OK;
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    for (cudaEvent_t e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->s2) cudaStreamDestroy(h->s2);
    if (h->stagg) pade_destroy(h->stagg);
    if (h->po) pade_poisson_destroy(h->po);
    if (h->spE) pade_spectral_destroy(h->spE);
    if (h->spC) pade_spectral_destroy(h->spC);
    delete h;
    return PS_OK;
}

int pade_les_set_fields(pade_les h, const double* u, const double* v, const double* w, void* stream) {
    if (!h || !device_ptr(u) || !device_ptr(v) || !device_ptr(w)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // igrid.F90:625-648: transform, dealias, divergence report, project, prepare
    CK(spectral_fft(h->spC, u, h->uhat, s));
    CK(spectral_fft(h->spC, v, h->vhat, s));
    CK(spectral_fft(h->spE, w, h->what, s));
    set_cur(h, false);
    CK(dealias(h, h->uhat, 0, s));
    CK(dealias(h, h->vhat, 0, s));
    CK(dealias(h, h->what, 1, s));
    CK(pade_poisson_projection(h->po, h->uhat, h->vhat, h->what, s));
    CK(prep_physical(h, s));
    h->step = 0;
    h->mstep = 0;
    h->newTimeStep = true;
    if (cudaMemsetAsync(h->d_tsim, 0, sizeof(double), s) != cudaSuccess) return PS_ECUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? PS_OK : PS_ECUDA;
}

int pade_les_set_time(pade_les h, double tsim, int step) {
    if (!h || step < 0 || !std::isfinite(tsim)) return PS_EINVAL;
    if (cudaMemcpy(h->d_tsim, &tsim, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return PS_ECUDA;
    h->step = step;
    h->mstep = step;
    return PS_OK;
}

int pade_les_step(pade_les h, int use_graph, void* stream) {
    if (!h) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool divcheck = h->prm.t_DivergenceCheck > 0 && h->step % h->prm.t_DivergenceCheck == 0;
    bool fixed_shape;  // the same kernel sequence every step, so one captured graph serves all
    if (!h->prm.useSGS)
        fixed_shape = true;
    else if (h->prm.learnedSGS)
        fixed_shape = h->prm.JudgeFreq <= 0;
    else
        fixed_shape = !h->prm.dynamic || h->prm.DynProcFreq <= 1;
    if (use_graph && !divcheck && fixed_shape && s != nullptr) {
        if (!h->gexec || h->gstream != s) {
            if (h->gexec) cudaGraphExecDestroy(h->gexec);
            if (h->graph) cudaGraphDestroy(h->graph);
            h->gexec = nullptr;
            h->graph = nullptr;
            const int saved_m = h->mstep;
            const bool saved_n = h->newTimeStep;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return PS_ECUDA;
            const int rc = enqueue_step(h, s);
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(s, &g);
            h->mstep = saved_m;
            h->newTimeStep = saved_n;
            if (rc != PS_OK || ce != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return rc != PS_OK ? rc : PS_ECUDA;
            }
            if (cudaGraphInstantiate(&h->gexec, g, 0) != cudaSuccess) {
                cudaGraphDestroy(g);
                cudaGetLastError();
                return PS_ECUDA;
            }
            h->graph = g;
            h->gstream = s;
        }
        if (cudaGraphLaunch(h->gexec, s) != cudaSuccess) return PS_ECUDA;
        if (h->prm.useSGS) h->mstep++;  // the captured step ran populate_rhs with newTimeStep once
        h->newTimeStep = true;
    } else {
        CK(enqueue_step(h, s));
        h->newTimeStep = true;
    }
    h->step++;
    return PS_OK;
}

int pade_les_set_mlp(pade_les h, pade_mlp mlp) {
    if (!h) return PS_EINVAL;
    h->mlp = mlp;
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->gexec = nullptr;
    h->graph = nullptr;
    return PS_OK;
}

int pade_les_info(pade_les h, double* dt, double* tsim, int* step, double* lambda1d) {
    if (!h) return PS_EINVAL;
    double d[2] = {0, 0};
    if (cudaMemcpy(&d[0], h->d_dt, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
    if (cudaMemcpy(&d[1], h->d_tsim, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
    if (dt) *dt = d[0];
    if (tsim) *tsim = d[1];
    if (step) *step = h->step;
    if (lambda1d && cudaMemcpy(lambda1d, h->lambda, sizeof(double) * h->nz, cudaMemcpyDeviceToHost) != cudaSuccess)
        return PS_ECUDA;
    return PS_OK;
}

int pade_les_judge_info(pade_les h, double* err, double* lambda_closure, long long* n_fallback) {
    if (!h) return PS_EINVAL;
    if (!h->prm.learnedSGS || !h->judge_err) return PS_ENOTSUP;
    if (cudaDeviceSynchronize() != cudaSuccess) return PS_ECUDA;
    if (err && cudaMemcpy(err, h->judge_err, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
    if (lambda_closure &&
        cudaMemcpy(lambda_closure, h->lamL, sizeof(double) * h->nz, cudaMemcpyDeviceToHost) != cudaSuccess)
        return PS_ECUDA;
    if (n_fallback) {
        unsigned long long c = 0;
        if (cudaMemcpy(&c, h->fbcount, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
        *n_fallback = (long long)c;
    }
    return PS_OK;
}

int pade_les_scalar_sgs(pade_les h, const double* T, const void* That_, const double* dTdxC, const double* dTdyC,
                        const double* dTdzC, const double* dTdzE, void* Trhs_, double Pr, int dynamic,
                        double* beta1d, void* stream) {
    if (!h || !h->prm.useSGS) return PS_EINVAL;
    for (const void* q : {(const void*)T, That_, (const void*)dTdxC, (const void*)dTdyC, (const void*)dTdzC,
                          (const void*)dTdzE, (const void*)Trhs_})
        if (!q || !device_ptr(q)) return PS_EINVAL;
    if (dynamic && h->prm.SGSModelID != 0) return PS_ENOTSUP;  // Dsgs is the Smagorinsky kernel
    if (!dynamic && !(Pr > 0.0)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double2* That = static_cast<const double2*>(That_);
    double2* Trhs = static_cast<double2*>(Trhs_);
    const long n = h->NC, nE = h->NE;
    const unsigned g = grid_for(n), gE = grid_for(nE), gs = grid_for(h->SC);
    double* kC = h->rC1b;  // kappa at cells and edges (the second stream's scratch is free between steps)
    double* kE = h->rE1b;
    if (dynamic) {
        // the momentum procedure's arrays (kept when the LES itself is dynamic; allocated here otherwise)
        const size_t r8 = sizeof(double);
        int rc = PS_OK;
        for (int i = 0; i < 6 && rc == PS_OK; i++)
            if (!h->Sf[i]) rc = al(h, &h->Sf[i], r8 * n);
        for (int i = 0; i < 6 && rc == PS_OK; i++)
            if (!h->Lm[i]) rc = al(h, &h->Lm[i], r8 * n);
        for (int i = 0; i < 3 && rc == PS_OK; i++)
            if (!h->uf[i]) rc = al(h, &h->uf[i], r8 * n);
        if (rc == PS_OK && !h->Df) rc = al(h, &h->Df, r8 * n);
        if (rc == PS_OK && !h->Dsgs) rc = al(h, &h->Dsgs, r8 * n);
        if (rc == PS_OK && !h->part) rc = al(h, &h->part, r8 * 2 * kPlaneChunks * h->nz);
        if (rc == PS_OK && !h->betaT) rc = al(h, &h->betaT, r8 * h->nz);
        if (rc != PS_OK) return rc;
        const Ptr9 dC = p9(h->dC);
        // Dsgs = |S|, the test-filtered |S| and velocities of the current fields
        // (standardDynamicProcedure.F90:88-105, as the momentum procedure computes them)
        k_nu_kernel<<<g, 256, 0, s>>>(dC, h->rC2, h->Dsgs, n);
        KCHECK();
        for (int i = 0; i < 6; i++) {
            k_sij<<<g, 256, 0, s>>>(dC, i, nullptr, h->rC1, n);
            KCHECK();
            CK(test_filter(h, h->rC1, h->Sf[i], s));
        }
        k_smag6<<<g, 256, 0, s>>>(h->Sf[0], h->Sf[1], h->Sf[2], h->Sf[3], h->Sf[4], h->Sf[5], h->Df, n);
        KCHECK();
        CK(spectral_ifft_masked(h->spC, h->uhat_cur, h->uf[0], h->tf_x, h->tf_y, s));
        CK(spectral_ifft_masked(h->spC, h->vhat_cur, h->uf[1], h->tf_x, h->tf_y, s));
        CK(spectral_ifft_masked(h->spC, h->whatC, h->uf[2], h->tf_x, h->tf_y, s));
        // DoStandardDynamicProcedureScalar (standardDynamicProcedure.F90:22-68); the filtered
        // gradients take Sf[0..2], the filtered T Sf[3], R and P the arrays Lm
        const double dr2 = h->prm.deltaRatio * h->prm.deltaRatio;
        const double* dT[3] = {dTdxC, dTdyC, dTdzC};
        for (int i = 0; i < 3; i++) CK(test_filter(h, dT[i], h->Sf[i], s));
        for (int i = 0; i < 3; i++) {
            k_prod<<<g, 256, 0, s>>>(h->Dsgs, dT[i], h->rC1, n);
            KCHECK();
            CK(test_filter(h, h->rC1, h->rC2, s));
            k_mij<<<g, 256, 0, s>>>(h->rC2, h->Df, h->Sf[i], dr2, h->Lm[i], n);
            KCHECK();
        }
        CK(spectral_ifft_masked(h->spC, That, h->Sf[3], h->tf_x, h->tf_y, s));
        const double* U[3] = {h->u, h->v, h->wC};
        for (int i = 0; i < 3; i++) {
            k_prod<<<g, 256, 0, s>>>(U[i], T, h->rC1, n);
            KCHECK();
            CK(test_filter(h, h->rC1, h->rC2, s));
            k_lij<<<g, 256, 0, s>>>(h->rC2, h->uf[i], h->Sf[3], h->Lm[3 + i], n);
            KCHECK();
        }
        k_num_den3<<<g, 256, 0, s>>>(h->Lm[0], h->Lm[1], h->Lm[2], h->Lm[3], h->Lm[4], h->Lm[5], h->rC1, h->rC2, n);
        KCHECK();
        dim3 grid(kPlaneChunks, h->nz);
        k_plane_sums<<<grid, 256, 0, s>>>(h->rC1, h->rC2, h->plane, h->part);
        KCHECK();
        k_lambda<<<(h->nz + 127) / 128, 128, 0, s>>>(h->part, kPlaneChunks, h->meanfact, h->nz, h->betaT);
        KCHECK();
        // kappa = Dsgs Beta(z), interpolated to the edges (interpolate_kappaSGS, eddyViscosity.F90:120-129)
        k_kappa<<<g, 256, 0, s>>>(h->Dsgs, h->betaT, 0.0, h->plane, kC, n);
        KCHECK();
        CK(zop(h, OP_I_C2E, 0, kC, kE, s));
    } else {
        k_kappa<<<g, 256, 0, s>>>(h->nuC, nullptr, 1.0 / Pr, h->plane, kC, n);
        KCHECK();
        k_kappa<<<gE, 256, 0, s>>>(h->nuE, nullptr, 1.0 / Pr, h->plane, kE, nE);
        KCHECK();
    }
    // getRHS_SGS_Scalar (sgsmod_igrid.F90:282-301): Trhs -= ik1 q1hat + ik2 q2hat + ddz_E2C(q3hat)
    const double* k1 = h->spC->d_k1;
    const double* k2 = h->spC->d_k2;
    k_negmul<<<g, 256, 0, s>>>(kC, dTdxC, h->rC2, n);
    KCHECK();
    CK(spectral_fft(h->spC, h->rC2, h->tC1, s));
    k_sub_ik<<<gs, 256, 0, s>>>(Trhs, 1, nullptr, 0, h->tC1, k1, k2, h->nxh, h->splane, h->SC);
    KCHECK();
    k_negmul<<<g, 256, 0, s>>>(kC, dTdyC, h->rC2, n);
    KCHECK();
    CK(spectral_fft(h->spC, h->rC2, h->tC1, s));
    k_sub_ik<<<gs, 256, 0, s>>>(Trhs, 2, nullptr, 0, h->tC1, k1, k2, h->nxh, h->splane, h->SC);
    KCHECK();
    k_negmul<<<gE, 256, 0, s>>>(kE, dTdzE, h->rE2, nE);
    KCHECK();
    CK(spectral_fft(h->spE, h->rE2, h->tE1, s));
    CK(zop(h, OP_DDZ_E2C, 1, h->tE1, h->tC1, s));
    k_csub2<<<gs, 256, 0, s>>>(Trhs, h->tC1, h->SC);
    KCHECK();
    if (beta1d && dynamic) {
        if (cudaMemcpyAsync(beta1d, h->betaT, sizeof(double) * h->nz, cudaMemcpyDefault, s) != cudaSuccess)
            return PS_ECUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return PS_ECUDA;
    }
    return PS_OK;
}

int pade_les_field(pade_les h, int which, void** ptr) {
    if (!h || !ptr) return PS_EINVAL;
    void* p = nullptr;
    if (which >= 10 && which < 19) {
        p = h->dC[which - 10];
    } else if (which >= 20 && which < 29) {
        p = h->dE[which - 20];
    } else {
        switch (which) {
            case PADE_LES_UHAT: p = h->uhat; break;
            case PADE_LES_VHAT: p = h->vhat; break;
            case PADE_LES_WHAT: p = h->what; break;
            case PADE_LES_U: p = h->u; break;
            case PADE_LES_V: p = h->v; break;
            case PADE_LES_WC: p = h->wC; break;
            case PADE_LES_W: p = h->w; break;
            case PADE_LES_UE: p = h->uE; break;
            case PADE_LES_VE: p = h->vE; break;
            case PADE_LES_NUC: p = h->nuC; break;
            case PADE_LES_NUE: p = h->nuE; break;
            default: return PS_EINVAL;
        }
    }
    *ptr = p;
    return PS_OK;
}

}  // extern "C"
