// Spectral (x-y Fourier) layer, PadePoisson's periodic projection and divergence check,
// PoissonPeriodic, and the pencil transposes, on one GPU.
//
// One GPU holds the whole grid, so the x, y and z pencils of the reference's 2DECOMP
// decomposition are the same (i, j, k) Fortran-ordered array: every transform runs on
// strided lines in place and the transposes are plain copies.
//
//  spectral  (spectral.F90:1413-1452, fft_3d.F90:616-663)
//      fft:  r2c along x, c2c forward along y          (nx, ny, nz) -> (nx/2+1, ny, nz)
//      ifft: c2c backward along y, optional oddball (x-Nyquist) zeroing, c2r along x,
//            scaled by 1/(nx ny)
//      wavenumbers k1, k2 (spectral.F90:1025-1075, 1200-1215): GetWaveNums with the
//      oddball's sign flipped, and zeroed at the Nyquist index when fixOddball is set.
//  padepoisson, periodic in z (PadePoisson.F90:76-128, 386-432, 1165-1246)
//      PressureProjection: dwdz = ddz_E2C(what) (staggered CD06), one fused z kernel
//      (divergence, z FFT, division by -|k|^2 with the CD06-stagg modified z wavenumber,
//      inverse FFT, pressure store, uhat/vhat update), ddz_C2E(p), what -= that.
//      DivergenceCheck: ddz_E2C(what) + i (k1 uhat + k2 vhat), ifft, signed maximum;
//      with fixDiv it re-projects above 1e-13 and once more above 1e-10.
//  PoissonPeriodic (PoissonPeriodic.F90:37-111, 114-204)
//      r2c x, c2c y, fused z (FFT, -1/(|k|^2 + 1e-20) with the zero mode 0, inverse),
//      c2c y, c2r x scaled by 1/(nx ny nz); optional modified-wavenumber callbacks.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "fft.h"
#include "operators.h"
#include "spectral_internal.h"

namespace pade {

bool device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

namespace {
bool pow2_len(int n) { return n >= 2 && n <= 8192 && (n & (n - 1)) == 0; }
}  // namespace

// GetWaveNums (spectral.F90:1748-1764, PoissonPeriodic.F90:226-242): k(i) =
// (-pi + (i-1)*2*pi/dummy)/dx for i = 1..n, dummy = n - mod(n,2), then ifftshift.
std::vector<double> wavenums(int n, double dx) {
    const double pi = 3.141592653589793238462643383279502884;  // 4*atan(1) in FP64
    const int dummy = n - n % 2;
    std::vector<double> k(n), s(n);
    for (int i = 1; i <= n; i++) k[i - 1] = (-pi + (double)(i - 1) * 2.0 * pi / (double)dummy) / dx;
    if (n % 2 == 0) {
        for (int i = 0; i < n / 2; i++) s[i] = k[n / 2 + i];
        for (int i = 0; i < n / 2; i++) s[n / 2 + i] = k[i];
    } else {
        const int h = (n + 1) / 2;
        for (int i = 0; i < h; i++) s[i] = k[h - 1 + i];
        for (int i = 0; i < (n - 1) / 2; i++) s[h + i] = k[i];
    }
    return s;
}

// getmodCD06stagg (PadeDerOps.F90:1034-1053): modified wavenumber of the staggered CD06
// first derivative, alpha = 9/62, a = 63/62, b = 17/62 (beta = c = 0).
void modk_cd06stagg(const double* k, int n, double dx, double* kp) {
    const double alpha = 9.0 / 62.0, beta = 0.0, a = 63.0 / 62.0, b = 17.0 / 62.0, c = 0.0;
    for (int i = 0; i < n; i++) {
        const double w = k[i] * dx;
        const double num = 2.0 * a * std::sin(w / 2.0) + (2.0 / 3.0) * b * std::sin(3.0 * w / 2.0) +
                           (2.0 / 5.0) * c * std::sin(5.0 * w / 2.0);
        const double den = 1.0 + 2.0 * alpha * std::cos(w) + 2.0 * beta * std::cos(2.0 * w);
        kp[i] = (num / den) / dx;
    }
}

int dalloc(void** p, size_t bytes) {
    if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return PS_ENOMEM;
    }
    return PS_OK;
}

unsigned grid_for(long n) {
    const long b = (n + 255) / 256;
    return (unsigned)std::max(1L, std::min(b, 152L * 16));
}

namespace {

// y -= x (complex), what -= dwdzHATz_Periodic (PadePoisson.F90:415)
__global__ void k_csub(double2* __restrict__ y, const double2* __restrict__ x, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const double2 a = y[e], b = x[e];
        y[e] = make_double2(a.x - b.x, a.y - b.y);
    }
}

// f += i k1 uhat + i k2 vhat (PadePoisson.F90:1191-1198), evaluated in that order
__global__ void k_div_add(double2* __restrict__ f, const double2* __restrict__ u, const double2* __restrict__ v,
                          const double* __restrict__ k1, const double* __restrict__ k2, long nxh, long nxy, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long r = e % nxy;
        const double a = k1[r % nxh], b = k2[r / nxh];
        const double2 ff = f[e], uu = u[e], vv = v[e];
        const double re = __dadd_rn(__dadd_rn(ff.x, -__dmul_rn(a, uu.y)), -__dmul_rn(b, vv.y));
        const double im = __dadd_rn(__dadd_rn(ff.y, __dmul_rn(a, uu.x)), __dmul_rn(b, vv.x));
        f[e] = make_double2(re, im);
    }
}

// per-block maximum of a real array; the host reduces the partial results
__global__ void k_max_partial(const double* __restrict__ x, long n, double* __restrict__ part) {
    __shared__ double s[32];
    double m = -INFINITY;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        m = fmax(m, x[e]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) part[blockIdx.x] = m;
    }
}

}  // namespace

int spectral_fft(pade_spectral h, const double* in, void* out, cudaStream_t s) {
    const FftExtra ex{};
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nx, h->nxh);
    int rc = fft_launch(IN_REAL, OUT_HALF, FK_PLAIN, h->nx, -1, 1.0, 0, in, out, lx, ex, s);
    if (rc != PS_OK) return rc;
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    return fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, -1, 1.0, 0, out, out, ly, ex, s);
}

int spectral_ifft(pade_spectral h, const void* in, double* out, int oddball, cudaStream_t s, int mul) {
    FftExtra ex{};
    ex.mul = mul;
    ex.km = mul == MUL_IK_A ? h->d_k1 : h->d_k2;
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    int rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, 1, 1.0, 0, in, h->work, ly, ex, s);
    if (rc != PS_OK) return rc;
    ex = FftExtra{};
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nxh, h->nx);
    const double norm = 1.0 / ((double)h->nx * (double)h->ny);
    return fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, oddball, h->work, out, lx, ex, s);
}

int spectral_ifft_pair(pade_spectral h, const void* in, double* out, double* out_dx, cudaStream_t s) {
    FftExtra ex{};
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    int rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, 1, 1.0, 0, in, h->work, ly, ex, s);
    if (rc != PS_OK) return rc;
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nxh, h->nx);
    const double norm = 1.0 / ((double)h->nx * (double)h->ny);
    // both real outputs from one complex transform where that kernel applies
    rc = fft_c2r_pair(h->work, nullptr, out, out_dx, lx, h->nx, norm, h->d_k1, s);
    if (rc != PS_ENOTSUP) return rc;
    rc = fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, 0, h->work, out, lx, ex, s);
    if (rc != PS_OK) return rc;
    // i k1 on the y-transformed half spectrum: k1 depends on the x index alone, so it
    // commutes with the y transform
    ex.mul = MUL_IK_P;
    ex.km = h->d_k1;
    rc = fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, 0, h->work, out_dx, lx, ex, s);
    if (rc != PS_ENOTSUP) return rc;
    return spectral_ifft(h, in, out_dx, 0, s, MUL_IK_A);  // transforms without that multiplier
}

int spectral_fft_two(pade_spectral h, const double* in1, const double* in2, void* out1, void* out2, cudaStream_t s) {
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nx, h->nxh);
    int rc = fft_r2c_pair(in1, in2, out1, out2, lx, h->nx, 1.0, s);
    if (rc == PS_ENOTSUP) {
        rc = spectral_fft(h, in1, out1, s);
        if (rc != PS_OK) return rc;
        return spectral_fft(h, in2, out2, s);
    }
    if (rc != PS_OK) return rc;
    const FftExtra ex{};
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, -1, 1.0, 0, out1, out1, ly, ex, s);
    if (rc != PS_OK) return rc;
    return fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, -1, 1.0, 0, out2, out2, ly, ex, s);
}

int spectral_ifft_two(pade_spectral h, const void* in1, int mul1, const void* in2, int mul2, double* out1,
                      double* out2, void* w1, void* w2, cudaStream_t s) {
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    for (int t = 0; t < 2; t++) {
        FftExtra ex{};
        ex.mul = t == 0 ? mul1 : mul2;
        ex.km = ex.mul == MUL_IK_A ? h->d_k1 : h->d_k2;
        const int rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, 1, 1.0, 0, t == 0 ? in1 : in2,
                                  t == 0 ? w1 : w2, ly, ex, s);
        if (rc != PS_OK) return rc;
    }
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nxh, h->nx);
    const double norm = 1.0 / ((double)h->nx * (double)h->ny);
    int rc = fft_c2r_pair(w1, w2, out1, out2, lx, h->nx, norm, nullptr, s);
    if (rc != PS_ENOTSUP) return rc;
    FftExtra ex{};
    rc = fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, 0, w1, out1, lx, ex, s);
    if (rc != PS_OK) return rc;
    return fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, 0, w2, out2, lx, ex, s);
}

int spectral_ifft_masked(pade_spectral h, const void* in, double* out, double cut1, double cut2, cudaStream_t s) {
    FftExtra ex{};
    ex.mul = MUL_MASK_AP;
    ex.ka = h->d_k1;
    ex.kb = h->d_k2;
    ex.cut_a = cut1;
    ex.cut_b = cut2;
    FftLines ly = fft_lines(2, h->nxh, h->ny, h->nz, h->ny, h->ny);
    int rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, h->ny, 1, 1.0, 0, in, h->work, ly, ex, s);
    if (rc != PS_OK) return rc;
    ex = FftExtra{};
    FftLines lx = fft_lines(1, h->nx, h->ny, h->nz, h->nxh, h->nx);
    const double norm = 1.0 / ((double)h->nx * (double)h->ny);
    return fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, h->nx, 1, norm, 0, h->work, out, lx, ex, s);
}

}  // namespace pade

using namespace pade;

namespace {

int projection(pade_poisson h, void* uhat, void* vhat, void* what, cudaStream_t s) {
    if (!h->periodic) return wall_projection(h, uhat, vhat, what, s);
    const int nxh = h->nxh, ny = h->ny, nz = h->nz;
    // dwdz at cell centres (PadePoisson.F90:405)
    int rc = pade_apply(h->stagg, 0, 3, 1, what, h->f2d, nxh, ny, 0, 0, PADE_PATH_DF, s);
    if (rc != PS_OK) return rc;
    FftExtra ex{};
    ex.ka = h->d_k1r;
    ex.kb = h->d_k2r;
    ex.kc = h->d_k3m;
    ex.k1 = h->sp->d_k1;
    ex.k2 = h->sp->d_k2;
    ex.u = static_cast<double2*>(uhat);
    ex.v = static_cast<double2*>(vhat);
    ex.nxh = nxh;
    ex.plane = (long)nxh * ny;
    ex.mtab = h->d_mtab;
    FftLines lz = fft_lines(3, nxh, ny, nz, nz, nz);
    rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PROJECT, nz, -1, 1.0 / (double)nz, 0, h->f2d, h->f2d, lz, ex, s);
    if (rc != PS_OK) return rc;
    // what -= ddz_C2E(p) (PadePoisson.F90:414-416)
    rc = pade_apply(h->stagg, 1, 3, 1, h->f2d, h->dwE, nxh, ny, 0, 0, PADE_PATH_DF, s);
    if (rc != PS_OK) return rc;
    const long nE = (long)nxh * ny * (nz + 1);
    k_csub<<<grid_for(nE), 256, 0, s>>>(static_cast<double2*>(what), h->dwE, nE);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

// getPressure / getPressureAndUpdateRHS (PadePoisson.F90:716-1163): the projection's
// pressure (plus the Stokes pressure with walls), as a real (nx, ny, nz) field; `update`
// also projects uhat, vhat, what, otherwise they are left unchanged (the projection runs
// on copies).
int get_pressure(pade_poisson h, void* uhat, void* vhat, void* what, double* pressure, int update, cudaStream_t s) {
    const size_t plane = (size_t)h->nxh * h->ny;
    const size_t bc = sizeof(double2) * plane * h->nz, be = sizeof(double2) * plane * (h->nz + 1);
    void *u = uhat, *v = vhat, *w = what;
    int rc = PS_OK;
    if (!update) {
        if (!h->su) rc = dalloc((void**)&h->su, bc);
        if (rc == PS_OK && !h->sv) rc = dalloc((void**)&h->sv, bc);
        if (rc == PS_OK && !h->sw) rc = dalloc((void**)&h->sw, be);
        if (rc != PS_OK) return rc;
        if (cudaMemcpyAsync(h->su, uhat, bc, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(h->sv, vhat, bc, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(h->sw, what, be, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return PS_ECUDA;
        u = h->su;
        v = h->sv;
        w = h->sw;
    }
    if ((rc = projection(h, u, v, w, s)) != PS_OK) return rc;  // leaves the pressure in f2d (periodic)
    if (!h->periodic && (rc = wall_pressure(h, s)) != PS_OK) return rc;
    return spectral_ifft(h->sp, h->f2d, pressure, 0, s);
}

int divergence(pade_poisson h, const void* uhat, const void* vhat, const void* what, double* div, cudaStream_t s) {
    const int nxh = h->nxh, ny = h->ny, nz = h->nz;
    int rc = pade_apply(h->stagg, 0, 3, 1, what, h->f2d, nxh, ny, 0, 0, PADE_PATH_DF, s);
    if (rc != PS_OK) return rc;
    const long n = (long)nxh * ny * nz;
    k_div_add<<<grid_for(n), 256, 0, s>>>(h->f2d, static_cast<const double2*>(uhat),
                                           static_cast<const double2*>(vhat), h->sp->d_k1, h->sp->d_k2, nxh,
                                           (long)nxh * ny, n);
    if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
    return spectral_ifft(h->sp, h->f2d, div, 0, s);
}

int max_of(pade_poisson h, const double* x, long n, double* out, cudaStream_t s) {
    const unsigned g = (unsigned)std::min<long>(kMaxPartials, std::max(1L, (n + 1023) / 1024));
    k_max_partial<<<g, 256, 0, s>>>(x, n, h->part);
    if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
    std::vector<double> p(g);
    if (cudaMemcpyAsync(p.data(), h->part, sizeof(double) * g, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return PS_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PS_ECUDA;
    double m = -INFINITY;
    for (double v : p) m = std::fmax(m, v);
    *out = m;
    return PS_OK;
}

}  // namespace

extern "C" {

int pade_wavenumbers(int n, double dx, double* k) {
    if (n < 1 || !k || !(dx > 0 || dx < 0)) return PS_EINVAL;
    const std::vector<double> w = wavenums(n, dx);
    for (int i = 0; i < n; i++) k[i] = w[i];
    return PS_OK;
}

int pade_modified_wavenumbers_cd06stagg(const double* k, int n, double dz, double* kp) {
    if (n < 1 || !k || !kp || !(dz > 0 || dz < 0)) return PS_EINVAL;
    modk_cd06stagg(k, n, dz, kp);
    return PS_OK;
}

// ---------------------------------------------------------------- spectral
int pade_spectral_init(pade_spectral* out, int nx, int ny, int nz, double dx, double dy, int fix_oddball) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    if (nz < 1 || !(dx > 0) || !(dy > 0)) return PS_EINVAL;
    if (!pow2_len(nx) || !pow2_len(ny)) return PS_ENOTSUP;
    auto* h = new pade_spectral_s();
    h->nx = nx;
    h->ny = ny;
    h->nz = nz;
    h->nxh = nx / 2 + 1;
    h->dx = dx;
    h->dy = dy;
    h->fix_oddball = fix_oddball ? 1 : 0;
    std::vector<double> k1 = wavenums(nx, dx), k2 = wavenums(ny, dy);
    k1[nx / 2] = -k1[nx / 2];  // flip the sign of the oddball (spectral.F90:1029-1032)
    k2[ny / 2] = -k2[ny / 2];
    if (h->fix_oddball) {       // spectral.F90:1200-1215
        k1[nx / 2] = 0.0;
        k2[ny / 2] = 0.0;
    }
    h->k1.assign(k1.begin(), k1.begin() + h->nxh);
    h->k2 = k2;
    int rc = upload(&h->d_k1, h->k1);
    if (rc == PS_OK) rc = upload(&h->d_k2, h->k2);
    if (rc == PS_OK) rc = dalloc((void**)&h->work, sizeof(double2) * (size_t)h->nxh * ny * nz);
    if (rc != PS_OK) {
        pade_spectral_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_spectral_destroy(pade_spectral h) {
    if (!h) return PS_OK;
    cudaFree(h->d_k1);
    cudaFree(h->d_k2);
    cudaFree(h->work);
    cudaFree(h->work2);
    delete h;
    return PS_OK;
}

int pade_spectral_get_wavenumbers(pade_spectral h, double* k1, double* k2) {
    if (!h || !k1 || !k2) return PS_EINVAL;
    for (int i = 0; i < h->nxh; i++) k1[i] = h->k1[i];
    for (int j = 0; j < h->ny; j++) k2[j] = h->k2[j];
    return PS_OK;
}

int pade_spectral_fft(pade_spectral h, const double* in, void* out, void* stream) {
    if (!h || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    return spectral_fft(h, in, out, static_cast<cudaStream_t>(stream));
}

int pade_spectral_ifft(pade_spectral h, const void* in, double* out, int set_oddball, void* stream) {
    if (!h || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    return spectral_ifft(h, in, out, set_oddball ? 1 : 0, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------- fused spectral layer
namespace {
int mul_of(int d) { return d == 1 ? MUL_IK_A : d == 2 ? MUL_IK_P : MUL_NONE; }
}  // namespace

int pade_spectral_ifft_ik(pade_spectral h, const void* in, double* out, int d, void* stream) {
    if (!h || (d != 1 && d != 2) || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    return spectral_ifft(h, in, out, 0, static_cast<cudaStream_t>(stream), mul_of(d));
}

int pade_spectral_ifft_and_ddx(pade_spectral h, const void* in, double* out, double* out_dx, void* stream) {
    if (!h || !device_ptr(in) || !device_ptr(out) || !device_ptr(out_dx)) return PS_EINVAL;
    return spectral_ifft_pair(h, in, out, out_dx, static_cast<cudaStream_t>(stream));
}

int pade_spectral_fft_two(pade_spectral h, const double* in1, const double* in2, void* out1, void* out2,
                          void* stream) {
    if (!h || !device_ptr(in1) || !device_ptr(in2) || !device_ptr(out1) || !device_ptr(out2)) return PS_EINVAL;
    return spectral_fft_two(h, in1, in2, out1, out2, static_cast<cudaStream_t>(stream));
}

int pade_spectral_ifft_two(pade_spectral h, const void* in1, int d1, const void* in2, int d2, double* out1,
                           double* out2, void* stream) {
    if (!h || d1 < 0 || d1 > 2 || d2 < 0 || d2 > 2) return PS_EINVAL;
    if (!device_ptr(in1) || !device_ptr(in2) || !device_ptr(out1) || !device_ptr(out2)) return PS_EINVAL;
    if (!h->work2) {
        const size_t bytes = sizeof(double2) * (size_t)h->nxh * h->ny * h->nz;
        if (cudaMalloc(&h->work2, bytes) != cudaSuccess) {
            cudaGetLastError();
            h->work2 = nullptr;
            return PS_ENOMEM;
        }
    }
    return spectral_ifft_two(h, in1, mul_of(d1), in2, mul_of(d2), out1, out2, h->work, h->work2,
                             static_cast<cudaStream_t>(stream));
}

int pade_spectral_ifft_testfilter(pade_spectral h, const void* in, double* out, double filtfact, void* stream) {
    if (!h || !(filtfact > 0) || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    const double pi = 3.141592653589793238462643383279502884;
    const double cut1 = ((2.0 / 3.0) * pi / h->dx) / filtfact;
    const double cut2 = ((2.0 / 3.0) * pi / h->dy) / filtfact;
    return spectral_ifft_masked(h, in, out, cut1, cut2, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------- padepoisson
int pade_poisson_periodic_init(pade_poisson* out, pade_spectral sp, double dx, double dy, double dz) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    if (!sp || !(dx > 0) || !(dy > 0) || !(dz > 0)) return PS_EINVAL;
    if (!pow2_len(sp->nz)) return PS_ENOTSUP;
    auto* h = new pade_poisson_s();
    h->sp = sp;
    h->nx = sp->nx;
    h->ny = sp->ny;
    h->nz = sp->nz;
    h->nxh = sp->nxh;
    h->dz = dz;
    int rc = pade_cd06stagg_init_periodic(&h->stagg, h->nz, dz);
    if (rc != PS_OK) {
        delete h;
        return rc;
    }
    std::vector<double> k1 = wavenums(h->nx, dx), k2 = wavenums(h->ny, dy), k3 = wavenums(h->nz, dz);
    k1.resize(h->nxh);
    h->k3mod.resize(h->nz);
    modk_cd06stagg(k3.data(), h->nz, dz, h->k3mod.data());
    rc = upload(&h->d_k1r, k1);
    if (rc == PS_OK) rc = upload(&h->d_k2r, k2);
    if (rc == PS_OK) rc = upload(&h->d_k3m, h->k3mod);
    const size_t plane = (size_t)h->nxh * h->ny;
    if (rc == PS_OK) rc = dalloc((void**)&h->f2d, sizeof(double2) * plane * h->nz);
    if (rc == PS_OK) rc = dalloc((void**)&h->dwE, sizeof(double2) * plane * (h->nz + 1));
    if (rc == PS_OK) rc = dalloc((void**)&h->part, sizeof(double) * kMaxPartials);
    if (rc == PS_OK) rc = fft_df_mult_table(FK_PROJECT, h->d_k1r, h->d_k2r, h->d_k3m, h->nxh, h->ny, h->nz, &h->d_mtab,
                                            nullptr);
    if (rc == PS_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) rc = PS_ECUDA;
    if (rc != PS_OK) {
        pade_poisson_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_poisson_wall_init(pade_poisson* out, pade_spectral sp, double dx, double dy, double dz, double Lz,
                           int compute_stokes_pressure) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    if (!sp || !(dx > 0) || !(dy > 0) || !(dz > 0)) return PS_EINVAL;
    if (compute_stokes_pressure && !(Lz > 0)) return PS_EINVAL;
    if (!pow2_len(sp->nz) || !pow2_len(2 * sp->nz)) return PS_ENOTSUP;
    auto* h = new pade_poisson_s();
    h->sp = sp;
    h->nx = sp->nx;
    h->ny = sp->ny;
    h->nz = sp->nz;
    h->nxh = sp->nxh;
    h->dz = dz;
    h->periodic = 0;
    h->stokes = compute_stokes_pressure ? 1 : 0;
    // DivergenceCheck's derivZ%ddz_E2C(.., -1, -1): the odd-odd staggered operator
    int rc = pade_cd06stagg_init_nonperiodic(&h->stagg, h->nz, dz, 0, 0, 0, 0);
    if (rc == PS_OK) rc = wall_setup(h, dx, dy, dz, Lz);
    const size_t plane = (size_t)h->nxh * h->ny;
    if (rc == PS_OK) rc = dalloc((void**)&h->f2d, sizeof(double2) * plane * h->nz);
    if (rc == PS_OK) rc = dalloc((void**)&h->part, sizeof(double) * kMaxPartials);
    if (rc != PS_OK) {
        pade_poisson_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_poisson_destroy(pade_poisson h) {
    if (!h) return PS_OK;
    if (h->stagg) pade_destroy(h->stagg);
    void* bufs[] = {h->d_k1r, h->d_k2r, h->d_k3m, h->f2d, h->dwE, h->part, h->d_k3e, h->d_k3mc, h->d_k3mp,
                    h->fext, h->wext, h->d_den, h->d_coshb, h->d_cosht, h->d_sinhb, h->d_sinht, h->d_chats,
                    h->su, h->sv, h->sw, h->d_mtab};
    for (void* b : bufs) cudaFree(b);
    delete h;
    return PS_OK;
}

int pade_poisson_get_modified_k3(pade_poisson h, double* k3mod) {
    if (!h || !k3mod) return PS_EINVAL;
    if (!h->periodic) return PS_ENOTSUP;
    for (int k = 0; k < h->nz; k++) k3mod[k] = h->k3mod[k];
    return PS_OK;
}

int pade_poisson_projection(pade_poisson h, void* uhat, void* vhat, void* what, void* stream) {
    if (!h || !device_ptr(uhat) || !device_ptr(vhat) || !device_ptr(what)) return PS_EINVAL;
    return projection(h, uhat, vhat, what, static_cast<cudaStream_t>(stream));
}

int pade_poisson_divergence_check(pade_poisson h, void* uhat, void* vhat, void* what, double* div, int fix_div,
                                  double* maxdiv, void* stream) {
    if (!h || !device_ptr(uhat) || !device_ptr(vhat) || !device_ptr(what) || !device_ptr(div)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = divergence(h, uhat, vhat, what, div, s);
    if (rc != PS_OK) return rc;
    const long n = (long)h->nx * h->ny * h->nz;
    if (!fix_div) {
        if (!maxdiv) return PS_OK;
        return max_of(h, div, n, maxdiv, s);
    }
    double m = 0;
    if ((rc = max_of(h, div, n, &m, s)) != PS_OK) return rc;
    if (m > 1e-13) {  // PadePoisson.F90:1206-1238
        if ((rc = projection(h, uhat, vhat, what, s)) != PS_OK) return rc;
        if ((rc = divergence(h, uhat, vhat, what, div, s)) != PS_OK) return rc;
        if ((rc = max_of(h, div, n, &m, s)) != PS_OK) return rc;
        if (m > 1e-10 && (rc = projection(h, uhat, vhat, what, s)) != PS_OK) return rc;
    }
    if (maxdiv) *maxdiv = m;
    return PS_OK;
}

int pade_poisson_get_pressure(pade_poisson h, const void* uhat, const void* vhat, const void* what, double* pressure,
                              void* stream) {
    if (!h || !device_ptr(uhat) || !device_ptr(vhat) || !device_ptr(what) || !device_ptr(pressure)) return PS_EINVAL;
    return get_pressure(h, const_cast<void*>(uhat), const_cast<void*>(vhat), const_cast<void*>(what), pressure, 0,
                        static_cast<cudaStream_t>(stream));
}

int pade_poisson_get_pressure_and_update_rhs(pade_poisson h, void* uhat, void* vhat, void* what, double* pressure,
                                             void* stream) {
    if (!h || !device_ptr(uhat) || !device_ptr(vhat) || !device_ptr(what) || !device_ptr(pressure)) return PS_EINVAL;
    return get_pressure(h, uhat, vhat, what, pressure, 1, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------- PoissonPeriodic
int pade_poisson3d_init(pade_poisson3d* out, int nx, int ny, int nz, double dx, double dy, double dz, int dir_id,
                        pade_modk_fn modkx, pade_modk_fn modky, pade_modk_fn modkz) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    if (dir_id < 1 || dir_id > 3) return PS_EINVAL;  // PoissonPeriodic.F90:167
    if (!(dx > 0) || !(dy > 0) || !(dz > 0)) return PS_EINVAL;
    if (!pow2_len(nx) || !pow2_len(ny) || !pow2_len(nz)) return PS_ENOTSUP;
    auto* h = new pade_poisson3d_s();
    h->nx = nx;
    h->ny = ny;
    h->nz = nz;
    h->nxh = nx / 2 + 1;
    h->dir_id = dir_id;
    h->kx = wavenums(nx, dx);
    h->kx.resize(h->nxh);
    h->ky = wavenums(ny, dy);
    h->kz = wavenums(nz, dz);
    // modified wavenumbers act on k*d (PoissonPeriodic.F90:183-199)
    struct {
        std::vector<double>* k;
        double d;
        pade_modk_fn fn;
    } mods[3] = {{&h->kx, dx, modkx}, {&h->ky, dy, modky}, {&h->kz, dz, modkz}};
    for (auto& m : mods) {
        if (!m.fn) continue;
        for (double& v : *m.k) v = v * m.d;
        m.fn(m.k->data(), (int)m.k->size());
        for (double& v : *m.k) v = v / m.d;
    }
    int rc = upload(&h->d_kx, h->kx);
    if (rc == PS_OK) rc = upload(&h->d_ky, h->ky);
    if (rc == PS_OK) rc = upload(&h->d_kz, h->kz);
    if (rc == PS_OK) rc = dalloc((void**)&h->hat, sizeof(double2) * (size_t)h->nxh * ny * nz);
    if (rc == PS_OK) rc = fft_df_mult_table(FK_POISSON3D, h->d_kx, h->d_ky, h->d_kz, h->nxh, ny, nz, &h->d_mtab, nullptr);
    if (rc == PS_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) rc = PS_ECUDA;
    if (rc != PS_OK) {
        pade_poisson3d_destroy(h);
        return rc;
    }
    *out = h;
    return PS_OK;
}

int pade_poisson3d_destroy(pade_poisson3d h) {
    if (!h) return PS_OK;
    cudaFree(h->d_kx);
    cudaFree(h->d_ky);
    cudaFree(h->d_kz);
    cudaFree(h->hat);
    cudaFree(h->d_mtab);
    delete h;
    return PS_OK;
}

int pade_poisson3d_solve(pade_poisson3d h, const double* rhs, double* f, void* stream) {
    if (!h || !device_ptr(rhs) || !device_ptr(f)) return PS_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nx = h->nx, ny = h->ny, nz = h->nz, nxh = h->nxh;
    FftExtra ex{};
    FftLines lx = fft_lines(1, nx, ny, nz, nx, nxh);
    int rc = fft_launch(IN_REAL, OUT_HALF, FK_PLAIN, nx, -1, 1.0, 0, rhs, h->hat, lx, ex, s);
    if (rc != PS_OK) return rc;
    FftLines ly = fft_lines(2, nxh, ny, nz, ny, ny);
    if ((rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, ny, -1, 1.0, 0, h->hat, h->hat, ly, ex, s)) != PS_OK)
        return rc;
    ex.ka = h->d_kx;
    ex.kb = h->d_ky;
    ex.kc = h->d_kz;
    ex.nxh = nxh;
    ex.plane = (long)nxh * ny;
    ex.mtab = h->d_mtab;
    FftLines lz = fft_lines(3, nxh, ny, nz, nz, nz);
    if ((rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_POISSON3D, nz, -1, 1.0, 0, h->hat, h->hat, lz, ex, s)) != PS_OK)
        return rc;
    ex = FftExtra{};
    if ((rc = fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, ny, 1, 1.0, 0, h->hat, h->hat, ly, ex, s)) != PS_OK)
        return rc;
    FftLines lxb = fft_lines(1, nx, ny, nz, nxh, nx);
    const double norm = 1.0 / ((double)nx * (double)ny * (double)nz);  // fft_3d.F90:360
    return fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, nx, 1, norm, 0, h->hat, f, lxb, ex, s);
}

// ---------------------------------------------------------------- FFT building blocks
int pade_fft_c2c(int dir, int sign, const void* in, void* out, int n1, int n2, int n3, double scale, void* stream) {
    if (dir < 1 || dir > 3 || (sign != -1 && sign != 1) || n1 < 1 || n2 < 1 || n3 < 1) return PS_EINVAL;
    if (!device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    const long n = dir == 1 ? n1 : (dir == 2 ? n2 : n3);
    FftLines ls = fft_lines(dir, n1, n2, n3, n, n);
    return fft_launch(IN_COMPLEX, OUT_COMPLEX, FK_PLAIN, (int)n, sign, scale, 0, in, out, ls, FftExtra{},
                      static_cast<cudaStream_t>(stream));
}

int pade_fft_r2c_x(const double* in, void* out, int nx, int ny, int nz, void* stream) {
    if (nx < 2 || ny < 1 || nz < 1 || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    FftLines ls = fft_lines(1, nx, ny, nz, nx, nx / 2 + 1);
    return fft_launch(IN_REAL, OUT_HALF, FK_PLAIN, nx, -1, 1.0, 0, in, out, ls, FftExtra{},
                      static_cast<cudaStream_t>(stream));
}

int pade_fft_c2r_x(const void* in, double* out, int nx, int ny, int nz, double scale, void* stream) {
    if (nx < 2 || ny < 1 || nz < 1 || !device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    FftLines ls = fft_lines(1, nx, ny, nz, nx / 2 + 1, nx);
    return fft_launch(IN_HALF, OUT_REAL, FK_PLAIN, nx, 1, scale, 0, in, out, ls, FftExtra{},
                      static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------- FFT arithmetic
int pade_fft_set_arith(int arith) {
    if (arith != PADE_FFT_DF && arith != PADE_FFT_FP64) return PS_EINVAL;
    fft_set_arith(arith == PADE_FFT_FP64 ? FFT_ARITH_FP64 : FFT_ARITH_DF);
    return PS_OK;
}

int pade_fft_get_arith(void) { return fft_get_arith() == FFT_ARITH_FP64 ? PADE_FFT_FP64 : PADE_FFT_DF; }

// ---------------------------------------------------------------- pencil transposes
int pade_transpose(int from_pencil, int to_pencil, const void* in, void* out, int n1, int n2, int n3,
                   int elem_bytes, void* stream) {
    if (from_pencil < 1 || from_pencil > 3 || to_pencil < 1 || to_pencil > 3) return PS_EINVAL;
    if (from_pencil == to_pencil || (from_pencil == 1 && to_pencil == 3) || (from_pencil == 3 && to_pencil == 1))
        return PS_EINVAL;  // 2DECOMP provides x<->y and y<->z only
    if (n1 < 1 || n2 < 1 || n3 < 1 || (elem_bytes != 8 && elem_bytes != 16)) return PS_EINVAL;
    if (!device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    const size_t bytes = (size_t)n1 * n2 * n3 * elem_bytes;
    if (in == out) return PS_OK;
    return cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)) ==
                   cudaSuccess
               ? PS_OK
               : PS_ECUDA;
}

}  // extern "C"
