// padepoisson with walls at z = 0 and z = Lz (PeriodicInZ false; PadePoisson.F90:130-318
// init, 434-624 PressureProjection, 320-384 ProjectStokesPressure).
//
// The pressure is solved on the even extension of the divergence and the odd extension of
// w to 2 nz points along z, where the staggered CD06 derivative is diagonal: i k3mod
// exp(-+ i k3 dz / 2) from edges to centres and back.  Device work per projection: the
// optional Stokes-pressure wall correction (one thread per (kx, ky) column, walking z),
// one extension pass, two forward z transforms of length 2 nz (the library FFT), one
// pointwise pass (pressure and w projection), two backward transforms, one restriction
// pass that also updates uhat and vhat.  The extension arrays are 2 x (nx/2+1) ny 2 nz
// complex values (the reference holds the same two arrays).
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <vector>

#include "spectral_internal.h"

namespace pade {
namespace {

constexpr int PS_OK_ = 0;

// Stokes-pressure correction of both walls: bottom (chat = -w(z=0) / (lambda sinh(lambda
// Lz))) then top from the corrected w(z=Lz) (ProjectStokesPressure 331-381)
__global__ void k_wall_stokes(double2* __restrict__ u, double2* __restrict__ v, double2* __restrict__ w,
                              const double* __restrict__ k1, const double* __restrict__ k2,
                              const double* __restrict__ den, const double* __restrict__ coshb,
                              const double* __restrict__ cosht, const double* __restrict__ sinhb,
                              const double* __restrict__ sinht, double2* __restrict__ chats, int nxh, long plane,
                              int nz) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= plane) return;
    const double a = k1[q % nxh], b = k2[q / nxh], d = den[q];
    double2 c = make_double2(-w[q].x * d, -w[q].y * d);
    chats[q] = c;
    for (int k = 0; k < nz; k++) {
        const long e = q + k * plane;
        const double cb = coshb[e];
        const double2 ph = make_double2(-c.y * cb, c.x * cb);  // i chat cosh
        u[e].x -= a * ph.x;
        u[e].y -= a * ph.y;
        v[e].x -= b * ph.x;
        v[e].y -= b * ph.y;
    }
    w[q] = make_double2(0.0, 0.0);
    for (int k = 1; k <= nz; k++) {
        const long e = q + k * plane;
        const double sb = sinhb[e];
        w[e].x -= c.x * sb;
        w[e].y -= c.y * sb;
    }
    const long top = q + nz * plane;
    c = make_double2(w[top].x * d, w[top].y * d);
    chats[plane + q] = c;
    for (int k = 0; k < nz; k++) {
        const long e = q + k * plane;
        const double ct = cosht[e], st = sinht[e];
        const double2 ph = make_double2(-c.y * ct, c.x * ct);
        u[e].x -= a * ph.x;
        u[e].y -= a * ph.y;
        v[e].x -= b * ph.x;
        v[e].y -= b * ph.y;
        w[e].x -= c.x * st;
        w[e].y -= c.y * st;
    }
    w[top] = make_double2(0.0, 0.0);
}

// even extension of i (k1 u + k2 v) and odd extension of w (PressureProjection 476-510)
__global__ void k_wall_extend(const double2* __restrict__ u, const double2* __restrict__ v,
                              const double2* __restrict__ w, const double* __restrict__ k1,
                              const double* __restrict__ k2, double2* __restrict__ fext, double2* __restrict__ wext,
                              int nxh, long plane, int nz) {
    const long n = plane * 2 * nz;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long q = e % plane;
        const int kk = (int)(e / plane);
        const double a = k1[q % nxh], b = k2[q / nxh];
        const long src = q + (long)(kk < nz ? nz - 1 - kk : kk - nz) * plane;
        const double dx = a * u[src].x + b * v[src].x, dy = a * u[src].y + b * v[src].y;
        fext[e] = make_double2(-dy, dx);
        if (kk < nz - 1) {
            const double2 t = w[q + (long)(nz - 1 - kk) * plane];
            wext[e] = make_double2(-t.x, -t.y);
        } else {
            wext[e] = w[q + (long)(kk - (nz - 1)) * plane];
        }
    }
}

// F = -(F + i k3mc W) / |k|^2, then W -= i k3mp F (PressureProjection 518-536)
__global__ void k_wall_solve(double2* __restrict__ F, double2* __restrict__ W, const double* __restrict__ k1,
                             const double* __restrict__ k2, const double* __restrict__ k3,
                             const double2* __restrict__ k3mc, const double2* __restrict__ k3mp, int nxh, long plane,
                             int nze) {
    const long n = plane * nze;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long q = e % plane;
        const int kk = (int)(e / plane);
        const double a = k1[q % nxh], b = k2[q / nxh], c3 = k3[kk];
        const double kr = a * a + b * b + c3 * c3;
        const double kinv = kr <= 1e-14 ? 0.0 : 1.0 / kr;
        const double2 wv = W[e], cm = k3mc[kk], cp = k3mp[kk];
        const double2 icm = make_double2(-cm.y, cm.x);  // i k3mc
        double fx = F[e].x + (icm.x * wv.x - icm.y * wv.y);
        double fy = F[e].y + (icm.x * wv.y + icm.y * wv.x);
        fx = -fx * kinv;
        fy = -fy * kinv;
        F[e] = make_double2(fx, fy);
        const double2 icp = make_double2(-cp.y, cp.x);  // i k3mp
        W[e] = make_double2(wv.x - (icp.x * fx - icp.y * fy), wv.y - (icp.x * fy + icp.y * fx));
    }
}

// pressure p = F(nz + k) (already times 1/(2 nz)): u -= i k1 p, v -= i k2 p; w = W(nz - 1 + k)
// with both wall values zero (PressureProjection 539-615)
__global__ void k_wall_restrict(const double2* __restrict__ F, const double2* __restrict__ W,
                                double2* __restrict__ u, double2* __restrict__ v, double2* __restrict__ w,
                                const double* __restrict__ k1, const double* __restrict__ k2, int nxh, long plane,
                                int nz) {
    const long n = plane * (nz + 1);
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long q = e % plane;
        const int k = (int)(e / plane);
        if (k < nz) {
            const double a = k1[q % nxh], b = k2[q / nxh];
            const double2 p = F[q + (long)(nz + k) * plane];
            u[e].x -= -a * p.y;
            u[e].y -= a * p.x;
            v[e].x -= -b * p.y;
            v[e].y -= b * p.x;
        }
        w[e] = (k == 0 || k == nz) ? make_double2(0.0, 0.0) : W[q + (long)(nz - 1 + k) * plane];
    }
}

// the pressure of the projection, p(k) = F(nz + k) (times 1/(2 nz) already), plus the
// Stokes pressure i chat_bot cosh_bot + i chat_top cosh_top (getPressure 862-871)
__global__ void k_wall_pressure(const double2* __restrict__ F, const double2* __restrict__ chats,
                                const double* __restrict__ coshb, const double* __restrict__ cosht,
                                double2* __restrict__ p, long plane, int nz) {
    const long n = plane * nz;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long q = e % plane;
        const int k = (int)(e / plane);
        double2 v = F[q + (long)(nz + k) * plane];
        if (chats) {
            const double2 cb = chats[q], ct = chats[plane + q];
            const double hb = coshb[e], ht = cosht[e];
            v.x = (v.x + (-cb.y * hb)) + (-ct.y * ht);
            v.y = (v.y + cb.x * hb) + ct.x * ht;
        }
        p[e] = v;
    }
}

}  // namespace

int wall_pressure(pade_poisson h, cudaStream_t s) {
    const long plane = (long)h->nxh * h->ny;
    k_wall_pressure<<<grid_for(plane * h->nz), 256, 0, s>>>(h->fext, h->stokes ? h->d_chats : nullptr, h->d_coshb,
                                                            h->d_cosht, h->f2d, plane, h->nz);
    return cudaGetLastError() == cudaSuccess ? PS_OK_ : PADE_ECUDA;
}

int wall_setup(pade_poisson h, double dx, double dy, double dz, double Lz) {
    const int nxh = h->nxh, ny = h->ny, nz = h->nz, nze = 2 * nz;
    std::vector<double> k1r = wavenums(h->nx, dx), k2r = wavenums(ny, dy), k3 = wavenums(nze, dz);
    k1r.resize(nxh);
    std::vector<double> k3mod(nze);
    modk_cd06stagg(k3.data(), nze, dz, k3mod.data());
    std::vector<double2> cm(nze), cp(nze);
    for (int k = 0; k < nze; k++) {
        const std::complex<double> tfm = std::exp(std::complex<double>(0.0, -dz / 2.0 * k3[k]));
        const std::complex<double> tfp = std::exp(std::complex<double>(0.0, dz / 2.0 * k3[k]));
        cm[k] = make_double2(k3mod[k] * tfm.real(), k3mod[k] * tfm.imag());
        cp[k] = make_double2(k3mod[k] * tfp.real(), k3mod[k] * tfp.imag());
    }
    int rc = upload(&h->d_k1r, k1r);
    if (rc == PS_OK_) rc = upload(&h->d_k2r, k2r);
    if (rc == PS_OK_) rc = upload(&h->d_k3e, k3mod);
    if (rc == PS_OK_) rc = upload(&h->d_k3mc, cm);
    if (rc == PS_OK_) rc = upload(&h->d_k3mp, cp);
    const size_t plane = (size_t)nxh * ny;
    if (rc == PS_OK_) rc = dalloc((void**)&h->fext, sizeof(double2) * plane * nze);
    if (rc == PS_OK_) rc = dalloc((void**)&h->wext, sizeof(double2) * plane * nze);
    if (rc != PS_OK_ || !h->stokes) return rc;
    rc = dalloc((void**)&h->d_chats, sizeof(double2) * plane * 2);
    if (rc != PS_OK_) return rc;
    // Stokes-pressure tables (init 235-306), with the reference's overflow guards
    std::vector<double> den(plane), cb(plane * nz), ct(plane * nz), sb(plane * (nz + 1)), st(plane * (nz + 1));
    std::vector<double> zE(nz + 1), zC(nz);
    for (int k = 0; k <= nz; k++) zE[k] = Lz * (double)k / (double)nz;
    for (int k = 0; k < nz; k++) zC[k] = 0.5 * (zE[k] + zE[k + 1]);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nxh; i++) {
            const size_t q = (size_t)j * nxh + i;
            const double lam = std::sqrt(k1r[i] * k1r[i] + k2r[j] * k2r[j]);
            double d = lam * Lz < 500.0 ? 1.0 / (lam * std::sinh(lam * Lz) + 1e-13) : 0.0;
            if (d < 1e-16) d = 0.0;
            if (q == 0) d = 0.0;
            den[q] = d;
            for (int k = 0; k < nz; k++) {
                double t = lam * (Lz - zC[k]);
                cb[q + k * plane] = t < 32.0 ? std::cosh(t) : 4e13;
                t = lam * zC[k];
                ct[q + k * plane] = t < 32.0 ? std::cosh(t) : 1e13;
            }
            for (int k = 0; k <= nz; k++) {
                double t = lam * (Lz - zE[k]);
                sb[q + k * plane] = t < 32.0 ? -lam * std::sinh(t) : -4e13;
                t = lam * zE[k];
                st[q + k * plane] = t < 32.0 ? lam * std::sinh(t) : 4e13;
            }
        }
    rc = upload(&h->d_den, den);
    if (rc == PS_OK_) rc = upload(&h->d_coshb, cb);
    if (rc == PS_OK_) rc = upload(&h->d_cosht, ct);
    if (rc == PS_OK_) rc = upload(&h->d_sinhb, sb);
    if (rc == PS_OK_) rc = upload(&h->d_sinht, st);
    return rc;
}

int wall_projection(pade_poisson h, void* uhat, void* vhat, void* what, cudaStream_t s) {
    const int nxh = h->nxh, ny = h->ny, nz = h->nz, nze = 2 * nz;
    const long plane = (long)nxh * ny;
    double2* u = static_cast<double2*>(uhat);
    double2* v = static_cast<double2*>(vhat);
    double2* w = static_cast<double2*>(what);
    // the Stokes-pressure path uses GetWaveNums' k1, k2 throughout; otherwise the spectral
    // type's (PressureProjection 445-470, 583-616)
    const double* k1 = h->stokes ? h->d_k1r : h->sp->d_k1;
    const double* k2 = h->stokes ? h->d_k2r : h->sp->d_k2;
    if (h->stokes) {
        k_wall_stokes<<<(unsigned)((plane + 127) / 128), 128, 0, s>>>(u, v, w, h->d_k1r, h->d_k2r, h->d_den, h->d_coshb,
                                                                     h->d_cosht, h->d_sinhb, h->d_sinht, h->d_chats,
                                                                     nxh, plane, nz);
        if (cudaGetLastError() != cudaSuccess) return PADE_ECUDA;
    }
    k_wall_extend<<<grid_for(plane * nze), 256, 0, s>>>(u, v, w, k1, k2, h->fext, h->wext, nxh, plane, nz);
    if (cudaGetLastError() != cudaSuccess) return PADE_ECUDA;
    int rc = pade_fft_c2c(3, -1, h->fext, h->fext, nxh, ny, nze, 1.0, s);
    if (rc == PS_OK_) rc = pade_fft_c2c(3, -1, h->wext, h->wext, nxh, ny, nze, 1.0, s);
    if (rc != PS_OK_) return rc;
    k_wall_solve<<<grid_for(plane * nze), 256, 0, s>>>(h->fext, h->wext, h->d_k1r, h->d_k2r, h->d_k3e, h->d_k3mc,
                                                       h->d_k3mp, nxh, plane, nze);
    if (cudaGetLastError() != cudaSuccess) return PADE_ECUDA;
    const double mfact = 1.0 / (double)nze;
    rc = pade_fft_c2c(3, 1, h->fext, h->fext, nxh, ny, nze, mfact, s);
    if (rc == PS_OK_) rc = pade_fft_c2c(3, 1, h->wext, h->wext, nxh, ny, nze, mfact, s);
    if (rc != PS_OK_) return rc;
    k_wall_restrict<<<grid_for(plane * (nz + 1)), 256, 0, s>>>(h->fext, h->wext, u, v, w, k1, k2, nxh, plane, nz);
    return cudaGetLastError() == cudaSuccess ? PS_OK_ : PADE_ECUDA;
}

}  // namespace pade
