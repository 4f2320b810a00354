// Pade6stagg's Fourier-collocation scheme in z (PadeDerOps.F90 scheme fourierColl), i.e. the
// spectral layer's periodic-z operators (src/incompressible/spectral.F90:365-700, factors of
// its init 843-856): each line along z is transformed, multiplied per mode and transformed
// back with 1/nz.
//   ddz_C2E: i k e^{-i k dz/2}    ddz_E2C: i k e^{+i k dz/2}    d2dz2_C2C / d2dz2_E2E: -k^2
//   interpz_C2E:   e^{-i k dz/2}  interpz_E2C:   e^{+i k dz/2}
// with k = GetWaveNums(nz, dz).  Real arrays go through r2c / c2r, where the reference
// multiplies modes 0 .. nz/2 - 1 only (the Nyquist mode passes unchanged); complex arrays
// through c2c, every mode multiplied.  Edge inputs use their first nz planes; edge outputs
// repeat plane 0 as plane nz.  Device pointers only, like the spectral layer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "fft.h"
#include "operators.h"
#include "spectral_internal.h"

namespace pade {

struct FourierColl {
    int nz = 0;
    double dz = 1.0;
    double2* fac = nullptr;  // 6 x nz per-mode factors (Pade6stagg operation order)
    double2* work = nullptr;
    size_t work_elems = 0;
    ~FourierColl() {
        cudaFree(fac);
        cudaFree(work);
    }
};

namespace {

// modes [0, nmul) of every line (point stride `plane` complex elements) times fac[mode]
__global__ void k_mode_mul(double2* __restrict__ x, const double2* __restrict__ fac, long plane, int nmul) {
    const long n = plane * nmul;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int k = (int)(e / plane);
        const double2 a = x[e], f = fac[k];
        x[e] = make_double2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
    }
}

bool pow2(int n) { return n >= 2 && n <= 8192 && (n & (n - 1)) == 0; }

}  // namespace

int fourier_coll_create(int nz, double dz, FourierColl** out) {
    if (!out) return PS_EINVAL;
    *out = nullptr;
    if (!(dz > 0.0)) return PS_EINVAL;
    if (!pow2(nz)) return PS_ENOTSUP;
    std::vector<double> k(nz);
    const int rc = pade_wavenumbers(nz, dz, k.data());
    if (rc != PS_OK) return rc;
    std::vector<double2> h(6 * (size_t)nz);
    const std::complex<double> I(0.0, 1.0);
    for (int m = 0; m < nz; m++) {
        const std::complex<double> em = std::exp(-I * k[m] * dz / 2.0), ep = std::exp(I * k[m] * dz / 2.0);
        const std::complex<double> f[6] = {I * k[m] * em, I * k[m] * ep, em, ep, -(k[m] * k[m]), -(k[m] * k[m])};
        for (int o = 0; o < 6; o++) h[(size_t)o * nz + m] = make_double2(f[o].real(), f[o].imag());
    }
    auto* fc = new FourierColl();
    fc->nz = nz;
    fc->dz = dz;
    if (cudaMalloc(&fc->fac, sizeof(double2) * h.size()) != cudaSuccess ||
        cudaMemcpy(fc->fac, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        delete fc;
        return PS_ECUDA;
    }
    *out = fc;
    return PS_OK;
}

void fourier_coll_destroy(FourierColl* fc) { delete fc; }

int fourier_coll_apply(FourierColl* fc, int op, int cplx, const double* in, double* out, int n1, int n2,
                       cudaStream_t s) {
    if (!fc || op < 0 || op > 5 || n1 < 0 || n2 < 0) return PS_EINVAL;
    if (n1 == 0 || n2 == 0) return PS_OK;
    if (!device_ptr(in) || !device_ptr(out)) return PS_EINVAL;
    const int nz = fc->nz;
    const long plane = (long)n1 * n2;
    const long half = cplx ? nz : nz / 2 + 1;
    const size_t need = (size_t)plane * half;
    if (need > fc->work_elems) {
        cudaFree(fc->work);
        fc->work = nullptr;
        fc->work_elems = 0;
        if (cudaMalloc(&fc->work, sizeof(double2) * need) != cudaSuccess) {
            cudaGetLastError();
            return PS_ENOMEM;
        }
        fc->work_elems = need;
    }
    const FftLines ls = fft_lines(3, n1, n2, nz, nz, nz);
    const FftExtra ex{};
    int rc = fft_launch(cplx ? IN_COMPLEX : IN_REAL, cplx ? OUT_COMPLEX : OUT_HALF, FK_PLAIN, nz, -1, 1.0, 0, in,
                        fc->work, ls, ex, s);
    if (rc != PS_OK) return rc;
    const int nmul = cplx ? nz : nz / 2;  // real lines: the Nyquist mode is not multiplied
    const long total = plane * nmul;
    const unsigned g = (unsigned)std::min<long>((total + 255) / 256, 152L * 16);
    k_mode_mul<<<g, 256, 0, s>>>(fc->work, fc->fac + (size_t)op * nz, plane, nmul);
    if (cudaGetLastError() != cudaSuccess) return PS_ECUDA;
    rc = fft_launch(cplx ? IN_COMPLEX : IN_HALF, cplx ? OUT_COMPLEX : OUT_REAL, FK_PLAIN, nz, 1, 1.0 / nz, 0,
                    fc->work, out, ls, ex, s);
    if (rc != PS_OK) return rc;
    const bool edges_out = op == 0 || op == 2 || op == 5;  // ddz_C2E, interpz_C2E, d2dz2_E2E
    if (edges_out) {
        const size_t bytes = sizeof(double) * (size_t)plane * (cplx ? 2 : 1);
        const char* src = reinterpret_cast<const char*>(out);
        if (cudaMemcpyAsync(reinterpret_cast<char*>(out) + (size_t)nz * bytes, src, bytes, cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess)
            return PS_ECUDA;
    }
    return PS_OK;
}

}  // namespace pade
