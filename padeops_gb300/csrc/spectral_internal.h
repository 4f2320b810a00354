// Internal definitions shared by spectral.cu and les.cu.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/padeops_gb300.h"

struct pade_spectral_s {
    int nx = 0, ny = 0, nz = 0, nxh = 0;
    double dx = 0, dy = 0;
    int fix_oddball = 1;
    std::vector<double> k1, k2;
    double* d_k1 = nullptr;
    double* d_k2 = nullptr;
    double2* work = nullptr;  // (nxh, ny, nz): the ifft's y-transform output
    double2* work2 = nullptr; // (nxh, ny, nz): second y-transform output of pade_spectral_ifft_two (on first use)
};

struct pade_poisson_s {
    pade_spectral sp = nullptr;
    int nx = 0, ny = 0, nz = 0, nxh = 0;
    double dz = 0;
    pade_op stagg = nullptr;
    std::vector<double> k3mod;
    double* d_k1r = nullptr;   // GetWaveNums(nx, dx)(1:nx/2+1)
    double* d_k2r = nullptr;   // GetWaveNums(ny, dy)
    double* d_k3m = nullptr;   // CD06-stagg modified z wavenumbers
    double2* f2d = nullptr;    // (nxh, ny, nz): dwdz, then the pressure
    double2* dwE = nullptr;    // (nxh, ny, nz+1)
    double* part = nullptr;    // kMaxPartials
    double* d_mtab = nullptr;  // periodic: the fused z kernel's -1/|k|^2 per (line, position)
    // walls at z = 0 and Lz (PeriodicInZ false): stagg is then the odd-odd operator
    int periodic = 1, stokes = 0;
    double* d_k3e = nullptr;    // CD06-stagg modified wavenumbers of the 2 nz extension
    double2* d_k3mc = nullptr;  // k3mod exp(-i dz k3 / 2)
    double2* d_k3mp = nullptr;  // k3mod exp(+i dz k3 / 2)
    double2* fext = nullptr;    // (nxh, ny, 2 nz)
    double2* wext = nullptr;    // (nxh, ny, 2 nz)
    double* d_den = nullptr;    // Stokes pressure: 1 / (lambda sinh(lambda Lz)) (nxh, ny)
    double* d_coshb = nullptr;  // (nxh, ny, nz)
    double* d_cosht = nullptr;  // (nxh, ny, nz)
    double* d_sinhb = nullptr;  // (nxh, ny, nz + 1)
    double* d_sinht = nullptr;  // (nxh, ny, nz + 1)
    double2* d_chats = nullptr; // Stokes pressure coefficients of the last projection (2 x nxh x ny)
    double2* su = nullptr;      // getPressure: copies of its inputs (allocated on first use)
    double2* sv = nullptr;
    double2* sw = nullptr;
};

struct pade_poisson3d_s {
    int nx = 0, ny = 0, nz = 0, nxh = 0, dir_id = 1;
    std::vector<double> kx, ky, kz;
    double* d_kx = nullptr;
    double* d_ky = nullptr;
    double* d_kz = nullptr;
    double2* hat = nullptr;  // (nxh, ny, nz)
    double* d_mtab = nullptr;  // the fused z kernel's multiplier per (line, position)
};

namespace pade {

constexpr int kMaxPartials = 152 * 8;

std::vector<double> wavenums(int n, double dx);
void modk_cd06stagg(const double* k, int n, double dx, double* kp);
bool device_ptr(const void* p);

// Pade6stagg's Fourier-collocation z operators (fourier_coll.cu): op in Pade6stagg order
// (0 ddz_C2E, 1 ddz_E2C, 2 interpz_C2E, 3 interpz_E2C, 4 d2dz2_C2C, 5 d2dz2_E2E) on device
// arrays of (n1, n2) lines; nz a power of two (PADE_ENOTSUP otherwise)
struct FourierColl;
int fourier_coll_create(int nz, double dz, FourierColl** out);
void fourier_coll_destroy(FourierColl* fc);
int fourier_coll_apply(FourierColl* fc, int op, int cplx, const double* in, double* out, int n1, int n2,
                       cudaStream_t s);
unsigned grid_for(long n);
int dalloc(void** p, size_t bytes);
// copy a host vector into a new device array
template <typename T>
int upload(T** d, const std::vector<T>& h) {
    if (cudaMalloc(d, sizeof(T) * (h.empty() ? 1 : h.size())) != cudaSuccess) {
        cudaGetLastError();
        *d = nullptr;
        return 1002;  // PADE_ENOMEM
    }
    if (!h.empty() && cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return 1003;  // PADE_ECUDA
    return 0;
}

// spectral fft (r2c x, c2c y) and ifft (c2c y with optional i*k pre-multiplication
// (FftMul) of the spectral input, oddball, c2r x, 1/(nx ny))
int spectral_fft(pade_spectral h, const double* in, void* out, cudaStream_t s);
int spectral_ifft(pade_spectral h, const void* in, double* out, int oddball, cudaStream_t s, int mul = 0);
// walled padepoisson (poisson_wall.cu): tables of init, and PressureProjection
int wall_setup(pade_poisson h, double dx, double dy, double dz, double Lz);
int wall_projection(pade_poisson h, void* uhat, void* vhat, void* what, cudaStream_t s);
// the pressure of the last walled projection (plus its Stokes pressure) into f2d
int wall_pressure(pade_poisson h, cudaStream_t s);
// out = ifft2(in) and out_dx = ifft2(i k1 in) from one y transform (oddball 0)
int spectral_ifft_pair(pade_spectral h, const void* in, double* out, double* out_dx, cudaStream_t s);
// out1 = fft2(in1), out2 = fft2(in2); the two x transforms in one launch where the paired
// kernel applies
int spectral_fft_two(pade_spectral h, const double* in1, const double* in2, void* out1, void* out2, cudaStream_t s);
// out1 = ifft2(in1 [times i k: mul1]) and out2 = ifft2(in2 [mul2]) (oddball 0), the y
// transforms into w1 and w2 (which may be in1 and in2: those are then overwritten), the two
// x transforms in one launch where the paired kernel applies
int spectral_ifft_two(pade_spectral h, const void* in1, int mul1, const void* in2, int mul2, double* out1,
                      double* out2, void* w1, void* w2, cudaStream_t s);
// ifft of fhat * G, G = 1 where |k1| < cut1 and |k2| < cut2 (the test filter's TestFilter_oop)
int spectral_ifft_masked(pade_spectral h, const void* in, double* out, double cut1, double cut2, cudaStream_t s);

// Learned closure inside the LES (mlp.cu, called by les.cu): points whose features leave
// the training range (pade_mlp_set_range), or every point while *all is nonzero, take the
// fallback coefficient Cs^2 Delta^2 = lam[z plane] instead of the network's.
struct MlpFallback {
    const double* lam;          // per z plane; null: no fallback
    long plane;                 // points per z plane
    const int* all;             // device flag (may be null)
    unsigned long long* count;  // device counter of the points given the fallback (may be null)
};
int mlp_infer_nu_fb(pade_mlp h, const double* const* duidxj, long n, double delta, double nu, double* nu_out,
                    float* cs2_out, const MlpFallback& fb, cudaStream_t s);

}  // namespace pade
