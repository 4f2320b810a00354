// Batched FP64 line FFTs (fft.cu) used by the spectral and Poisson layers (spectral.cu).
#pragma once
#include <cuda_runtime.h>

namespace pade {

// Lines of a 3-D array: line l has a = l % na, b = l / na and point p at
// a * fa + b * fb + p * fp (input) and a * oa + b * ob + p * op (output), in elements of
// the respective input/output type (double2 for complex, double for real).
struct FftLines {
    long nlines, na;
    long fa, fb, fp;
    long oa, ob, op;
};

enum FftIn { IN_COMPLEX = 0, IN_REAL = 1, IN_HALF = 2 };
enum FftOut { OUT_COMPLEX = 0, OUT_HALF = 1, OUT_REAL = 2 };

// What happens between loading and storing a line.
enum FftKind {
    FK_PLAIN = 0,      // one transform with the given sign
    FK_PROJECT = 1,    // PadePoisson periodic projection along z (see FftExtra)
    FK_POISSON3D = 2,  // PoissonPeriodic: forward, multiply, backward along z
    FK_DEALIAS = 3,    // spectral dealias along z: forward, 0/1 mask, backward (see FftExtra)
};

// FK_PLAIN pre-multiplication on load (mtimes_ik1 / mtimes_ik2 of spectral.F90:235-310):
// MUL_IK_A multiplies point (a, p) by i*km[a] (km indexed by the line's first index, the
// x wavenumber of a y line), MUL_IK_P by i*km[p] (the wavenumber along the line).
// MUL_MASK_AP keeps point (a, p) where |ka[a]| < cut_a and |kb[p]| < cut_b and zeroes it
// otherwise (the x-y sharp test filter on a y line).
enum FftMul { MUL_NONE = 0, MUL_IK_A = 1, MUL_IK_P = 2, MUL_MASK_AP = 3 };

// Extra operands of FK_PROJECT / FK_POISSON3D.  Lines run along z through complex
// (nxh, ny, nz) arrays: line l = i + nxh * j, point stride plane = nxh * ny.
struct FftExtra {
    const double* ka;  // per i: wavenumber entering |k|^2
    const double* kb;  // per j
    const double* kc;  // per point along the line
    const double* k1;  // FK_PROJECT: spectral wavenumbers of d/dx, d/dy (per i, per j)
    const double* k2;
    double2* u;        // FK_PROJECT: uhat, vhat, read for the divergence, updated in place
    double2* v;
    long nxh;
    long plane;
    int mul;           // FftMul (FK_PLAIN)
    const double* km;
    double cut_a, cut_b, cut_c;  // FK_DEALIAS: keep |ka| < cut_a and |kb| < cut_b and |kc| < cut_c
    int edge_copy;     // FK_DEALIAS: also store point 0 at point n (periodic edge plane)
    const double* mtab;  // FK_PROJECT / FK_POISSON3D, double-float kernel: the multiplier of
                         // each (line, bit-reversed position), fft_df_mult_table; null: computed
};

FftLines fft_lines(int dir, long n1, long n2, long n3, long in_len, long out_len);

// Launch one batched transform of length n (a power of two, 2..8192).  sign -1 is the
// forward (exp(-i...)) transform, +1 the backward one; outputs are multiplied by scale.
// oddball (IN_HALF only) zeroes the Nyquist entry before the complex-to-real transform.
int fft_launch(int in_mode, int out_mode, int kind, int n, int sign, double scale, int oddball, const void* in,
               void* out, const FftLines& ls, const FftExtra& ex, cudaStream_t s);

// The multipliers of FK_PROJECT (-1/|k|^2, 0 where |k|^2 <= 1e-14) or FK_POISSON3D
// (-1/(|k|^2 + 1e-20), 0 for the zero mode) of z lines (i, j) of nz points (a power of two),
// as the double-float kernel reads them: table[(i + nxh j) nz + q] for bit-reversed position
// q (frequency brev(q)).  Allocates *out (nxh ny nz doubles) and fills it on stream s.
int fft_df_mult_table(int kind, const double* ka, const double* kb, const double* kc, int nxh, int ny, int nz,
                      double** out, cudaStream_t s);

// out1 = c2r(X) and out2 = c2r(Y) of half-spectrum lines along x (IN_HALF -> OUT_REAL lines
// ls, n = 256, oddball 0), Y = in2 or, with in2 null, i km X; both times scale, in one
// launch.  PS_ENOTSUP where this path does not apply (other lengths, strided lines, FP64
// arithmetic): use two fft_launch.
int fft_c2r_pair(const void* in, const void* in2, double* out1, double* out2, const FftLines& ls, int n, double scale,
                 const double* km, cudaStream_t s);
int fft_c2r_pair_df(const void* in, const void* in2, double* out1, double* out2, const FftLines& ls, int n,
                    double scale, const double* km, cudaStream_t s);
// out1 = r2c(in1), out2 = r2c(in2) of real lines along x (IN_REAL -> OUT_HALF lines ls, n =
// 256), both times scale, in one launch; PS_ENOTSUP where this path does not apply.
int fft_r2c_pair(const double* in1, const double* in2, void* out1, void* out2, const FftLines& ls, int n,
                 double scale, cudaStream_t s);
int fft_r2c_pair_df(const double* in1, const double* in2, void* out1, void* out2, const FftLines& ls, int n,
                    double scale, cudaStream_t s);

// The same transform in double-float arithmetic (fft_df.cu); logn = log2(n)
int fft_launch_df(int in_mode, int out_mode, int kind, int logn, int sign, double scale, int oddball, const void* in,
                  void* out, const FftLines& ls, const FftExtra& ex, cudaStream_t s);

// Arithmetic of every transform: FFT_ARITH_DF (default) or FFT_ARITH_FP64
enum FftArith { FFT_ARITH_DF = 0, FFT_ARITH_FP64 = 1 };
void fft_set_arith(int a);
int fft_get_arith();

}  // namespace pade
