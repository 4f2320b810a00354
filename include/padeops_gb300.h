/*
 * padeops_gb300.h -- C ABI of the GB300 compact-operator library.
 *
 * Drop-in boundary for the PadeOps derivative/filter objects.  Each reference Fortran
 * type (cd06, cd10, cf90, gaussian, cd06stagg) becomes an opaque `pade_op` handle; each
 * type-bound procedure becomes one function with the same argument meaning.  A Fortran
 * shim keeps the reference's module/type names, stores the handle as type(c_ptr) and
 * calls these functions through ISO_C_BINDING (the modules under fortran/).
 *
 * Conventions
 *  - Arrays are column-major (Fortran order, x fastest), FP64, as in the reference.
 *  - Field pointers may be DEVICE pointers (the call is asynchronous on `stream`, safe
 *    to capture in a CUDA graph) or HOST pointers (the library stages the data through
 *    device memory and returns after the result is back in host memory).
 *  - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *  - Complex arrays (`*_cmplx`) are complex(rkind): interleaved (re, im) FP64 pairs.
 *  - Every function returns a status.  Positive values below 1000 are the reference's own
 *    init `ierr` / GracefulExit codes, so a shim can forward them unchanged; values from
 *    1000 up are library errors.  The library never aborts the process.
 */
#ifndef PADEOPS_GB300_H
#define PADEOPS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PADE_OK 0
#define PADE_EREF_NONPERIODIC_N 2 /* cd06/cd10 init: n < 8 (cd06.F90:181, cd10.F90:224, 270) */
#define PADE_EREF_PERIODIC_N 3    /* cd06 init periodic: n < 6 (cd06.F90:158) */
#define PADE_EREF_FILTER_N 7      /* cf90 init: n < 10 (cf90.F90:128, 166) */
#define PADE_EREF_STAGG_N 21      /* cd06stagg init: n <= 4 (cd06stagg.F90:183, 218) */
#define PADE_EREF_BC 324          /* boundary code outside {0,1,-1} (cd10.F90:2045; cf90.F90:1036) */
#define PADE_EINVAL 1001
#define PADE_ENOMEM 1002
#define PADE_ECUDA 1003
#define PADE_ENOTSUP 1004
#define PADE_ETIMEOUT 1005
#define PADE_ERANGE 1006 /* a line given to the double-float path holds an infinity or NaN */
#define PADE_ESCRATCH 1007 /* pade_apply_noalloc: a host buffer exceeds its static staging capacity */

/* ---- arithmetic paths (pade_set_path) ---- */
#define PADE_PATH_DF 0     /* default: double-float arithmetic on the FP32 pipes, FP64 in/out */
#define PADE_PATH_NATIVE 1 /* native FP64 arithmetic, one thread per line */
#define PADE_PATH_FP32 2   /* FP32 in/out (pade_apply only) */

typedef struct pade_op_s* pade_op;

/* ---- cd06: 6th-order collocated compact derivative (src/derivatives/cd06.F90) ---- */
/* replaces cd06%init(n, dx, periodic, bc1, bcn) -> ierr   (cd06.F90:129-201) */
int pade_cd06_init(pade_op* op, int n, double dx, int periodic, int bc1, int bcn);
/* replace cd06%dd1/dd2/dd3(f, df, na, nb)   (cd06.F90:775-839) */
int pade_cd06_dd1(pade_op op, const double* f, double* df, int na, int nb, void* stream);
int pade_cd06_dd2(pade_op op, const double* f, double* df, int na, int nb, void* stream);
int pade_cd06_dd3(pade_op op, const double* f, double* df, int na, int nb, void* stream);
/* periodic second derivative; upstream cd06.F90:745-773 and 492-513 leave it incomplete
 * (derivatives.F90:525 GracefulExit); here completed with 1/dx^2 and the LU2 solve.
 * Non-periodic objects return PADE_ENOTSUP like the reference's GracefulExit. */
int pade_cd06_d2d1(pade_op op, const double* f, double* df, int na, int nb, void* stream);
int pade_cd06_d2d2(pade_op op, const double* f, double* df, int na, int nb, void* stream);
int pade_cd06_d2d3(pade_op op, const double* f, double* df, int na, int nb, void* stream);

/* ---- cd10: 10th-order collocated compact derivative (src/derivatives/cd10.F90) ---- */
/* replaces cd10%init(n, dx, periodic, bc1, bcn) -> ierr   (cd10.F90:195-315) */
int pade_cd10_init(pade_op* op, int n, double dx, int periodic, int bc1, int bcn);
/* replace cd10%dd1..dd3(f, df, na, nb, bc1_, bcn_)   (cd10.F90:2029-2237);
 * the reference's omitted optional bc arguments are 0 */
int pade_cd10_dd1(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);
int pade_cd10_dd2(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);
int pade_cd10_dd3(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);
/* replace cd10%d2d1..d2d3(f, df, na, nb, bc1_, bcn_)   (cd10.F90:2239-2447) */
int pade_cd10_d2d1(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);
int pade_cd10_d2d2(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);
int pade_cd10_d2d3(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream);

/* ---- cf90: 8th-order compact filter (src/filters/cf90.F90) ---- */
/* replaces cf90%init(n, periodic) -> ierr   (cf90.F90:107-175) */
int pade_cf90_init(pade_op* op, int n, int periodic);
/* replace cf90%filter1/filter2/filter3(f, ff, na, nb, bc1_, bcn_)   (cf90.F90:1020-1228) */
int pade_cf90_filter1(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
int pade_cf90_filter2(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
int pade_cf90_filter3(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
/* replaces cf90%filter3 on complex(rkind) (cf90.F90:1230-1251); the reference always
 * solves with penta_nn here, this entry uses the factorisation of (bc1, bcn) */
int pade_cf90_filter3_cmplx(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn,
                            void* stream);

/* ---- gaussian: explicit 9-point filter of width 4 dx (src/filters/gaussian.F90) ---- */
/* replaces gaussian%init(n, periodic) -> ierr   (gaussian.F90:74-93) */
int pade_gaussian_init(pade_op* op, int n, int periodic);
/* replace gaussian%filter1/filter2/filter3 (gaussian.F90:104-582) */
int pade_gaussian_filter1(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
int pade_gaussian_filter2(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
int pade_gaussian_filter3(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream);
int pade_gaussian_filter3_cmplx(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn,
                                void* stream);

/* ---- cd06stagg: staggered 6th-order compact operators (src/derivatives/cd06stagg.F90) ---- */
/* replace the generic cd06stagg%init: init_periodic(n, dx) (cd06stagg.F90:170-195) and
 * init_nonperiodic(n, dx, isTopEven, isBotEven, isTopSided, isBotSided) (197-232) */
int pade_cd06stagg_init_periodic(pade_op* op, int n, double dx);
int pade_cd06stagg_init_nonperiodic(pade_op* op, int n, double dx, int isTopEven, int isBotEven, int isTopSided,
                                    int isBotSided);
/* replace ddz_E2C/C2E/C2C/E2E, d2dz2_C2C/E2E, InterpZ_E2C/C2E, REAL overloads
 * (cd06stagg.F90:820-1059).  Input (n1,n2,nin), output (n1,n2,nout); E = n+1 points. */
int pade_cd06stagg_ddz_E2C(pade_op op, const double* fE, double* dfC, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_C2E(pade_op op, const double* fC, double* dfE, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_C2C(pade_op op, const double* fC, double* dfC, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_E2E(pade_op op, const double* fE, double* dfE, int n1, int n2, void* stream);
int pade_cd06stagg_d2dz2_C2C(pade_op op, const double* fC, double* d2fC, int n1, int n2, void* stream);
int pade_cd06stagg_d2dz2_E2E(pade_op op, const double* fE, double* d2fE, int n1, int n2, void* stream);
int pade_cd06stagg_InterpZ_E2C(pade_op op, const double* fE, double* IfC, int n1, int n2, void* stream);
int pade_cd06stagg_InterpZ_C2E(pade_op op, const double* fC, double* IfE, int n1, int n2, void* stream);
/* CMPLX overloads of the same eight procedures (complex(rkind) arrays) */
int pade_cd06stagg_ddz_E2C_cmplx(pade_op op, const double* fE, double* dfC, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_C2E_cmplx(pade_op op, const double* fC, double* dfE, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_C2C_cmplx(pade_op op, const double* fC, double* dfC, int n1, int n2, void* stream);
int pade_cd06stagg_ddz_E2E_cmplx(pade_op op, const double* fE, double* dfE, int n1, int n2, void* stream);
int pade_cd06stagg_d2dz2_C2C_cmplx(pade_op op, const double* fC, double* d2fC, int n1, int n2, void* stream);
int pade_cd06stagg_d2dz2_E2E_cmplx(pade_op op, const double* fE, double* d2fE, int n1, int n2, void* stream);
int pade_cd06stagg_InterpZ_E2C_cmplx(pade_op op, const double* fE, double* IfC, int n1, int n2, void* stream);
int pade_cd06stagg_InterpZ_C2E_cmplx(pade_op op, const double* fC, double* IfE, int n1, int n2, void* stream);

/* ---- Pade6stagg: igrid's staggered z-operator facade (src/incompressible/PadeDerOps.F90) ----
 * replaces Pade6stagg%init(gpC, sp_gpC, gpE, sp_gpE, dz, scheme, isPeriodic) (PadeDerOps.F90:
 * 57-124) with nz = gpC%zsz(3); the x-y extents (n1, n2) of each array are given per call.
 * scheme: 1 cd06 (the compact sixth-order operators), 0 fd02 (the second-order staggered
 * operators of staggOps.F90, nz >= 3), 2 fourierColl (periodic only, as the reference: the
 * spectral layer's z operators of spectral.F90:365-700; nz a power of two, otherwise
 * PADE_ENOTSUP; device arrays only); other values return the reference's GracefulExit codes
 * 434 (periodic) / 323 (non-periodic).  Non-periodic cd06 objects hold the nine cd06stagg objects of
 * PadeDerOps.F90:92-110 and select one per call by (bot, top), each -1 (odd), 0 (one-sided)
 * or 1 (even), as PadeDerOps.F90:146-995; fd02 objects apply the per-code choices of the
 * same routines' fd02 branches; periodic objects ignore the codes. */
typedef struct pade_pade6stagg_s* pade_pade6stagg;
int pade_pade6stagg_init(pade_pade6stagg* p, int nz, double dz, int scheme, int isPeriodic);
int pade_pade6stagg_destroy(pade_pade6stagg p);
/* generic entry: op 0 ddz_C2E, 1 ddz_E2C, 2 interpz_C2E, 3 interpz_E2C, 4 d2dz2_C2C,
 * 5 d2dz2_E2E on (n1, n2, nz) cell / (n1, n2, nz + 1) edge arrays, real or complex(rkind).
 * The combinations the reference has no operator for (d2dz2 with a one-sided end, codes
 * outside {-1, 0, 1}) give a zero output, as PadeDerOps.F90 sets output = 0. */
int pade_pade6stagg_apply(pade_pade6stagg p, int op, int is_complex, const double* in, double* out, int n1, int n2,
                          int bot, int top, void* stream);
/* the named procedures of the type (PadeDerOps.F90:146-995), REAL and CMPLX overloads */
int pade_pade6stagg_ddz_C2E(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                            void* stream);
int pade_pade6stagg_ddz_E2C(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                            void* stream);
int pade_pade6stagg_interpz_C2E(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                                void* stream);
int pade_pade6stagg_interpz_E2C(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                                void* stream);
int pade_pade6stagg_d2dz2_C2C(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                              void* stream);
int pade_pade6stagg_d2dz2_E2E(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                              void* stream);
int pade_pade6stagg_ddz_C2E_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                                  void* stream);
int pade_pade6stagg_ddz_E2C_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top,
                                  void* stream);
int pade_pade6stagg_interpz_C2E_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot,
                                      int top, void* stream);
int pade_pade6stagg_interpz_E2C_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot,
                                      int top, void* stream);
int pade_pade6stagg_d2dz2_C2C_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot,
                                    int top, void* stream);
int pade_pade6stagg_d2dz2_E2E_cmplx(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot,
                                    int top, void* stream);
/* getModifiedWavenumbers (PadeDerOps.F90:997-1016): kp of the object's scheme for the n
 * wavenumbers k (cd06: getmodCD06stagg 1034-1053; fd02: getmodFD02stagg 1055-1074).  Host. */
int pade_pade6stagg_getModifiedWavenumbers(pade_pade6stagg p, const double* k, double* kp, int n);
/* getApproxPoincareConstant (PadeDerOps.F90:1018-1032).  Host. */
int pade_pade6stagg_getApproxPoincareConstant(pade_pade6stagg p, double* c);

/* ---- common ---- */
/* replaces the destroy procedure of every type above */
int pade_destroy(pade_op op);
/* arithmetic path for the FP64 entry points of this object (PADE_PATH_DF or _NATIVE) */
int pade_set_path(pade_op op, int path);
/* Generic entry: family operation `opcode` (cd06/cd10: 1 = first, 2 = second derivative;
 * cf90/gaussian: 0; cd06stagg: 0 ddz_E2C, 1 ddz_C2E, 2 ddz_C2C, 3 ddz_E2E, 4 d2dz2_C2C,
 * 5 d2dz2_E2E, 6 InterpZ_E2C, 7 InterpZ_C2E) along direction `dir` (1, 2, 3) of an array
 * whose other two extents are na, nb (either 0: nothing to do, f and out may be null).
 * path PADE_PATH_FP32 takes float arrays. */
int pade_apply(pade_op op, int opcode, int dir, int is_complex, const void* f, void* out, int na, int nb, int bc1,
               int bcn, int path, void* stream);
/* No counterpart in the reference.  The FP64 operator application of pade_apply (the
 * object's arithmetic path; device or host buffers) for callers that cannot allocate
 * device memory once their time loop runs: it calls no cudaMalloc, cudaFree or other
 * allocating routine.  Host-buffer staging and the error flag live in one file-scope
 * device array of PADE_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the library
 * until exit; host buffers larger than half of it return PADE_ESCRATCH.  All calls share
 * the array (the flag is cleared per call), so calls whose GPU work overlaps race.  The
 * first call on a device resolves the array's address; under CUDA's lazy module loading
 * the driver may load the module and create the array then.  A call with na or nb = 0 does
 * only that set-up: make it before the time loop and before any stream capture.
 * Device-pointer calls are asynchronous and do not report PADE_ERANGE. */
#define PADE_NOALLOC_SCRATCH_BYTES (32u << 20)
int pade_apply_noalloc(pade_op op, int opcode, int dir, int is_complex, const void* f, void* out, int na, int nb,
                       int bc1, int bcn, void* stream);
/* Read and clear the sticky error flags raised by asynchronous device-pointer calls
 * (synchronises the device).  *flags != 0 means some input left the df range. */
int pade_get_status(pade_op op, int* flags);
/* line lengths of an operation: input and output points along the operated direction */
int pade_get_lengths(pade_op op, int opcode, int* n_in, int* n_out);
const char* pade_strerror(int status);

/* ==== dense operator on the tensor cores (reduced precision; no counterpart in the reference) ====
 * out = D f along x with D = A^-1 B of the object's operation (opcode, bc1, bcn) as a
 * dense matrix, on tcgen05 in "3xTF32" (D and f split into TF32 hi + lo, three products,
 * FP32 accumulation): relative error ~1e-6 of sum|D||f|.  Device pointers; lines along
 * dir 1, 2 or 3 of an (n, na, nb) / (na, n, nb) / (na, nb, n) array; n_out in
 * {128, 256, 512} and n_in a multiple of 32, otherwise PADE_ENOTSUP.  f must be 16-byte
 * aligned. */
int pade_dense_apply(pade_op op, int opcode, int dir, const double* f, double* out, int na, int nb, int bc1, int bcn,
                     void* stream);
/* *timed_out = 1 if a tensor-core wait gave up since the last call (then cleared) */
int pade_dense_status(int* timed_out);

/* ==== spectral layer, Poisson solvers and pencil transposes (device pointers only) ====
 * One GPU holds the whole grid: the reference's x/y/z pencils are the same (i,j,k)
 * Fortran-ordered array.  FFT lengths must be powers of two from 2 to 8192 (otherwise
 * PADE_ENOTSUP); transforms are FFTW-convention (forward exp(-i..), unnormalised).
 * Calls on one handle share its workspace: order them on one stream. */
typedef struct pade_spectral_s* pade_spectral;
typedef struct pade_poisson_s* pade_poisson;
typedef struct pade_poisson3d_s* pade_poisson3d;
/* modified-wavenumber callback: maps k*d to k'*d in place (PoissonPeriodic.F90:11-16) */
typedef void (*pade_modk_fn)(double* kd, int n);

/* GetWaveNums (src/incompressible/spectral.F90:1748-1764 = src/utilities/PoissonPeriodic.F90:
 * 226-242): ifftshifted wavenumbers of n points at spacing dx.  Host only. */
int pade_wavenumbers(int n, double dx, double* k);
/* getmodCD06stagg (src/incompressible/PadeDerOps.F90:1034-1053).  Host only. */
int pade_modified_wavenumbers_cd06stagg(const double* k, int n, double dz, double* kp);

/* spectral (src/incompressible/spectral.F90:867-1215 init for two periodic directions,
 * fft/ifft 1413-1452 -> fft_3d.F90:616-663 fft2_x2y / ifft2_y2x).  fix_oddball zeroes the
 * Nyquist wavenumbers k1(nx/2+1), k2(ny/2+1) (the reference default). */
int pade_spectral_init(pade_spectral* sp, int nx, int ny, int nz, double dx, double dy, int fix_oddball);
int pade_spectral_destroy(pade_spectral sp);
/* k1 (nx/2+1 entries) and k2 (ny entries) as the spectral type stores them */
int pade_spectral_get_wavenumbers(pade_spectral sp, double* k1, double* k2);
/* real (nx,ny,nz) -> complex (nx/2+1,ny,nz): r2c along x, forward c2c along y */
int pade_spectral_fft(pade_spectral sp, const double* in, void* out, void* stream);
/* complex (nx/2+1,ny,nz) -> real (nx,ny,nz): backward c2c y, c2r x, times 1/(nx ny);
 * set_oddball zeroes the x-Nyquist modes first (fft_3d.F90:633-635).  `in` is not modified. */
int pade_spectral_ifft(pade_spectral sp, const void* in, double* out, int set_oddball, void* stream);

/* The fused spectral layer: the transforms above with spectral's pointwise multipliers and
 * pairings folded into their passes (the inputs are not modified).
 * ifft(mTimes_ik1_oop(in)) (d = 1) or ifft(mTimes_ik2_oop(in)) (d = 2)
 * (spectral.F90:235-273 then 1413-1452): the x or y derivative of a spectral field. */
int pade_spectral_ifft_ik(pade_spectral sp, const void* in, double* out, int d, void* stream);
/* ifft(in) and ifft(mTimes_ik1_oop(in)): a field and its x derivative (igrid compute_duidxj,
 * igrid.F90:2553-2684), one complex x transform for both when nx = 256 */
int pade_spectral_ifft_and_ddx(pade_spectral sp, const void* in, double* out, double* out_dx, void* stream);
/* fft(in1) and fft(in2) of two real fields, the x transforms of both in one launch when
 * nx = 256 (each field keeps its own scaling, whatever their magnitudes) */
int pade_spectral_fft_two(pade_spectral sp, const double* in1, const double* in2, void* out1, void* out2,
                          void* stream);
/* ifft of two spectral fields, each with an optional multiplier d1, d2 (0 none, 1 i k1,
 * 2 i k2), the x transforms of both in one launch when nx = 256; the first call allocates
 * a second workspace of the handle */
int pade_spectral_ifft_two(pade_spectral sp, const void* in1, int d1, const void* in2, int d2, double* out1,
                           double* out2, void* stream);
/* ifft(TestFilter_oop(in)): the sharp x-y cutoff of InitTestFilter(filtfact)
 * (spectral.F90:1333-1367, 736-753) fused into the inverse transform.  The reference
 * refuses its test filter for periodic-z problems; this entry has no such restriction. */
int pade_spectral_ifft_testfilter(pade_spectral sp, const void* in, double* out, double filtfact, void* stream);

/* padepoisson with PeriodicInZ (src/incompressible/PadePoisson.F90:130-200, 76-128): the
 * periodic staggered-CD06 projection.  Keeps a pointer to `sp` (which must outlive it). */
int pade_poisson_periodic_init(pade_poisson* p, pade_spectral sp, double dx, double dy, double dz);
/* padepoisson with walls (PeriodicInZ false; PadePoisson.F90:130-318 init, 434-624
 * PressureProjection, 320-384 ProjectStokesPressure): the projection solves on the even /
 * odd extension of the fields to 2 nz points in z; compute_stokes_pressure adds the wall
 * correction with the lambda-profiles of a domain of height Lz.  DivergenceCheck then uses
 * the odd-odd staggered ddz_E2C (Pade6stagg bot = top = -1).  Keeps `sp`. */
int pade_poisson_wall_init(pade_poisson* p, pade_spectral sp, double dx, double dy, double dz, double Lz,
                           int compute_stokes_pressure);
int pade_poisson_destroy(pade_poisson p);
/* k3 modified wavenumbers used in |k|^2 (nz entries; PADE_ENOTSUP for a walled solver) */
int pade_poisson_get_modified_k3(pade_poisson p, double* k3mod);
/* PressureProjection (PadePoisson.F90:386-441 periodic, 434-624 walls): uhat, vhat complex
 * (nx/2+1,ny,nz), what complex (nx/2+1,ny,nz+1), all updated in place. */
int pade_poisson_projection(pade_poisson p, void* uhat, void* vhat, void* what, void* stream);
/* getPressure (PadePoisson.F90:716-750 periodic, 752-898 walls): the pressure that the
 * projection of (uhat, vhat, what) -- right-hand sides in the solver -- would remove, as a
 * real (nx,ny,nz) field, including the Stokes pressure with walls; the inputs are not
 * modified.  getPressureAndUpdateRHS (900-1163): the same pressure, and the inputs are
 * projected in place.  (With walls and the Stokes pressure the reference's
 * getPressureAndUpdateRHS adds the Stokes-pressure arrays that only getPressure fills; here
 * the Stokes pressure of the current call is added.) */
int pade_poisson_get_pressure(pade_poisson p, const void* uhat, const void* vhat, const void* what, double* pressure,
                              void* stream);
int pade_poisson_get_pressure_and_update_rhs(pade_poisson p, void* uhat, void* vhat, void* what, double* pressure,
                                             void* stream);
/* DivergenceCheck (PadePoisson.F90:1165-1246): divergence real (nx,ny,nz).  fix_div
 * re-projects when max(divergence) > 1e-13 (and again above 1e-10).  maxdiv (host, may be
 * NULL when fix_div is 0) receives the signed maximum of the last divergence computed;
 * asking for it synchronises the stream. */
int pade_poisson_divergence_check(pade_poisson p, void* uhat, void* vhat, void* what, double* divergence,
                                  int fix_div, double* maxdiv, void* stream);

/* PoissonPeriodic (src/utilities/PoissonPeriodic.F90:120-210 init, 37-111 poisson_solve):
 * triply periodic solve of lap f = rhs, f and rhs real (nx,ny,nz); rhs == f solves in
 * place.  dir_id 1..3 names the input pencil (all the same array here); the callbacks
 * (may be NULL) modify k*dx, k*dy, k*dz. */
int pade_poisson3d_init(pade_poisson3d* p, int nx, int ny, int nz, double dx, double dy, double dz, int dir_id,
                        pade_modk_fn modkx, pade_modk_fn modky, pade_modk_fn modkz);
int pade_poisson3d_destroy(pade_poisson3d p);
int pade_poisson3d_solve(pade_poisson3d p, const double* rhs, double* f, void* stream);

/* FFT building blocks (the FFTW plans of fft_3d.F90:198-350): c2c along dir of complex
 * (n1,n2,n3), sign -1 forward / +1 backward, times scale; r2c along x (nx,ny,nz) ->
 * (nx/2+1,ny,nz); c2r along x, times scale.  in == out is allowed for c2c. */
int pade_fft_c2c(int dir, int sign, const void* in, void* out, int n1, int n2, int n3, double scale, void* stream);
int pade_fft_r2c_x(const double* in, void* out, int nx, int ny, int nz, void* stream);
int pade_fft_c2r_x(const void* in, double* out, int nx, int ny, int nz, double scale, void* stream);

/* Arithmetic of every transform above (process-wide): PADE_FFT_DF (default, double-float
 * on the FP32 pipes, each line scaled by a power of two so its maximum is in [1, 2);
 * ~48 significant bits, elements below 2^-74 of their line's maximum count as zero) or
 * PADE_FFT_FP64 (native FP64, bound by GB300's FP64 rate).  A captured LES step graph
 * keeps the arithmetic it was captured with. */
#define PADE_FFT_DF 0
#define PADE_FFT_FP64 1
int pade_fft_set_arith(int arith);
int pade_fft_get_arith(void);

/* 2DECOMP transpose_x_to_y / y_to_z / z_to_y / y_to_x (pencil 1 = x, 2 = y, 3 = z) for
 * one rank: the pencils share the (i,j,k) layout, so this is a device copy of n1*n2*n3
 * elements of elem_bytes (8 real, 16 complex). */
int pade_transpose(int from_pencil, int to_pencil, const void* in, void* out, int n1, int n2, int n3,
                   int elem_bytes, void* stream);

/* ==== LES time step of the incompressible solver (src/incompressible/igrid.F90) ====
 * Periodic in x, y (Fourier) and z (staggered CD06), rotational advection, TVD-RK3,
 * viscosity 1/Re, Smagorinsky / standard dynamic procedure (sgsmod_igrid.F90,
 * standardDynamicProcedure.F90).  Fields live on the device; grid sizes are powers of two.
 * The reference's own dynamic test filter is not available for periodic z (spectral.F90:
 * 1338-1341); this library applies the same x-y cutoff there. */
typedef struct pade_les_s* pade_les;
typedef struct {
    int nx, ny, nz;
    double Lx, Ly, Lz;
    double Re;             /* molecular viscosity 1/Re (addViscousTerm) */
    int isInviscid;
    double CFL;            /* > 0: dt from compute_deltaT (igrid.F90:1374-1403) */
    double dt;             /* fixed time step when CFL <= 0 */
    int useSGS, dynamic;   /* dynamic: DynamicProcedureType 1 (planar averages) */
    double Csgs;           /* Smagorinsky constant when not dynamic */
    double deltaRatio;     /* test-filter width ratio (default 2) */
    int DynProcFreq;       /* dynamic procedure every DynProcFreq steps */
    double dealiasFact;    /* 2/3 rule by default */
    int t_DivergenceCheck; /* check/fix the divergence every t steps (0: never) */
    int learnedSGS;        /* 1: nu from the learned closure (pade_les_set_mlp) */
    int JudgeFreq;         /* learnedSGS: run the dynamic procedure every JudgeFreq steps as the
                              judge of the closure (pade_les_judge_info): its lambda(z) is compared
                              with the closure's plane-averaged Cs^2 Delta^2 and becomes the fallback
                              coefficient; 0: never (the fallback is then (Csgs Delta)^2) */
    int learnedPlaneAvg;   /* learnedSGS: 1 = the closure's coefficient averaged over each x-y plane
                              (nu = <Cs^2 Delta^2>_xy |S|, the dynamic procedure's form);
                              0 = pointwise (nu = Cs^2(x) Delta^2 |S|) */
    int SGSModelID;        /* eddy-viscosity kernel (init_destroy_sgs_igrid.F90:158-165): 0 Smagorinsky,
                              1 sigma (sigma.F90), 2 AMD (AMD.F90); 1 and 2 with constant coefficients
                              (DynamicProcedureType 0) */
    double JudgeTol;       /* learnedSGS with JudgeFreq > 0: when the judge's relative error
                              max_z |<Cs^2 Delta^2>_xy - lambda| / max(max_z |lambda|,
                              max_z <Cs^2 Delta^2>_xy) (0: agree, 1: one of them is zero) exceeds
                              JudgeTol (> 0),
                              every point takes the fallback (the dynamic lambda(z)) until the next
                              judge step; 0: never.  Points whose features leave the closure's
                              training range (pade_mlp_set_range) always take the fallback. */
} pade_les_params;
#define PADE_LES_UHAT 0
#define PADE_LES_VHAT 1
#define PADE_LES_WHAT 2
#define PADE_LES_U 3
#define PADE_LES_V 4
#define PADE_LES_WC 5
#define PADE_LES_W 6
#define PADE_LES_UE 7
#define PADE_LES_VE 8
#define PADE_LES_NUC 30
#define PADE_LES_NUE 31
/* duidxjC(:,:,:,i) is field 10+i-1, duidxjE(:,:,:,i) is 20+i-1 (i = 1..9, igrid order) */
int pade_les_init(pade_les* les, const pade_les_params* params);
int pade_les_destroy(pade_les les);
/* initial physical fields (device): u, v (nx,ny,nz), w on edges (nx,ny,nz+1); runs the
 * igrid init sequence (igrid.F90:625-648) and synchronises */
int pade_les_set_fields(pade_les les, const double* u, const double* v, const double* w, void* stream);
/* one TVD-RK3 step on `stream`; use_graph replays a captured CUDA graph for steps without
 * a divergence check (needs a non-NULL stream) */
int pade_les_step(pade_les les, int use_graph, void* stream);
/* last dt, simulated time, completed steps and the dynamic coefficient per z plane (nz
 * entries, may be NULL); synchronises */
int pade_les_info(pade_les les, double* dt, double* tsim, int* step, double* lambda1d);
/* simulated time and step counter, as a restart sets them (igrid.F90:2719-2765 reads tsim;
 * the step continues from the restart's time index) */
int pade_les_set_time(pade_les les, double tsim, int step);
/* the learned closure's judge (no counterpart in the reference): the relative error of the
 * last judge step (-1 before any), the closure's plane-averaged Cs^2 Delta^2 there (nz
 * entries, may be NULL) and the number of point evaluations given the fallback coefficient
 * since init; synchronises */
int pade_les_judge_info(pade_les les, double* err, double* lambda_closure, long long* n_fallback);
/* Scalar SGS flux divergence for a scalar T carried by the caller beside the LES
 * (getRHS_SGS_Scalar / getQjSGS, sgsmod_igrid.F90:268-335): Trhs -= i k1 q1^ + i k2 q2^ +
 * ddz_E2C(q3^) with q1 = -kappa dT/dx, q2 = -kappa dT/dy at the cells and q3 = -kappa dT/dz at
 * the edges.  dynamic = 0: kappa = nu_sgs / Pr, the LES's eddy viscosity at the cells and
 * edges as its last stage computed it.  dynamic = 1 (Smagorinsky kernel only):
 * DoStandardDynamicProcedureScalar (standardDynamicProcedure.F90:1-71): kappa = Beta(z) |S|,
 * Beta(z) the planar ratio <R_i P_i> / <R_i R_i> of the test-filtered fluxes, with |S|, its
 * test-filtered value and the test-filtered velocities taken from the LES's current fields
 * (the state the next pade_les_step starts from); Beta(z) is copied to beta1d (nz, host or
 * device, may be NULL; synchronises).  T: physical cells (nx, ny, nz); That: its x-y spectrum
 * (nx/2+1, ny, nz, complex); dTdxC, dTdyC, dTdzC: cells; dTdzE: edges (nx, ny, nz + 1);
 * Trhs: spectral cells, updated in place; device pointers, ordered on stream. */
int pade_les_scalar_sgs(pade_les les, const double* T, const void* That, const double* dTdxC, const double* dTdyC,
                        const double* dTdzC, const double* dTdzE, void* Trhs, double Pr, int dynamic,
                        double* beta1d, void* stream);
/* device pointer of an internal field (PADE_LES_*), valid until pade_les_destroy */
int pade_les_field(pade_les les, int which, void** ptr);
/* attach the learned closure used when learnedSGS is set (the object must outlive the
 * solver's use of it); drops a captured step graph, so call it again after retraining */
typedef struct pade_mlp_s* pade_mlp;
int pade_les_set_mlp(pade_les les, pade_mlp mlp);

/* ==== learned SGS closure (no counterpart in the reference) ====
 * MLP 10 -> 64 -> 64 -> 1 (GELU, softplus output = Cs^2) for the eddy viscosity
 * nu = Cs^2 Delta^2 |S|; it takes the place of DoStandardDynamicProcedure's coefficient
 * (sgsmod_igrid.F90:176-183).  Features per point: the 9 velocity gradients divided by
 * |S| = sqrt(2 Sij Sij) and ln(1 + Delta sqrt(|S|/nu)).  Parameters are one float array:
 * W1 (64x10 row-major), b1, W2 (64x64), b2, w3, b3.  Inference runs on the tensor cores
 * (BF16 operands, FP32 accumulation); training is FP32 with AdamW. */
#define PADE_MLP_NPARAM 4929
int pade_mlp_create(pade_mlp* mlp); /* parameters zero until pade_mlp_set_params */
int pade_mlp_destroy(pade_mlp mlp);
int pade_mlp_set_params(pade_mlp mlp, const float* host_params); /* also resets the AdamW state */
/* training range of the 10 features (host arrays lo, hi; both NULL: no range).  Inside the
 * LES, points whose features leave it take the fallback coefficient (the dynamic procedure's
 * last lambda(z), or the constant Smagorinsky one); pade_mlp_infer_nu itself ignores it. */
int pade_mlp_set_range(pade_mlp mlp, const float* lo, const float* hi);
int pade_mlp_get_params(pade_mlp mlp, float* host_params);
/* mean squared error of Cs^2 against y over B samples X (device, B x 10 row-major) and its
 * gradient (host, PADE_MLP_NPARAM); synchronises */
int pade_mlp_loss_grad(pade_mlp mlp, const float* X, const float* y, int B, float* loss, float* grad, void* stream);
/* one AdamW step (beta 0.9/0.999, eps 1e-8, decoupled weight decay wd) on that loss;
 * loss (host, may be NULL) synchronises */
int pade_mlp_train_step(pade_mlp mlp, const float* X, const float* y, int B, float lr, float wd, float* loss,
                        void* stream);
/* features of n points from the 9 gradient arrays (device pointers) into X (n x 10) */
int pade_mlp_features(const double* const* duidxj, long n, double delta, double nu, float* X, void* stream);
/* nu_out = Cs^2 Delta^2 |S| per point (FP64); cs2_out (may be NULL) receives Cs^2 */
int pade_mlp_infer_nu(pade_mlp mlp, const double* const* duidxj, long n, double delta, double nu, double* nu_out,
                      float* cs2_out, void* stream);
/* 1 in *timed_out if an inference launch since the last call gave up waiting on its tensor
 * cores (its outputs are then incomplete); clears the word; synchronises */
int pade_mlp_status(int* timed_out);

/* ---- host-only plan inspection (no GPU needed; never called by the entry points above) ----
 * family: 0 cd06, 1 cd10, 2 cf90, 3 gaussian, 4 cd06stagg, 5 Pade6stagg's fd02 (bc1, bcn =
 * the boundary codes bot, top; opcodes as pade_apply's staggered operations).
 * params: cd06/cd10 {n, dx, periodic}; cf90/gaussian {n, periodic};
 *         cd06stagg {n, dx, periodic, isTopEven, isBotEven, isTopSided, isBotSided};
 *         fd02 {nz, dz, periodic}. */
#define PADE_FAMILY_CD06 0
#define PADE_FAMILY_CD10 1
#define PADE_FAMILY_CF90 2
#define PADE_FAMILY_GAUSSIAN 3
#define PADE_FAMILY_CD06STAGG 4
#define PADE_FAMILY_FD02 5
/* Apply the device plan's arithmetic (banded LU + cyclic correction) in FP64 on the CPU to
 * `nlines` contiguous lines; lets tests validate operator plans without a GPU. */
int pade_plan_check(int family, const double* params, int opcode, int bc1, int bcn, const double* f, double* out,
                    int nlines);
/* Dense n_out x n_in matrix of the operator (row-major), for tests and the dense path. */
int pade_plan_dense(int family, const double* params, int opcode, int bc1, int bcn, double* mat, int* n_in,
                    int* n_out);

#ifdef __cplusplus
}
#endif
#endif /* PADEOPS_GB300_H */
