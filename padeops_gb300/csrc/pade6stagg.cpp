// Pade6stagg: igrid's staggered z-operator facade (src/incompressible/PadeDerOps.F90).
//
// Scheme cd06 (1): periodic lines use one periodic cd06stagg object; non-periodic lines hold
// the nine cd06stagg objects of PadeDerOps.F90:92-110 and pick one per call from the
// boundary codes (bot, top), each -1 (odd), 0 (one-sided) or 1 (even), as
// PadeDerOps.F90:146-995 do.  The second derivatives have no one-sided variant: like the
// reference, a 0 (or any code outside {-1, 0, 1}) gives a zero output.
// Scheme fd02 (0): the second-order staggered operators of staggOps.F90, with the per-code
// choices of PadeDerOps.F90's fd02 branches, in one handle (operators.cpp def_fd02); its
// ddz_E2C and interpz_E2C ignore the codes, as the reference's do.
// Scheme fourierColl (2), periodic only (the reference's GracefulExit 323 otherwise): the
// spectral layer's periodic-z operators (fourier_coll.cu), for nz a power of two, on device
// arrays only (the spectral layer's rule).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/padeops_gb300.h"
#include "capi_internal.h"
#include "spectral_internal.h"

struct pade_pade6stagg_s {
    int nz = 0, scheme = 1, periodic = 1;
    double dz = 1.0;
    pade_op per = nullptr;   // periodic object
    pade_op der[3][3] = {};  // non-periodic objects, [bot + 1][top + 1]
    pade_op fd = nullptr;    // fd02: every operator and code pair, built at the first call
    pade::FourierColl* fc = nullptr;  // fourierColl: mode factors, built at the first call
    std::mutex mu;
    ~pade_pade6stagg_s() {
        if (per) pade_destroy(per);
        if (fd) pade_destroy(fd);
        if (fc) pade::fourier_coll_destroy(fc);
        for (auto& r : der)
            for (auto& o : r)
                if (o) pade_destroy(o);
    }
};

namespace {

constexpr int kFD02 = 0, kCD06 = 1, kFourier = 2;

// cd06stagg flags (isTopEven, isBotEven, isTopSided, isBotSided) of der<Top><Bot>
// (PadeDerOps.F90:92-110): a one-sided end takes the other end's parity for both flags.
void flags(int bot, int top, int& te, int& be, int& ts, int& bs) {
    ts = top == 0;
    bs = bot == 0;
    if (ts && bs) {
        te = be = 1;
    } else if (ts) {
        te = be = (bot == 1);
    } else if (bs) {
        te = be = (top == 1);
    } else {
        te = (top == 1);
        be = (bot == 1);
    }
}

bool device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// facade operation -> cd06stagg opcode (pade_apply numbering)
const int kStaggOpcode[6] = {1, 0, 7, 6, 4, 5};  // ddz_C2E, ddz_E2C, interpz_C2E, interpz_E2C, d2dz2_C2C, d2dz2_E2E

}  // namespace

extern "C" {

int pade_pade6stagg_init(pade_pade6stagg* out, int nz, double dz, int scheme, int isPeriodic) {
    if (!out) return PADE_EINVAL;
    *out = nullptr;
    if (!(dz > 0.0) || nz < 1) return PADE_EINVAL;
    if (scheme != kFD02 && scheme != kCD06 && scheme != kFourier)
        return isPeriodic ? 434 : 323;  // PadeDerOps.F90:83, 118 GracefulExit codes
    if (scheme == kFourier) {
        if (!isPeriodic) return 323;                                      // PadeDerOps.F90:118
        if (nz < 2 || nz > 8192 || (nz & (nz - 1)) != 0) return PADE_ENOTSUP;  // FFT lengths
    }
    auto* h = new pade_pade6stagg_s();
    h->nz = nz;
    h->dz = dz;
    h->scheme = scheme;
    h->periodic = isPeriodic ? 1 : 0;
    if (scheme == kFD02 && nz < 3) {
        delete h;
        return PADE_EINVAL;
    }
    if (scheme == kCD06) {
        int rc = PADE_OK;
        if (h->periodic) {
            rc = pade_cd06stagg_init_periodic(&h->per, nz, dz);
        } else {
            for (int b = -1; b <= 1 && rc == PADE_OK; b++)
                for (int t = -1; t <= 1 && rc == PADE_OK; t++) {
                    int te, be, ts, bs;
                    flags(b, t, te, be, ts, bs);
                    rc = pade_cd06stagg_init_nonperiodic(&h->der[b + 1][t + 1], nz, dz, te, be, ts, bs);
                }
        }
        if (rc != PADE_OK) {
            delete h;
            return rc;
        }
    }
    *out = h;
    return PADE_OK;
}

int pade_pade6stagg_destroy(pade_pade6stagg p) {
    if (!p) return PADE_EINVAL;
    delete p;
    return PADE_OK;
}

int pade_pade6stagg_apply(pade_pade6stagg p, int op, int is_complex, const double* in, double* out, int n1, int n2,
                          int bot, int top, void* stream) {
    if (!p || op < 0 || op > 5 || n1 < 0 || n2 < 0) return PADE_EINVAL;
    if (n1 == 0 || n2 == 0) return PADE_OK;
    if (!in || !out) return PADE_EINVAL;
    if (p->scheme == kFourier) {
        {
            std::lock_guard<std::mutex> lock(p->mu);
            if (!p->fc) {
                const int rc = pade::fourier_coll_create(p->nz, p->dz, &p->fc);
                if (rc != PADE_OK) return rc;
            }
        }
        return pade::fourier_coll_apply(p->fc, op, is_complex ? 1 : 0, in, out, n1, n2,
                                        static_cast<cudaStream_t>(stream));
    }
    const bool codes = bot >= -1 && bot <= 1 && top >= -1 && top <= 1;
    if (p->scheme == kFD02) {
        {
            std::lock_guard<std::mutex> lock(p->mu);
            if (!p->fd) {
                const int rc = pade::fd02_init(&p->fd, p->nz, p->dz, p->periodic);
                if (rc != PADE_OK) return rc;
            }
        }
        int b = 0, t = 0;
        if (!p->periodic) {
            if (op == 1 || op == 3) {
                b = t = 1;  // ddz_E2C, interpz_E2C: one operator whatever the codes
            } else if (codes) {
                b = bot;
                t = top;
            } else {
                b = 2;  // no operator: zero output below
            }
        }
        if (b != 2) return pade_apply(p->fd, kStaggOpcode[op], 3, is_complex ? 1 : 0, in, out, n1, n2, b, t,
                                      PADE_PATH_DF, stream);
    }
    pade_op o = p->per;
    if (!p->periodic || p->scheme == kFD02) {
        const bool d2 = op >= 4;
        const bool valid = p->scheme == kCD06 && codes && !(d2 && (bot == 0 || top == 0));
        if (!valid) {
            // PadeDerOps.F90: output = 0 for the combinations it has no operator for
            const int nout = (op == 0 || op == 2 || op == 5) ? p->nz + 1 : p->nz;
            const size_t bytes = sizeof(double) * (size_t)nout * n1 * n2 * (is_complex ? 2 : 1);
            if (device_ptr(out))
                return cudaMemsetAsync(out, 0, bytes, static_cast<cudaStream_t>(stream)) == cudaSuccess ? PADE_OK
                                                                                                       : PADE_ECUDA;
            std::memset(out, 0, bytes);
            return PADE_OK;
        }
        o = p->der[bot + 1][top + 1];
    }
    return pade_apply(o, kStaggOpcode[op], 3, is_complex ? 1 : 0, in, out, n1, n2, 0, 0, PADE_PATH_DF, stream);
}

#define P6(name, opc, cplx)                                                                                 \
    int name(pade_pade6stagg p, const double* in, double* out, int n1, int n2, int bot, int top, void* s) { \
        return pade_pade6stagg_apply(p, opc, cplx, in, out, n1, n2, bot, top, s);                            \
    }
P6(pade_pade6stagg_ddz_C2E, 0, 0)
P6(pade_pade6stagg_ddz_E2C, 1, 0)
P6(pade_pade6stagg_interpz_C2E, 2, 0)
P6(pade_pade6stagg_interpz_E2C, 3, 0)
P6(pade_pade6stagg_d2dz2_C2C, 4, 0)
P6(pade_pade6stagg_d2dz2_E2E, 5, 0)
P6(pade_pade6stagg_ddz_C2E_cmplx, 0, 1)
P6(pade_pade6stagg_ddz_E2C_cmplx, 1, 1)
P6(pade_pade6stagg_interpz_C2E_cmplx, 2, 1)
P6(pade_pade6stagg_interpz_E2C_cmplx, 3, 1)
P6(pade_pade6stagg_d2dz2_C2C_cmplx, 4, 1)
P6(pade_pade6stagg_d2dz2_E2E_cmplx, 5, 1)
#undef P6

int pade_pade6stagg_getModifiedWavenumbers(pade_pade6stagg p, const double* k, double* kp, int n) {
    if (!p || n < 0 || (n > 0 && (!k || !kp))) return PADE_EINVAL;
    if (p->scheme == kCD06) return pade_modified_wavenumbers_cd06stagg(k, n, p->dz, kp);
    if (p->scheme == kFourier) {  // PadeDerOps.F90:1004-1005: kp = k
        for (int i = 0; i < n; i++) kp[i] = k[i];
        return PADE_OK;
    }
    // getmodFD02stagg (PadeDerOps.F90:1055-1074): alpha = beta = b = c = 0, a = 1
    for (int i = 0; i < n; i++) {
        const double w = k[i] * p->dz;
        kp[i] = (2.0 * std::sin(w / 2.0)) / p->dz;
    }
    return PADE_OK;
}

int pade_pade6stagg_getApproxPoincareConstant(pade_pade6stagg p, double* c) {
    if (!p || !c) return PADE_EINVAL;
    // PadeDerOps.F90:1018-1032
    *c = p->scheme == kCD06 ? 1.0 / std::sqrt(10.0) : (p->scheme == kFD02 ? 1.0 / std::sqrt(3.0) : 1.0 / std::sqrt(12.0));
    return PADE_OK;
}

}  // extern "C"
