// C ABI of the compact-operator library (see include/padeops_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/padeops_gb300.h"
#include "capi_internal.h"
#include "engine.h"
#include "operators.h"
#include "plan.h"

using namespace pade;

namespace {

const int kBC[3] = {0, 1, -1};

}  // namespace


namespace {

int define(int family, int n, double dx, int periodic, const StaggCfg& sc, int opcode, int bc1, int bcn,
           OpDef& d) {
    switch (family) {
    case F_CD06: return def_cd06(n, dx, periodic != 0, bc1, bcn, opcode, d);
    case F_CD10: return def_cd10(n, dx, periodic != 0, bc1, bcn, opcode, d);
    case F_CF90: return def_cf90(n, periodic != 0, bc1, bcn, d);
    case F_GAUSS: return def_gaussian(n, periodic != 0, bc1, bcn, d);
    case F_STAGG: return def_stagg(sc, opcode, d);
    case F_FD02: return def_fd02(n, dx, periodic != 0, bc1, bcn, opcode, d);
    }
    return PS_EINVAL;
}

int add_plan(pade_op_s* h, int opcode, int bc1, int bcn) {
    OpDef d;
    // cd06 takes its boundary codes at init (cd06.F90:129-146), the other families per call
    const int dbc1 = h->family == F_CD06 ? h->bc1 : bc1, dbcn = h->family == F_CD06 ? h->bcn : bcn;
    int rc = define(h->family, h->n, h->dx, h->periodic, h->sc, opcode, dbc1, dbcn, d);
    if (rc != PS_OK) {
        h->plan_err[plan_key(opcode, bc1, bcn)] = rc;
        return rc;
    }
    HostPlan hp;
    rc = build_plan(d, hp);
    if (rc != PS_OK) return rc;
    auto dp = std::make_unique<DevicePlan>();
    rc = dp->upload(hp);
    if (rc != PS_OK) return rc;
    h->plans[plan_key(opcode, bc1, bcn)] = std::move(dp);
    return PS_OK;
}

int finish_init(pade_op_s* h, pade_op* out) {
    if (cudaMalloc(&h->status, sizeof(unsigned)) != cudaSuccess) {
        h->status = nullptr;
        delete h;
        return PS_ECUDA;
    }
    if (cudaMemset(h->status, 0, sizeof(unsigned)) != cudaSuccess) {
        delete h;
        return PS_ECUDA;
    }
    *out = h;
    return PS_OK;
}

// lines of the operated direction for Fortran-ordered arrays (see LineSet)
LineSet make_lines(int dir, int cplx, long m, long nout, long na, long nb) {
    LineSet s{};
    const long c = cplx ? 2 : 1;
    if (dir == 1) {
        if (!cplx) {
            s.nlines = na * nb;
            s.na = s.nlines;
            s.fa = m; s.fb = 0; s.fp = 1;
            s.oa = nout; s.ob = 0; s.op = 1;
        } else {
            s.nlines = 2 * na * nb;
            s.na = 2;
            s.fa = 1; s.fb = 2 * m; s.fp = 2;
            s.oa = 1; s.ob = 2 * nout; s.op = 2;
        }
    } else if (dir == 2) {
        s.nlines = c * na * nb;
        s.na = c * na;
        s.fa = 1; s.fb = c * na * m; s.fp = c * na;
        s.oa = 1; s.ob = c * na * nout; s.op = c * na;
    } else {
        s.nlines = c * na * nb;
        s.na = s.nlines;
        s.fa = 1; s.fb = 0; s.fp = c * na * nb;
        s.oa = 1; s.ob = 0; s.op = c * na * nb;
    }
    return s;
}

bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int grow(void** buf, size_t* cur, size_t need) {
    if (*cur >= need) return PS_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cur = 0;
    if (cudaMalloc(buf, need) != cudaSuccess) {
        *buf = nullptr;
        return PS_ENOMEM;
    }
    *cur = need;
    return PS_OK;
}

constexpr size_t kPipeMinBytes = 8u << 20;

}  // namespace

namespace pade {
int pipe_chunks() {
    static const int n = [] {
        const char* e = std::getenv("PADE_PIPE_CHUNKS");
        const int v = e ? std::atoi(e) : 0;
        return (v >= 1 && v <= kPipeChunks) ? v : 0;
    }();
    return n;
}

// Chunk boundaries of the host-buffer pipeline over `units` rows: equal chunks when
// PADE_PIPE_CHUNKS sets a count, otherwise a ramp of weights 1 2 4 8 ... 8 4 2 1: a
// synchronous call pays the first chunk's copy-in and the last chunk's compute and copy-out
// alone, so those are small, while the middle chunks keep both copy directions busy.
int pipe_bounds(long units, long* bounds) {
    static const int kRamp[] = {1, 2, 4, 8, 8, 8, 8, 8, 8, 8, 8, 4, 2, 1};
    const int fixed = pipe_chunks();
    int nch = fixed ? fixed : (int)(sizeof(kRamp) / sizeof(kRamp[0]));
    long wsum = 0;
    for (int c = 0; c < nch; c++) wsum += fixed ? 1 : kRamp[c];
    long acc = 0;
    int out = 0;
    bounds[0] = 0;
    for (int c = 0; c < nch; c++) {
        acc += fixed ? 1 : kRamp[c];
        const long b = (units * acc + wsum - 1) / wsum;  // ceil: the last bound is units
        if (b > bounds[out]) bounds[++out] = b;        // skip empty chunks of small inputs
    }
    return out;  // number of chunks
}
}  // namespace pade

namespace {

int ensure_pipe(pade_op h) {
    if (h->pipe_ok) return PS_OK;
    for (int i = 0; i < 3; i++)
        if (cudaStreamCreateWithFlags(&h->pipe[i], cudaStreamNonBlocking) != cudaSuccess) return PS_ECUDA;
    for (int k = 0; k < 2; k++)
        for (int c = 0; c < kPipeChunks; c++)
            if (cudaEventCreateWithFlags(&h->pev[k][c], cudaEventDisableTiming) != cudaSuccess) return PS_ECUDA;
    if (cudaEventCreateWithFlags(&h->pstart, cudaEventDisableTiming) != cudaSuccess) return PS_ECUDA;
    h->pipe_ok = true;
    return PS_OK;
}

// Host input and host output: the lines are split into chunks whose host->device copy,
// operator launch and device->host copy run on three streams, so the copies of one chunk
// overlap the computation of its neighbours.  Chunks follow the memory layout of the
// LineSet: whole b-rows (contiguous slabs) when lines are grouped (fb != 0), runs of
// contiguous lines for x lines, and pitched 2-D copies when lines are strided (z lines).
int apply_host_pipelined(pade_op h, const DevicePlan& P, int path, const void* f, void* out, const LineSet& ls,
                         size_t esz, int m, int nout, cudaStream_t s) {
    int rc = ensure_pipe(h);
    if (rc != PS_OK) return rc;
    const long nl = ls.nlines;
    const int mode = ls.fb != 0 ? 0 : (ls.fp == 1 ? 1 : 2);
    const long units = mode == 0 ? nl / ls.na : nl;  // b-rows or lines
    long bounds[kPipeChunks + 1];
    const int nch = pipe_bounds(units, bounds);
    const unsigned char* fh = static_cast<const unsigned char*>(f);
    unsigned char* oh = static_cast<unsigned char*>(out);
    unsigned char* fd = static_cast<unsigned char*>(h->stage_in);
    unsigned char* od = static_cast<unsigned char*>(h->stage_out);
    if (cudaEventRecord(h->pstart, s) != cudaSuccess) return PS_ECUDA;
    for (int i = 0; i < 3; i++)
        if (cudaStreamWaitEvent(h->pipe[i], h->pstart, 0) != cudaSuccess) return PS_ECUDA;
    for (int c = 0; c < nch; c++) {
        const long u0 = bounds[c], u1 = bounds[c + 1];
        LineSet cs = ls;
        size_t ioff = 0, ooff = 0;  // element offsets of the chunk
        if (mode == 0) {
            cs.nlines = ls.na * (u1 - u0);
            ioff = (size_t)(u0 * ls.fb);
            ooff = (size_t)(u0 * ls.ob);
        } else {
            cs.nlines = u1 - u0;
            cs.na = cs.nlines;
            ioff = (size_t)(u0 * ls.fa);
            ooff = (size_t)(u0 * ls.oa);
        }
        // host -> device
        if (mode == 2) {
            if (cudaMemcpy2DAsync(fd + ioff * esz, ls.fp * esz, fh + ioff * esz, ls.fp * esz, (u1 - u0) * esz, m,
                                  cudaMemcpyHostToDevice, h->pipe[0]) != cudaSuccess)
                return PS_ECUDA;
        } else {
            const size_t bytes = (size_t)((mode == 0 ? (u1 - u0) * ls.fb : (u1 - u0) * ls.fa)) * esz;
            if (cudaMemcpyAsync(fd + ioff * esz, fh + ioff * esz, bytes, cudaMemcpyHostToDevice, h->pipe[0]) !=
                cudaSuccess)
                return PS_ECUDA;
        }
        if (cudaEventRecord(h->pev[0][c], h->pipe[0]) != cudaSuccess) return PS_ECUDA;
        if (cudaStreamWaitEvent(h->pipe[1], h->pev[0][c], 0) != cudaSuccess) return PS_ECUDA;
        if ((rc = launch_lines(P, path, fd + ioff * esz, od + ooff * esz, cs, h->status, h->pipe[1])) != PS_OK)
            return rc;
        if (cudaEventRecord(h->pev[1][c], h->pipe[1]) != cudaSuccess) return PS_ECUDA;
        if (cudaStreamWaitEvent(h->pipe[2], h->pev[1][c], 0) != cudaSuccess) return PS_ECUDA;
        // device -> host
        if (mode == 2) {
            if (cudaMemcpy2DAsync(oh + ooff * esz, ls.op * esz, od + ooff * esz, ls.op * esz, (u1 - u0) * esz,
                                  nout, cudaMemcpyDeviceToHost, h->pipe[2]) != cudaSuccess)
                return PS_ECUDA;
        } else {
            const size_t bytes = (size_t)((mode == 0 ? (u1 - u0) * ls.ob : (u1 - u0) * ls.oa)) * esz;
            if (cudaMemcpyAsync(oh + ooff * esz, od + ooff * esz, bytes, cudaMemcpyDeviceToHost, h->pipe[2]) !=
                cudaSuccess)
                return PS_ECUDA;
        }
    }
    if (cudaStreamSynchronize(h->pipe[2]) != cudaSuccess) return PS_ECUDA;
    if (cudaStreamSynchronize(h->pipe[1]) != cudaSuccess) return PS_ECUDA;
    return PS_OK;
}

int apply(pade_op h, int opcode, int dir, int cplx, const void* f, void* out, int na, int nb, int bc1, int bcn,
          int path, void* stream) {
    if (!h) return PS_EINVAL;
    if (dir < 1 || dir > 3 || na < 0 || nb < 0) return PS_EINVAL;
    if (path < PATH_DF || path > PATH_FP32) return PS_EINVAL;
    if (h->family == F_CD10 || h->family == F_CF90 || h->family == F_GAUSS || h->family == F_FD02) {
        if (!bc_valid(bc1) || !bc_valid(bcn)) return PS_EREF_BC;
    } else {
        bc1 = bcn = 0;
    }
    auto e = h->plan_err.find(plan_key(opcode, bc1, bcn));
    if (e != h->plan_err.end()) return e->second;
    auto it = h->plans.find(plan_key(opcode, bc1, bcn));
    if (it == h->plans.end()) return PS_EINVAL;
    const DevicePlan& P = *it->second;
    const OpDef& d = P.host().def;
    if (cplx && path == PATH_FP32) return PS_ENOTSUP;
    if (na == 0 || nb == 0) return PS_OK;  // empty arrays: nothing to do (the reference's loops run zero times)
    if (!f || !out) return PS_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    LineSet ls = make_lines(dir, cplx, d.m, d.nout, na, nb);
    const size_t esz = path == PATH_FP32 ? sizeof(float) : sizeof(double);
    const size_t in_bytes = esz * (size_t)d.m * na * nb * (cplx ? 2 : 1);
    const size_t out_bytes = esz * (size_t)d.nout * na * nb * (cplx ? 2 : 1);
    const bool din = is_device_ptr(f), dout = is_device_ptr(out);
    if (din && dout) return launch_lines(P, path, f, out, ls, h->status, s);
    // host pointers: stage through device buffers and return when the result is on the host
    std::lock_guard<std::mutex> lock(h->mu);
    const void* fd = f;
    void* od = out;
    int rc;
    if (!din && !dout && in_bytes >= kPipeMinBytes) {
        if ((rc = grow(&h->stage_in, &h->stage_in_bytes, in_bytes)) != PS_OK) return rc;
        if ((rc = grow(&h->stage_out, &h->stage_out_bytes, out_bytes)) != PS_OK) return rc;
        if ((rc = apply_host_pipelined(h, P, path, f, out, ls, esz, d.m, d.nout, s)) != PS_OK) return rc;
        unsigned flag = 0;
        if (cudaMemcpy(&flag, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
        if (flag) {
            cudaMemset(h->status, 0, sizeof(unsigned));
            return PS_ERANGE;
        }
        return PS_OK;
    }
    if (!din) {
        if ((rc = grow(&h->stage_in, &h->stage_in_bytes, in_bytes)) != PS_OK) return rc;
        if (cudaMemcpyAsync(h->stage_in, f, in_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return PS_ECUDA;
        fd = h->stage_in;
    }
    if (!dout) {
        if ((rc = grow(&h->stage_out, &h->stage_out_bytes, out_bytes)) != PS_OK) return rc;
        od = h->stage_out;
    }
    rc = launch_lines(P, path, fd, od, ls, h->status, s);
    if (rc != PS_OK) return rc;
    if (!dout && cudaMemcpyAsync(out, od, out_bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return PS_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PS_ECUDA;
    unsigned flag = 0;
    if (cudaMemcpy(&flag, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
    if (flag) {
        cudaMemset(h->status, 0, sizeof(unsigned));
        return PS_ERANGE;
    }
    return PS_OK;
}

}  // namespace

extern "C" {

// ---- cd06 ----
int pade_cd06_init(pade_op* op, int n, double dx, int periodic, int bc1, int bcn) {
    if (!op) return PS_EINVAL;
    *op = nullptr;
    if (n < 1 || !(dx > 0.0)) return PS_EINVAL;
    if (periodic && n != 1 && n < 6) return PS_EREF_PERIODIC_N;
    if (!periodic && n != 1 && n < 8) return PS_EREF_NONPERIODIC_N;
    auto* h = new pade_op_s();
    h->family = F_CD06;
    h->n = n;
    h->dx = dx;
    h->periodic = periodic ? 1 : 0;
    h->bc1 = bc1;
    h->bcn = bcn;
    int rc;
    if ((rc = add_plan(h, 1, 0, 0)) != PS_OK) { delete h; return rc; }
    rc = add_plan(h, 2, 0, 0);
    if (rc != PS_OK && rc != PS_ENOTSUP) { delete h; return rc; }
    return finish_init(h, op);
}
#define CD06_DD(name, opc, dir)                                                                 \
    int name(pade_op op, const double* f, double* df, int na, int nb, void* stream) {           \
        if (!op || op->family != F_CD06) return PS_EINVAL;                                         \
        return apply(op, opc, dir, 0, f, df, na, nb, 0, 0, op->path, stream);                  \
    }
CD06_DD(pade_cd06_dd1, 1, 1)
CD06_DD(pade_cd06_dd2, 1, 2)
CD06_DD(pade_cd06_dd3, 1, 3)
CD06_DD(pade_cd06_d2d1, 2, 1)
CD06_DD(pade_cd06_d2d2, 2, 2)
CD06_DD(pade_cd06_d2d3, 2, 3)

// ---- cd10 ----
int pade_cd10_init(pade_op* op, int n, double dx, int periodic, int bc1, int bcn) {
    if (!op) return PS_EINVAL;
    *op = nullptr;
    if (n < 1 || !(dx > 0.0)) return PS_EINVAL;
    if (n != 1 && n < 8) return PS_EREF_NONPERIODIC_N;
    auto* h = new pade_op_s();
    h->family = F_CD10;
    h->n = n;
    h->dx = dx;
    h->periodic = periodic ? 1 : 0;
    h->bc1 = bc1;
    h->bcn = bcn;
    int rc;
    for (int order = 1; order <= 2; order++) {
        if (periodic) {
            if ((rc = add_plan(h, order, 0, 0)) != PS_OK) { delete h; return rc; }
        } else {
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++)
                    if ((rc = add_plan(h, order, kBC[a], kBC[b])) != PS_OK) { delete h; return rc; }
        }
    }
    return finish_init(h, op);
}
#define CD10_DD(name, opc, dir)                                                                          \
    int name(pade_op op, const double* f, double* df, int na, int nb, int bc1, int bcn, void* stream) {  \
        if (!op || op->family != F_CD10) return PS_EINVAL;                                                  \
        if (!bc_valid(bc1) || !bc_valid(bcn)) return PS_EREF_BC;                                            \
        if (op->periodic) bc1 = bcn = 0;                                                                 \
        return apply(op, opc, dir, 0, f, df, na, nb, bc1, bcn, op->path, stream);                       \
    }
CD10_DD(pade_cd10_dd1, 1, 1)
CD10_DD(pade_cd10_dd2, 1, 2)
CD10_DD(pade_cd10_dd3, 1, 3)
CD10_DD(pade_cd10_d2d1, 2, 1)
CD10_DD(pade_cd10_d2d2, 2, 2)
CD10_DD(pade_cd10_d2d3, 2, 3)

// ---- cf90 / gaussian ----
static int filter_init(pade_op* op, int family, int n, int periodic) {
    if (!op) return PS_EINVAL;
    *op = nullptr;
    if (n < 1) return PS_EINVAL;
    auto* h = new pade_op_s();
    h->family = family;
    h->n = n;
    h->periodic = periodic ? 1 : 0;
    int rc;
    if (periodic) {
        if ((rc = add_plan(h, 0, 0, 0)) != PS_OK) { delete h; return rc; }
    } else {
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                if ((rc = add_plan(h, 0, kBC[a], kBC[b])) != PS_OK) { delete h; return rc; }
    }
    return finish_init(h, op);
}
int pade_cf90_init(pade_op* op, int n, int periodic) { return filter_init(op, F_CF90, n, periodic); }
int pade_gaussian_init(pade_op* op, int n, int periodic) { return filter_init(op, F_GAUSS, n, periodic); }
#define FILT(name, fam, dir, cplx)                                                                       \
    int name(pade_op op, const double* f, double* ff, int na, int nb, int bc1, int bcn, void* stream) {  \
        if (!op || op->family != fam) return PS_EINVAL;                                                     \
        if (!bc_valid(bc1) || !bc_valid(bcn)) return PS_EREF_BC;                                            \
        if (op->periodic) bc1 = bcn = 0;                                                                 \
        return apply(op, 0, dir, cplx, f, ff, na, nb, bc1, bcn, op->path, stream);                      \
    }
FILT(pade_cf90_filter1, F_CF90, 1, 0)
FILT(pade_cf90_filter2, F_CF90, 2, 0)
FILT(pade_cf90_filter3, F_CF90, 3, 0)
FILT(pade_cf90_filter3_cmplx, F_CF90, 3, 1)
FILT(pade_gaussian_filter1, F_GAUSS, 1, 0)
FILT(pade_gaussian_filter2, F_GAUSS, 2, 0)
FILT(pade_gaussian_filter3, F_GAUSS, 3, 0)
FILT(pade_gaussian_filter3_cmplx, F_GAUSS, 3, 1)

// ---- cd06stagg ----
static int stagg_init(pade_op* op, const StaggCfg& c) {
    if (!op) return PS_EINVAL;
    *op = nullptr;
    if (!(c.dx > 0.0)) return PS_EINVAL;
    if (c.n <= 4) return PS_EREF_STAGG_N;
    auto* h = new pade_op_s();
    h->family = F_STAGG;
    h->n = c.n;
    h->dx = c.dx;
    h->periodic = c.periodic;
    h->sc = c;
    for (int o = 0; o < STAGG_NOPS; o++) {
        int rc = add_plan(h, o, 0, 0);
        if (rc != PS_OK && rc != PS_ENOTSUP) { delete h; return rc; }
    }
    return finish_init(h, op);
}
}  // extern "C"

int pade::fd02_init(pade_op* op, int nz, double dz, int periodic) {
    if (!op) return PS_EINVAL;
    *op = nullptr;
    if (!(dz > 0.0) || nz < 3) return PS_EINVAL;
    auto* h = new pade_op_s();
    h->family = F_FD02;
    h->n = nz;
    h->dx = dz;
    h->periodic = periodic ? 1 : 0;
    const int ops[6] = {D1_E2C, D1_C2E, D2_C2C, D2_E2E, I_E2C, I_C2E};
    for (int o : ops) {
        for (int b = -1; b <= 1; b++)
            for (int t = -1; t <= 1; t++) {
                if (h->periodic && (b != 0 || t != 0)) continue;  // periodic calls use codes (0, 0)
                const int rc = add_plan(h, o, b, t);
                if (rc != PS_OK) {
                    delete h;
                    return rc;
                }
            }
    }
    return finish_init(h, op);
}

extern "C" {

int pade_cd06stagg_init_periodic(pade_op* op, int n, double dx) {
    StaggCfg c;
    c.n = n;
    c.dx = dx;
    c.periodic = true;
    return stagg_init(op, c);
}
int pade_cd06stagg_init_nonperiodic(pade_op* op, int n, double dx, int isTopEven, int isBotEven, int isTopSided,
                                    int isBotSided) {
    StaggCfg c;
    c.n = n;
    c.dx = dx;
    c.periodic = false;
    c.topEven = isTopEven != 0;
    c.botEven = isBotEven != 0;
    c.topSided = isTopSided != 0;
    c.botSided = isBotSided != 0;
    return stagg_init(op, c);
}
#define STG(name, opc, cplx)                                                                 \
    int name(pade_op op, const double* fi, double* fo, int n1, int n2, void* stream) {       \
        if (!op || op->family != F_STAGG) return PS_EINVAL;                                     \
        return apply(op, opc, 3, cplx, fi, fo, n1, n2, 0, 0, op->path, stream);              \
    }
STG(pade_cd06stagg_ddz_E2C, D1_E2C, 0)
STG(pade_cd06stagg_ddz_C2E, D1_C2E, 0)
STG(pade_cd06stagg_ddz_C2C, D1_C2C, 0)
STG(pade_cd06stagg_ddz_E2E, D1_E2E, 0)
STG(pade_cd06stagg_d2dz2_C2C, D2_C2C, 0)
STG(pade_cd06stagg_d2dz2_E2E, D2_E2E, 0)
STG(pade_cd06stagg_InterpZ_E2C, I_E2C, 0)
STG(pade_cd06stagg_InterpZ_C2E, I_C2E, 0)
STG(pade_cd06stagg_ddz_E2C_cmplx, D1_E2C, 1)
STG(pade_cd06stagg_ddz_C2E_cmplx, D1_C2E, 1)
STG(pade_cd06stagg_ddz_C2C_cmplx, D1_C2C, 1)
STG(pade_cd06stagg_ddz_E2E_cmplx, D1_E2E, 1)
STG(pade_cd06stagg_d2dz2_C2C_cmplx, D2_C2C, 1)
STG(pade_cd06stagg_d2dz2_E2E_cmplx, D2_E2E, 1)
STG(pade_cd06stagg_InterpZ_E2C_cmplx, I_E2C, 1)
STG(pade_cd06stagg_InterpZ_C2E_cmplx, I_C2E, 1)

// ---- common ----
int pade_destroy(pade_op op) {
    if (!op) return PS_EINVAL;
    delete op;
    return PS_OK;
}

int pade_set_path(pade_op op, int path) {
    if (!op || (path != PATH_DF && path != PATH_NATIVE)) return PS_EINVAL;
    op->path = path;
    return PS_OK;
}

int pade_apply(pade_op op, int opcode, int dir, int is_complex, const void* f, void* out, int na, int nb, int bc1,
               int bcn, int path, void* stream) {
    if (!op) return PS_EINVAL;
    if (op->periodic && op->family != F_STAGG) bc1 = bcn = 0;
    return apply(op, opcode, dir, is_complex, f, out, na, nb, bc1, bcn, path, stream);
}

int pade_get_status(pade_op op, int* flags) {
    if (!op || !flags) return PS_EINVAL;
    if (cudaDeviceSynchronize() != cudaSuccess) return PS_ECUDA;
    unsigned v = 0;
    if (cudaMemcpy(&v, op->status, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return PS_ECUDA;
    if (cudaMemset(op->status, 0, sizeof(unsigned)) != cudaSuccess) return PS_ECUDA;
    *flags = (int)v;
    return PS_OK;
}

int pade_get_lengths(pade_op op, int opcode, int* n_in, int* n_out) {
    if (!op || !n_in || !n_out) return PS_EINVAL;
    for (auto& kv : op->plans)
        if (kv.first / 16 == opcode) {
            *n_in = kv.second->host().def.m;
            *n_out = kv.second->host().def.nout;
            return PS_OK;
        }
    auto e = op->plan_err.begin();
    for (; e != op->plan_err.end(); ++e)
        if (e->first / 16 == opcode) return e->second;
    return PS_EINVAL;
}

const char* pade_strerror(int s) {
    switch (s) {
    case PS_OK: return "ok";
    case PS_EREF_NONPERIODIC_N: return "n too small for this scheme (reference init ierr 2)";
    case PS_EREF_PERIODIC_N: return "periodic cd06 needs n >= 6 (reference init ierr 3)";
    case PS_EREF_FILTER_N: return "cf90 needs n >= 10 (reference init ierr 7)";
    case PS_EREF_STAGG_N: return "CD06_stagg requires at least 4 points (reference GracefulExit 21)";
    case PS_EREF_BC: return "Incorrect boundary specification (should be 0, 1 or -1) (reference GracefulExit 324)";
    case PS_EINVAL: return "invalid argument";
    case PS_ENOMEM: return "device allocation failed";
    case PS_ECUDA: return "CUDA error";
    case PS_ENOTSUP: return "operation not supported for this object";
    case PS_ETIMEOUT: return "timed out";
    case PS_ERANGE: return "input outside the double-float range";
    case PADE_ESCRATCH: return "buffer larger than the static staging capacity of pade_apply_noalloc";
    }
    return "unknown status";
}

// ---- host-only plan inspection ----
static int host_def(int family, const double* p, int opcode, int bc1, int bcn, OpDef& d) {
    if (!p) return PS_EINVAL;
    StaggCfg sc;
    int n = (int)p[0];
    double dx = 1.0;
    int periodic = 1;
    if (family == F_CD06 || family == F_CD10) { dx = p[1]; periodic = (int)p[2]; }
    else if (family == F_CF90 || family == F_GAUSS) periodic = (int)p[1];
    else if (family == F_FD02) { dx = p[1]; periodic = (int)p[2]; }
    else if (family == F_STAGG) {
        sc.n = n;
        sc.dx = p[1];
        sc.periodic = p[2] != 0;
        sc.topEven = p[3] != 0;
        sc.botEven = p[4] != 0;
        sc.topSided = p[5] != 0;
        sc.botSided = p[6] != 0;
    } else return PS_EINVAL;
    return define(family, n, dx, periodic, sc, opcode, bc1, bcn, d);
}

int pade_plan_check(int family, const double* params, int opcode, int bc1, int bcn, const double* f, double* out,
                    int nlines) {
    OpDef d;
    int rc = host_def(family, params, opcode, bc1, bcn, d);
    if (rc != PS_OK) return rc;
    HostPlan hp;
    if ((rc = build_plan(d, hp)) != PS_OK) return rc;
    for (int l = 0; l < nlines; l++) host_apply_line(hp, f + (size_t)l * d.m, 1, out + (size_t)l * d.nout, 1);
    return PS_OK;
}

int pade_plan_dense(int family, const double* params, int opcode, int bc1, int bcn, double* mat, int* n_in,
                    int* n_out) {
    OpDef d;
    int rc = host_def(family, params, opcode, bc1, bcn, d);
    if (rc != PS_OK) return rc;
    if (n_in) *n_in = d.m;
    if (n_out) *n_out = d.nout;
    if (!mat) return PS_OK;
    std::vector<double> M;
    if ((rc = dense_operator(d, M)) != PS_OK) return rc;
    memcpy(mat, M.data(), M.size() * sizeof(double));
    return PS_OK;
}

}  // extern "C"
