// pade_apply_noalloc: the operator application of pade_apply that allocates nothing.
//
// Some callers cannot call cudaMalloc once their time loop runs: a host solver that
// reserved the device memory for its own pool at start-up (a later cudaMalloc fails or
// fragments that pool), a process under a hard device-memory quota, or a loop that keeps
// several streams busy and cannot afford the device-wide synchronisation cudaMalloc and
// cudaFree may imply.  pade_apply stages host buffers and keeps its error flag in device
// memory the library allocates on first use; this entry takes both from one file-scope
// device array instead, so after pade_*_init it calls no allocating routine.
//
// Limits and sharing:
//  * The array holds PADE_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads the
//    library, until the process exits: a 256-byte status slot and two equal staging
//    halves.  A host-pointer input or output larger than one half is rejected with
//    PADE_ESCRATCH before anything is launched; device pointers need no staging.
//  * Every call, from every object and thread, shares the array and it keeps the last
//    call's contents.  The status slot is cleared at the start of each call; staging
//    halves are fully overwritten.  Calls whose GPU work overlaps (different streams, or
//    host threads calling concurrently) race on the array and must be ordered by the
//    caller.
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress while that device is current.  Under CUDA's lazy module loading
//    that lookup is also where the driver loads this module and creates the array, so the
//    first call may make the driver allocate.  A call with na or nb = 0 does that set-up
//    and nothing else: make it (or any first call) before the time loop and before any
//    stream capture begins.
//  * Device-pointer calls return without waiting, so an infinity or NaN in their input
//    (PADE_ERANGE for host-pointer calls) is not reported: the flag in the status slot is
//    cleared by the next call.  Callers that need the check pass host buffers or test
//    their fields themselves.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/padeops_gb300.h"
#include "capi_internal.h"
#include "engine.h"

namespace {

constexpr size_t kScratchBytes = PADE_NOALLOC_SCRATCH_BYTES;
constexpr size_t kStatusBytes = 256;
constexpr size_t kStageBytes = (kScratchBytes - kStatusBytes) / 2 / 256 * 256;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device (resolved once per device).
int scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return pade::PS_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return pade::PS_ENOTSUP;
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev]) {
        void* a = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
        if (e != cudaSuccess || !a) {
            cudaGetLastError();
            return pade::PS_ECUDA;
        }
        g_addr[dev] = a;
    }
    *out = g_addr[dev];
    return pade::PS_OK;
}

bool device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

pade::LineSet lines_of(int dir, int cplx, long m, long nout, long na, long nb) {
    pade::LineSet s{};
    const long c = cplx ? 2 : 1;
    if (dir == 1 && !cplx) {
        s.nlines = na * nb; s.na = s.nlines;
        s.fa = m; s.fb = 0; s.fp = 1;
        s.oa = nout; s.ob = 0; s.op = 1;
    } else if (dir == 1) {
        s.nlines = 2 * na * nb; s.na = 2;
        s.fa = 1; s.fb = 2 * m; s.fp = 2;
        s.oa = 1; s.ob = 2 * nout; s.op = 2;
    } else if (dir == 2) {
        s.nlines = c * na * nb; s.na = c * na;
        s.fa = 1; s.fb = c * na * m; s.fp = c * na;
        s.oa = 1; s.ob = c * na * nout; s.op = c * na;
    } else {
        s.nlines = c * na * nb; s.na = s.nlines;
        s.fa = 1; s.fb = 0; s.fp = c * na * nb;
        s.oa = 1; s.ob = 0; s.op = c * na * nb;
    }
    return s;
}

}  // namespace

extern "C" int pade_apply_noalloc(pade_op h, int opcode, int dir, int is_complex, const void* f, void* out, int na,
                                  int nb, int bc1, int bcn, void* stream) {
    using namespace pade;
    if (!h) return PS_EINVAL;
    if (dir < 1 || dir > 3 || na < 0 || nb < 0) return PS_EINVAL;
    if (h->family == F_CD10 || h->family == F_CF90 || h->family == F_GAUSS) {
        if (!bc_valid(bc1) || !bc_valid(bcn)) return PS_EREF_BC;
        if (h->periodic) bc1 = bcn = 0;
    } else {
        bc1 = bcn = 0;
    }
    auto e = h->plan_err.find(plan_key(opcode, bc1, bcn));
    if (e != h->plan_err.end()) return e->second;
    auto it = h->plans.find(plan_key(opcode, bc1, bcn));
    if (it == h->plans.end()) return PS_EINVAL;
    const DevicePlan& P = *it->second;
    const OpDef& d = P.host().def;
    void* base = nullptr;
    int rc = scratch_address(&base);  // per-device set-up (once), also for empty calls
    if (rc != PS_OK) return rc;
    if (na == 0 || nb == 0) return PS_OK;  // empty arrays: nothing to do
    if (!f || !out) return PS_EINVAL;
    const int cplx = is_complex ? 1 : 0;
    const size_t in_bytes = sizeof(double) * (size_t)d.m * na * nb * (cplx ? 2 : 1);
    const size_t out_bytes = sizeof(double) * (size_t)d.nout * na * nb * (cplx ? 2 : 1);
    const bool din = device_pointer(f), dout = device_pointer(out);
    if ((!din && in_bytes > kStageBytes) || (!dout && out_bytes > kStageBytes)) return PADE_ESCRATCH;

    unsigned char* b = static_cast<unsigned char*>(base);
    unsigned* status = reinterpret_cast<unsigned*>(b);
    void* stage_in = b + kStatusBytes;
    void* stage_out = b + kStatusBytes + kStageBytes;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(status, 0, sizeof(unsigned), s) != cudaSuccess) return PS_ECUDA;
    const void* fd = f;
    void* od = out;
    if (!din) {
        if (cudaMemcpyAsync(stage_in, f, in_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return PS_ECUDA;
        fd = stage_in;
    }
    if (!dout) od = stage_out;
    const LineSet ls = lines_of(dir, cplx, d.m, d.nout, na, nb);
    rc = launch_lines(P, h->path, fd, od, ls, status, s);
    if (rc != PS_OK) return rc;
    if (din && dout) return PS_OK;  // asynchronous; the range flag stays in the status slot
    if (!dout && cudaMemcpyAsync(out, od, out_bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return PS_ECUDA;
    unsigned flag = 0;
    if (cudaMemcpyAsync(&flag, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess) return PS_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PS_ECUDA;
    return flag ? PS_ERANGE : PS_OK;
}
