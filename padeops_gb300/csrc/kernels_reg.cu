// Instantiations of the register-resident periodic line kernel (reg_kernel.cuh) and its
// launcher.  Chunks of 32 rows; FP32 and double-float (FP64 in and out) arithmetic.
#include "reg_kernel.cuh"

namespace pade {

namespace {

template <class AR, int Q, int NP, bool SYM, int STG, bool RESID>
int launch_reg_t(const RegParams& c, const void* f, void* out, const LineSet& ls, unsigned* status, cudaStream_t s) {
    using IO = typename AR::IO;
    const int per = kRegThreads / c.P;  // lines per CTA
    const long blocks = (ls.nlines + per - 1) / per;
    if (blocks > 0x7fffffffL) return PS_ENOTSUP;
    k_lreg<AR, Q, NP, SYM, 32, STG, RESID, 4><<<(unsigned)blocks, kRegThreads, 0, s>>>(c, (const IO*)f, (IO*)out, ls,
                                                                                       status);
    return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
}

template <class AR>
int launch_reg_shapes(int shape, const RegParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                      cudaStream_t s) {
    switch (shape) {
        case SHAPE_T2A: return launch_reg_t<AR, 1, 2, false, 0, false>(c, f, out, ls, status, s);
        case SHAPE_T2S: return launch_reg_t<AR, 1, 2, true, 0, false>(c, f, out, ls, status, s);
        case SHAPE_P3A: return launch_reg_t<AR, 2, 3, false, 0, false>(c, f, out, ls, status, s);
        case SHAPE_P3S: return launch_reg_t<AR, 2, 3, true, 0, false>(c, f, out, ls, status, s);
        case SHAPE_P4S: return launch_reg_t<AR, 2, 4, true, 0, true>(c, f, out, ls, status, s);
        default: break;
    }
    if constexpr (AR::kScaled) {
        switch (shape) {
            case SHAPE_T2A_E2C: return launch_reg_t<AR, 1, 2, false, 1, false>(c, f, out, ls, status, s);
            case SHAPE_T2S_E2C: return launch_reg_t<AR, 1, 2, true, 1, false>(c, f, out, ls, status, s);
            case SHAPE_T2A_C2E: return launch_reg_t<AR, 1, 2, false, -1, false>(c, f, out, ls, status, s);
            case SHAPE_T2S_C2E: return launch_reg_t<AR, 1, 2, true, -1, false>(c, f, out, ls, status, s);
            default: break;
        }
    }
    return PS_ENOTSUP;
}

}  // namespace

int launch_line_reg(int shape, const RegParams& c, int fp32, const void* f, void* out, const LineSet& ls,
                    unsigned* status, cudaStream_t s) {
    RegParams p = c;
    // 16-byte loads and stores need contiguous lines whose starts are 16-byte aligned
    const long vq = fp32 ? 4 : 2;
    auto aligned = [&](const void* ptr, long a, long b, long st) {
        return st == 1 && (reinterpret_cast<uintptr_t>(ptr) & 15) == 0 && a % vq == 0 && b % vq == 0;
    };
    p.vec_in = aligned(f, ls.fa, ls.fb, ls.fp) ? 1 : 0;
    p.vec_out = aligned(out, ls.oa, ls.ob, ls.op) ? 1 : 0;
    return fp32 ? launch_reg_shapes<ArF32>(shape, p, f, out, ls, status, s)
                : launch_reg_shapes<ArDF>(shape, p, f, out, ls, status, s);
}

}  // namespace pade
