// Definition of the library handle, shared by the translation units of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>

#include "engine.h"
#include "operators.h"

namespace pade {

enum Family { F_CD06 = 0, F_CD10 = 1, F_CF90 = 2, F_GAUSS = 3, F_STAGG = 4, F_FD02 = 5 };

inline int bcid(int bc) { return bc == 0 ? 0 : (bc == 1 ? 1 : 2); }
inline bool bc_valid(int bc) { return bc == 0 || bc == 1 || bc == -1; }
// plans are keyed by opcode * 16 + bc index (bcid(bc1) * 3 + bcid(bcn))
inline int plan_key(int opcode, int bc1, int bcn) { return opcode * 16 + bcid(bc1) * 3 + bcid(bcn); }

// chunks of the host-buffer copy-in / compute / copy-out pipeline (capi.cpp): at most
// kPipeChunks; a ramp of 14 chunks by default (pipe_bounds), or PADE_PIPE_CHUNKS equal ones (a tuning override)
constexpr int kPipeChunks = 32;
int pipe_chunks();

}  // namespace pade

namespace pade {
// frees the dense (tensor-core path) matrices cached for a handle (dense_tc.cu)
void dense_release(const void* h);
// Pade6stagg's fd02 operators on nz cells (capi.cpp): one handle holding every operator for
// every boundary-code pair (bot, top) in {-1, 0, 1}^2 (passed as pade_apply's bc1, bc2), or
// the periodic operators
int fd02_init(struct pade_op_s** op, int nz, double dz, int periodic);
}  // namespace pade

struct pade_op_s {
    int family = 0;
    int n = 0;
    double dx = 1.0;
    int periodic = 1, bc1 = 0, bcn = 0;
    pade::StaggCfg sc;
    int path = pade::PATH_DF;
    // plans keyed by plan_key(opcode, bc1, bcn)
    std::map<int, std::unique_ptr<pade::DevicePlan>> plans;
    std::map<int, int> plan_err;  // opcodes the reference refuses (e.g. cd06 non-periodic d2)
    unsigned* status = nullptr;   // device flag word
    // staging for host-pointer calls
    std::mutex mu;
    void* stage_in = nullptr;
    void* stage_out = nullptr;
    size_t stage_in_bytes = 0, stage_out_bytes = 0;
    // host-pointer pipeline: copy-in, compute and copy-out streams and per-chunk events
    cudaStream_t pipe[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t pev[2][pade::kPipeChunks] = {};
    cudaEvent_t pstart = nullptr;
    bool pipe_ok = false;
    ~pade_op_s() {
        pade::dense_release(this);
        if (pipe_ok) {
            for (int i = 0; i < 3; i++) cudaStreamDestroy(pipe[i]);
            for (int k = 0; k < 2; k++)
                for (int c = 0; c < pade::kPipeChunks; c++) cudaEventDestroy(pev[k][c]);
            cudaEventDestroy(pstart);
        }
        if (status) cudaFree(status);
        if (stage_in) cudaFree(stage_in);
        if (stage_out) cudaFree(stage_out);
    }
};
