// CUDA kernels of the compact line operators (sm_103a), plan upload and launch dispatch.
//
//  * k_seq     one thread per line, native FP64, the plan's banded LU + cyclic Woodbury
//              correction; the reference-order baseline (FP64-pipe bound on GB300).
//  * k_chunk   the fast path, see chunk_kernel.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "chunk_kernel.cuh"
#include "reg_kernel.cuh"

namespace pade {

// ------------------------------------------------------------------------------------
// k_seq: one thread per line, native FP64
// ------------------------------------------------------------------------------------
__global__ void k_seq(const PlanView<double> P, const double* __restrict__ f, double* __restrict__ out,
                      const LineSet ls) {
    const long l = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= ls.nlines) return;
    const long a = l % ls.na, b = l / ls.na;
    const double* fl = f + a * ls.fa + b * ls.fb;
    double* ol = out + a * ls.oa + b * ls.ob;
    const long fp = ls.fp, op = ls.op;
    if (P.zero) {
        for (int i = 0; i < P.nout; i++) ol[i * op] = 0.0;
        return;
    }
    if (P.identity) {
        for (int i = 0; i < P.nout; i++) ol[i * op] = fl[i * fp];
        return;
    }
    const int ns = P.ns;
    // RHS
    for (int i = 0; i < ns; i++) {
        double r = 0.0;
        if (i < P.nlo || i >= ns - P.nhi) {
            const int t = i < P.nlo ? i : P.nlo + (i - (ns - P.nhi));
            for (int k = 0; k < P.tw; k++) r = fma(P.tc[t * P.tw + k], fl[(long)P.tidx[t * P.tw + k] * fp], r);
        } else {
            for (int k = 0; k < P.ntap; k++) r = fma(P.ic[k], fl[(long)(i + P.io[k]) * fp], r);
        }
        ol[i * op] = r;
    }
    if (P.q > 0) {
        double y1 = ol[0], y2 = 0.0;
        for (int i = 1; i < ns; i++) {
            double v = ol[i * op] - P.lu[i * 5 + 0] * y1 - P.lu[i * 5 + 1] * y2;
            ol[i * op] = v;
            y2 = y1;
            y1 = v;
        }
        double x1 = 0.0, x2 = 0.0;
        for (int i = ns - 1; i >= 0; i--) {
            double v = (ol[i * op] - P.lu[i * 5 + 2] * x1 - P.lu[i * 5 + 3] * x2) * P.lu[i * 5 + 4];
            ol[i * op] = v;
            x2 = x1;
            x1 = v;
        }
        if (P.nc > 0) {
            double g[kMaxNc], h[kMaxNc];
            for (int c = 0; c < P.nc; c++) {
                double s = 0.0;
                for (int t = 0; t < P.q; t++) s += P.wc[c * P.q + t] * ol[(long)P.wcol[c * P.q + t] * op];
                g[c] = s;
            }
            for (int c = 0; c < P.nc; c++) {
                double s = 0.0;
                for (int d = 0; d < P.nc; d++) s += P.Cinv[c * P.nc + d] * g[d];
                h[c] = s;
            }
            for (int i = 0; i < ns; i++) {
                double v = ol[i * op];
                for (int c = 0; c < P.nc; c++) v -= P.Z[(long)i * P.nc + c] * h[c];
                ol[i * op] = v;
            }
        }
    }
    if (P.resid)
        for (int i = 0; i < ns; i++) ol[i * op] = fl[i * fp] - ol[i * op];
    for (int i = ns; i < P.nout; i++) ol[i * op] = ol[(i - ns) * op];
}

// trivial operators (n == 1): zero or copy, any precision
template <class IO>
__global__ void k_trivial(int zero, int nout, const IO* __restrict__ f, IO* __restrict__ out, const LineSet ls) {
    const long l = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= ls.nlines) return;
    const long a = l % ls.na, b = l / ls.na;
    for (int i = 0; i < nout; i++)
        out[a * ls.oa + b * ls.ob + i * ls.op] = zero ? (IO)0 : f[a * ls.fa + b * ls.fb + i * ls.fp];
}

// ------------------------------------------------------------------------------------
// plan upload
// ------------------------------------------------------------------------------------
namespace {

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Arena {
    std::vector<unsigned char> host;
    size_t put(const void* p, size_t bytes) {
        size_t off = align_up(host.size(), 16);
        host.resize(off + std::max<size_t>(bytes, 16));
        if (bytes) memcpy(host.data() + off, p, bytes);
        return off;
    }
};

F2 split(double v) {
    F2 r;
    r.h = (float)v;
    r.l = (float)(v - (double)r.h);
    return r;
}

}  // namespace

DevicePlan::~DevicePlan() {
    if (dev_) cudaFree(dev_);
    delete creg_;
}

int DevicePlan::upload(const HostPlan& hp) {
    hp_ = hp;
    const OpDef& d = hp.def;
    Arena A;
    // --- native view ---
    size_t o_tidx = A.put(hp.tidx.data(), hp.tidx.size() * sizeof(int));
    size_t o_tc = A.put(hp.tc.data(), hp.tc.size() * sizeof(double));
    size_t o_lu = A.put(hp.lu.data(), hp.lu.size() * sizeof(double));
    size_t o_Z = A.put(hp.Z.data(), hp.Z.size() * sizeof(double));
    size_t o_Ci = A.put(hp.Cinv.data(), hp.Cinv.size() * sizeof(double));
    size_t o_wcol = A.put(hp.wcol.data(), hp.wcol.size() * sizeof(int));
    size_t o_wc = A.put(hp.wc.data(), hp.wc.size() * sizeof(double));

    // --- chunk plan ---
    const int M = (d.ns <= 512) ? 16 : 32;
    int rc = d.zero || d.identity ? PS_OK : build_chunk_plan(hp, M, ch_);
    cok_ = (rc == PS_OK && ch_.ok && ch_.use_pairs);
    size_t o_ctidx = 0, o_ctc[2] = {0, 0}, o_rc[2] = {0, 0}, o_fs[2] = {0, 0}, o_bs[2] = {0, 0}, o_fw[2] = {0, 0},
           o_bw[2] = {0, 0}, o_pf[2] = {0, 0}, o_pb[2] = {0, 0};
    // circulant: fold the forward scale 1/c into the stencil and edge rows
    const double cg = (cok_ && ch_.circ) ? ch_.rc[0] : 1.0;
    if (cok_) {
        o_ctidx = A.put(ch_.tidx.data(), ch_.tidx.size() * sizeof(int));
        for (int v = 0; v < 2; v++) {  // v=0: double-float coefficients, v=1: FP32
            auto conv = [&](const std::vector<double>& src, double scale) {
                std::vector<F2> o(src.size());
                for (size_t k = 0; k < src.size(); k++) {
                    o[k] = split(src[k] * scale);
                    if (v == 1) o[k].l = 0.0f;
                }
                return o;
            };
            auto tc = conv(ch_.tc, cg);
            o_ctc[v] = A.put(tc.data(), tc.size() * sizeof(F2));
            auto r = conv(ch_.rc, 1.0);
            o_rc[v] = A.put(r.data(), r.size() * sizeof(F2));
            auto fs = conv(ch_.fscan, 1.0);
            o_fs[v] = A.put(fs.data(), fs.size() * sizeof(F2));
            auto bs = conv(ch_.bscan, 1.0);
            o_bs[v] = A.put(bs.data(), bs.size() * sizeof(F2));
            auto fw = conv(ch_.fwrap, 1.0);
            o_fw[v] = A.put(fw.data(), fw.size() * sizeof(F2));
            auto bw = conv(ch_.bwrap, 1.0);
            o_bw[v] = A.put(bw.data(), bw.size() * sizeof(F2));
            auto pf = conv(ch_.phf, 1.0);
            o_pf[v] = A.put(pf.data(), pf.size() * sizeof(F2));
            auto pb = conv(ch_.phb, 1.0);
            o_pb[v] = A.put(pb.data(), pb.size() * sizeof(F2));
        }
    }
    // fixed-stencil kernel: whole chunks, pairs k = 1..NP about the row or (staggered,
    // periodic tridiagonal lines only) about a half point, one sign; banded lines also need
    // edge rows covering the stencil's reach at both ends
    line_shape_ = SHAPE_NONE;
    size_t o_lk[6] = {0, 0, 0, 0, 0, 0};
    // (periodic lines may carry the duplicated point n + 1 of the edge grid: m = ns + 1 is read
    // as ns rows, and an output of ns + 1 rows repeats row 0)
    if (cok_ && ch_.M == kLineM && (d.m == d.ns || (ch_.circ && d.m == d.ns + 1)) && d.ns % kLineM == 0 &&
        d.ns <= 512 && ch_.P <= kMaxLanes &&
        (ch_.Q == 1 || ch_.Q == 2) && (ch_.circ || d.nout == d.ns)) {
        const int np = ch_.npair;
        bool ok = np >= 1 && np <= kMaxPairs;
        bool seen[kMaxPairs + 1] = {};
        int sgn = 0;
        StencilParams cc{};
        // twice the stencil centre: 0 (centred), +1 (edges to cells), -1 (cells to edges)
        const int d2 = ok ? ch_.pair_op[0] + ch_.pair_om[0] : 0;
        if (d2 < -1 || d2 > 1) ok = false;
        for (int k = 0; k < np && ok; k++) {
            const int o = d2 < 0 ? -ch_.pair_om[k] : ch_.pair_op[k];  // the pair's index 1..np
            if (o < 1 || o > np || ch_.pair_op[k] + ch_.pair_om[k] != d2 || seen[o]) {
                ok = false;
                break;
            }
            seen[o] = true;
            cc.c[o - 1] = split(ch_.pair_c[k] * cg);
            if (sgn == 0) sgn = ch_.pair_sign[k];
            else if (sgn != ch_.pair_sign[k]) ok = false;
        }
        if (ch_.has_center && (ch_.center_off != 0 || sgn < 0 || d2 != 0)) ok = false;
        if (d2 != 0 && !(ch_.circ && ch_.Q == 1 && np == 2 && !ch_.resid && d.ns % 32 == 0)) ok = false;
        if (!ch_.circ && (ch_.nlo < np || ch_.nhi < np || ch_.nlo + ch_.nhi > 32)) ok = false;
        int shape = SHAPE_NONE;
        if (ok && d2 != 0) {
            shape = d2 > 0 ? (sgn < 0 ? SHAPE_T2A_E2C : SHAPE_T2S_E2C) : (sgn < 0 ? SHAPE_T2A_C2E : SHAPE_T2S_C2E);
        } else if (ok) {
            if (ch_.Q == 1 && np == 2) shape = sgn < 0 ? SHAPE_T2A : SHAPE_T2S;
            else if (ch_.Q == 2 && np == 3) shape = sgn < 0 ? SHAPE_P3A : SHAPE_P3S;
            else if (ch_.Q == 2 && np == 4 && sgn > 0) shape = SHAPE_P4S;
        }
        // residual-form operators keep the input beside the work rows (chunks of 16); the
        // others overwrite their input window and take chunks of 32 rows on periodic lines
        // (16 on banded lines: measured faster there)
        const bool alias = !ch_.resid;
        if (alias == (shape == SHAPE_P4S)) shape = SHAPE_NONE;  // instantiated pairings only
        int Ml = kLineM;
        if (alias && ch_.circ && d.ns % 32 == 0) Ml = 32;
        if (const char* e = std::getenv("PADE_LINE_CHUNK")) {  // tuning override: 16 or 32
            const int v = std::atoi(e);
            if (v == 16 || (v == 32 && alias && d.ns % 32 == 0)) Ml = v;
        }
        if (shape >= SHAPE_T2A_E2C) Ml = 32;  // the staggered shapes run in chunks of 32 only
        ChunkPlanHost c32;
        const ChunkPlanHost* cl = &ch_;
        if (shape != SHAPE_NONE && Ml != ch_.M) {
            if (build_chunk_plan(hp, Ml, c32) == PS_OK && c32.ok) {
                cl = &c32;
                auto put = [&](const std::vector<double>& src) {
                    std::vector<F2> o(src.size());
                    for (size_t k = 0; k < src.size(); k++) o[k] = split(src[k]);
                    return A.put(o.data(), o.size() * sizeof(F2));
                };
                o_lk[0] = put(c32.fscan);
                o_lk[1] = put(c32.bscan);
                o_lk[2] = put(c32.fwrap);
                o_lk[3] = put(c32.bwrap);
                o_lk[4] = put(c32.phf);
                o_lk[5] = put(c32.phb);
            } else {
                Ml = ch_.M;
            }
        }
        if (shape >= SHAPE_T2A_E2C && Ml != 32) shape = SHAPE_NONE;
        if (shape != SHAPE_NONE) {
            cc.M = Ml;
            cc.alias = alias ? 1 : 0;
            cc.ns = cl->ns;
            cc.nout = cl->nout;
            cc.P = cl->P;
            cc.Pp = cl->Pp;
            cc.nsteps = cl->nsteps;
            cc.L = (ch_.circ ? kLineThreadsCirc : kLineThreadsBand) / cl->Pp;
            cc.resid = ch_.resid;
            cc.xdup = (shape == SHAPE_T2A_E2C || shape == SHAPE_T2S_E2C) && d.m == d.ns + 1;
            cc.circ = ch_.circ;
            cc.nlo = ch_.circ ? 0 : ch_.nlo;
            cc.nhi = ch_.circ ? 0 : ch_.nhi;
            cc.tw = ch_.tw;
            cc.c0 = ch_.has_center ? split(ch_.center_c * cg) : F2{0.0f, 0.0f};
            cc.ca1 = split(ch_.circ ? ch_.rc[1] : 0.0);
            cc.ca2 = split(ch_.circ ? ch_.rc[2] : 0.0);
            cline_ = cc;
            line_shape_ = shape;
        }
    }
    // residual-form filters (cf90) keep 16-row chunks for k_line; the half-chunk kernel
    // takes 32-row chunks, with tables of their own
    size_t o_h32[6] = {0, 0, 0, 0, 0, 0};
    ChunkPlanHost h32;
    bool h32_ok = false;
    if (line_shape_ == SHAPE_P4S && cline_.M == 16 && cline_.resid && ch_.circ && d.ns % 32 == 0 &&
        build_chunk_plan(hp, 32, h32) == PS_OK && h32.ok && kLineThreadsCirc % h32.Pp == 0) {
        auto put = [&](const std::vector<double>& src) {
            std::vector<F2> o(src.size());
            for (size_t k = 0; k < src.size(); k++) o[k] = split(src[k]);
            return A.put(o.data(), o.size() * sizeof(F2));
        };
        o_h32[0] = put(h32.fscan);
        o_h32[1] = put(h32.bscan);
        o_h32[2] = put(h32.fwrap);
        o_h32[3] = put(h32.bwrap);
        o_h32[4] = put(h32.phf);
        o_h32[5] = put(h32.phb);
        h32_ok = true;
    }
    // the banded half-chunk kernel's tables: the NF leading lanes' rows, the last lane's and
    // the interior pattern (the last interior lane's), each per table k (g a1 a2 b1 b2 pf1 pf2
    // pb1 pb2) and pair j as {h(j), h(16 + j), l(j), l(16 + j)} of the lane's 32 rows; NF is the
    // fewest leading lanes after which every interior lane equals the pattern within 2^-50 of
    // the table's largest value (at most 3, else k_line keeps the operator)
    size_t o_hb = 0;
    int hb_nf = -1;
    if (line_shape_ >= SHAPE_T2A && line_shape_ <= SHAPE_P4S && !ch_.circ && cline_.M == 16 && ch_.M == 16 &&
        d.ns % 32 == 0 && d.nout == d.ns && ch_.nlo <= 16 && ch_.nhi <= 16 && ch_.Pp >= 2 &&
        kLineThreadsCirc % (ch_.Pp / 2) == 0 && ch_.rc.size() >= (size_t)d.ns * 5 &&
        ch_.phf.size() >= (size_t)d.ns * 2 && ch_.phb.size() >= (size_t)d.ns * 2) {
        const int ns = d.ns, PL = ns / 32, tp = std::max(PL - 2, 0);
        auto val = [&](int k, int r) -> double {
            return k < 5 ? ch_.rc[(size_t)r * 5 + k]
                         : (k < 7 ? ch_.phf[(size_t)r * 2 + (k - 5)] : ch_.phb[(size_t)r * 2 + (k - 7)]);
        };
        double tol[9];
        for (int k = 0; k < 9; k++) {
            double mx = 0.0;
            for (int r = 0; r < ns; r++) mx = std::max(mx, std::fabs(val(k, r)));
            tol[k] = std::ldexp(mx, -50);
        }
        auto lane_is_pattern = [&](int t) {
            for (int k = 0; k < 9; k++)
                for (int j = 0; j < 32; j++)
                    if (!(std::fabs(val(k, 32 * t + j) - val(k, 32 * tp + j)) <= tol[k])) return false;
            return true;
        };
        int nf = std::max(1, std::min(PL - 1, 1));  // the first lane always has its own tables
        while (nf < PL - 1 && !lane_is_pattern(nf)) nf++;
        bool ok = nf <= 3;
        for (int t = nf; t < PL - 1 && ok; t++) ok = lane_is_pattern(t);
        if (ok) {
            const int nb = nf + 2;
            std::vector<int> base_row(nb);
            for (int b = 0; b < nf; b++) base_row[b] = 32 * b;
            base_row[nf] = ns - 32;
            base_row[nf + 1] = 32 * tp;
            std::vector<float> tb((size_t)nb * 9 * 16 * 4);
            for (int b = 0; b < nb; b++)
                for (int k = 0; k < 9; k++)
                    for (int j = 0; j < 16; j++) {
                        const F2 a = split(val(k, base_row[b] + j)), c = split(val(k, base_row[b] + 16 + j));
                        float* q = &tb[(((size_t)b * 9 + k) * 16 + j) * 4];
                        q[0] = a.h;
                        q[1] = c.h;
                        q[2] = a.l;
                        q[3] = c.l;
                    }
            o_hb = A.put(tb.data(), tb.size() * sizeof(float));
            hb_nf = nf;
        }
    }
    // register-resident periodic kernel: whole chunks of 32 rows, a power-of-two number of
    // lanes per line; coefficients and fundamental solutions travel in the kernel parameters
    size_t o_rg[4] = {0, 0, 0, 0};
    reg_ok_ = false;
    delete creg_;
    creg_ = nullptr;
    if (line_shape_ != SHAPE_NONE && ch_.circ && d.ns % 32 == 0) {
        const int pr = d.ns / 32;
        ChunkPlanHost cr;
        if (pr >= 1 && pr <= kMaxLanes && (pr & (pr - 1)) == 0 && build_chunk_plan(hp, 32, cr) == PS_OK && cr.ok &&
            cr.P == pr && cr.Pp == pr) {
            creg_ = new RegParams{};
            RegParams& r = *creg_;
            r.ns = cr.ns;
            r.nout = cr.nout;
            r.P = cr.P;
            r.nsteps = cr.nsteps;
            r.xdup = cline_.xdup;
            r.c0 = cline_.c0;
            for (int k = 0; k < kMaxPairs; k++) r.c[k] = cline_.c[k];
            r.ca1 = cline_.ca1;
            r.ca2 = cline_.ca2;
            for (int j = 0; j < 32; j++) {
                r.phf[j][0] = split(cr.phf[(size_t)j * 2]);
                r.phf[j][1] = split(cr.phf[(size_t)j * 2 + 1]);
                r.phb[j][0] = split(cr.phb[(size_t)j * 2]);
                r.phb[j][1] = split(cr.phb[(size_t)j * 2 + 1]);
            }
            auto put = [&](const std::vector<double>& src) {
                std::vector<F2> o(src.size());
                for (size_t k = 0; k < src.size(); k++) o[k] = split(src[k]);
                return A.put(o.data(), o.size() * sizeof(F2));
            };
            o_rg[0] = put(cr.fscan);
            o_rg[1] = put(cr.bscan);
            o_rg[2] = put(cr.fwrap);
            o_rg[3] = put(cr.bwrap);
            reg_ok_ = true;
        }
    }
    const cudaError_t me = cudaMalloc(&dev_, A.host.size());
    if (me != cudaSuccess) {
        dev_ = nullptr;
        return me == cudaErrorMemoryAllocation ? PS_ENOMEM : PS_ECUDA;
    }
    if (cudaMemcpy(dev_, A.host.data(), A.host.size(), cudaMemcpyHostToDevice) != cudaSuccess) return PS_ECUDA;
    unsigned char* base = (unsigned char*)dev_;

    vd_ = PlanView<double>{};
    vd_.m = d.m;
    vd_.nout = d.nout;
    vd_.ns = d.ns;
    vd_.q = d.q;
    vd_.cyclic = d.cyclic;
    vd_.zero = d.zero;
    vd_.identity = d.identity;
    vd_.resid = d.resid;
    vd_.ntap = hp.ntap;
    vd_.nlo = hp.nlo;
    vd_.nhi = hp.nhi;
    vd_.tw = hp.tw;
    vd_.nc = hp.nc;
    for (int t = 0; t < hp.ntap; t++) {
        vd_.io[t] = hp.io[t];
        vd_.ic[t] = hp.ic[t];
    }
    vd_.tidx = (const int*)(base + o_tidx);
    vd_.tc = (const double*)(base + o_tc);
    vd_.lu = (const double*)(base + o_lu);
    vd_.Z = (const double*)(base + o_Z);
    vd_.Cinv = (const double*)(base + o_Ci);
    vd_.wcol = (const int*)(base + o_wcol);
    vd_.wc = (const double*)(base + o_wc);

    if (cok_) {
        for (int v = 0; v < 2; v++) {
            ChunkParams c{};
            c.m = ch_.m;
            c.nout = ch_.nout;
            c.ns = ch_.ns;
            c.P = ch_.P;
            c.Pp = ch_.Pp;
            c.nsteps = ch_.nsteps;
            c.L = ch_.L;
            c.LS = ch_.LS;
            c.has_center = ch_.has_center;
            c.center_off = ch_.center_off;
            c.npair = ch_.npair;
            c.nlo = ch_.nlo;
            c.nhi = ch_.nhi;
            c.tw = ch_.tw;
            c.resid = ch_.resid;
            for (int k = 0; k < kMaxPairs; k++) {
                c.pair_op[k] = ch_.pair_op[k];
                c.pair_om[k] = ch_.pair_om[k];
                c.pair_sign[k] = ch_.pair_sign[k];
                c.pair_c[k] = split(ch_.pair_c[k] * cg);
                if (v == 1) c.pair_c[k].l = 0.0f;
            }
            c.center_c = split(ch_.center_c * cg);
            c.ca1 = split(ch_.circ ? ch_.rc[1] : 0.0);
            c.ca2 = split(ch_.circ ? ch_.rc[2] : 0.0);
            if (v == 1) {
                c.center_c.l = 0.0f;
                c.ca1.l = 0.0f;
                c.ca2.l = 0.0f;
            }
            c.tidx = (const int*)(base + o_ctidx);
            c.tc = (const F2*)(base + o_ctc[v]);
            c.rc = (const F2*)(base + o_rc[v]);
            c.fscan = (const F2*)(base + o_fs[v]);
            c.bscan = (const F2*)(base + o_bs[v]);
            c.fwrap = (const F2*)(base + o_fw[v]);
            c.bwrap = (const F2*)(base + o_bw[v]);
            c.phf = (const F2*)(base + o_pf[v]);
            c.phb = (const F2*)(base + o_pb[v]);
            (v == 0 ? cdf_ : cf32_) = c;
        }
    }

    if (reg_ok_) {
        creg_->fscan = (const F2*)(base + o_rg[0]);
        creg_->bscan = (const F2*)(base + o_rg[1]);
        creg_->fwrap = (const F2*)(base + o_rg[2]);
        creg_->bwrap = (const F2*)(base + o_rg[3]);
    }
    if (line_shape_ != SHAPE_NONE) {
        unsigned char* lb = base;
        const bool own = cline_.M != ch_.M;  // separate chunk tables for the line kernel
        cline_.tidx = cdf_.tidx;
        cline_.tc = cdf_.tc;
        cline_.tcd = (const double*)(base + o_tc);
        cline_.rc = cdf_.rc;
        cline_.fscan = own ? (const F2*)(lb + o_lk[0]) : cdf_.fscan;
        cline_.bscan = own ? (const F2*)(lb + o_lk[1]) : cdf_.bscan;
        cline_.fwrap = own ? (const F2*)(lb + o_lk[2]) : cdf_.fwrap;
        cline_.bwrap = own ? (const F2*)(lb + o_lk[3]) : cdf_.bwrap;
        cline_.phf = own ? (const F2*)(lb + o_lk[4]) : cdf_.phf;
        cline_.phb = own ? (const F2*)(lb + o_lk[5]) : cdf_.phb;
    }
    halfb_ = false;
    if (hb_nf >= 1) {
        chalfb_ = cline_;
        chalfb_.L = kLineThreadsCirc / (ch_.Pp / 2);
        chalfb_.hpair = base + o_hb;
        chalfb_.hnf = hb_nf;
        halfb_ = true;
    }
    half32_ = false;
    if (h32_ok) {
        chalf32_ = cline_;
        chalf32_.M = 32;
        chalf32_.ns = h32.ns;
        chalf32_.nout = h32.nout;
        chalf32_.P = h32.P;
        chalf32_.Pp = h32.Pp;
        chalf32_.nsteps = h32.nsteps;
        chalf32_.L = kLineThreadsCirc / h32.Pp;
        chalf32_.fscan = (const F2*)(base + o_h32[0]);
        chalf32_.bscan = (const F2*)(base + o_h32[1]);
        chalf32_.fwrap = (const F2*)(base + o_h32[2]);
        chalf32_.bwrap = (const F2*)(base + o_h32[3]);
        chalf32_.phf = (const F2*)(base + o_h32[4]);
        chalf32_.phb = (const F2*)(base + o_h32[5]);
        half32_ = true;
    }
    // the same centred periodic operator on the 16-row chunk plan, for the half-chunk kernel
    half16_ = false;
    if (line_shape_ >= SHAPE_T2A && line_shape_ <= SHAPE_P3S && cok_ && ch_.circ && cline_.alias && cline_.M == 32 &&
        ch_.M == 16 && ch_.Pp >= 1 && kLineThreadsCirc % ch_.Pp == 0) {
        chalf16_ = cline_;
        chalf16_.M = 16;
        chalf16_.ns = ch_.ns;
        chalf16_.nout = ch_.nout;
        chalf16_.P = ch_.P;
        chalf16_.Pp = ch_.Pp;
        chalf16_.nsteps = ch_.nsteps;
        chalf16_.L = kLineThreadsCirc / ch_.Pp;
        chalf16_.fscan = cdf_.fscan;
        chalf16_.bscan = cdf_.bscan;
        chalf16_.fwrap = cdf_.fwrap;
        chalf16_.bwrap = cdf_.bwrap;
        chalf16_.phf = cdf_.phf;
        chalf16_.phb = cdf_.phb;
        half16_ = true;
    }
    return PS_OK;
}

// ------------------------------------------------------------------------------------
// launch
// ------------------------------------------------------------------------------------
// Chunk length of the half-chunk kernel on lines that have both plans: PADE_HALF_CHUNK
// (16 or 32, a tuning override); the default is the measured faster one.
constexpr int kHalfChunkDefault = 32;
static int half_chunk_choice() {
    static const int v = [] {
        const char* e = std::getenv("PADE_HALF_CHUNK");
        if (e && std::atoi(e) == 16) return 16;
        if (e && std::atoi(e) == 32) return 32;
        return kHalfChunkDefault;
    }();
    return v;
}

// Which periodic line kernel runs: the register-resident one for the FP32 path; for
// double-float the half-chunk kernel k_lhalf (packed FP32x2 arithmetic) wherever its shapes
// and sizes apply (it measured faster than both others: cd10 x/y 7-11 %, cf90 6-15 % against
// k_line, the staggered z operators ~10 % against the register kernel), else the register
// kernel for tridiagonal operators along strided lines (5-7 % faster than k_line there), else
// the shared-memory k_line (the unrolled pentadiagonal double-float code of the register
// kernel stalls on instruction fetch; contiguous lines stage faster through shared memory).
// PADE_LINE_KERNEL (a tuning override): "reg" the register kernel everywhere, "shared"
// k_line everywhere, "half" k_lhalf wherever it applies (no register kernel).
static int line_kernel_choice() {
    static const int v = [] {
        const char* e = std::getenv("PADE_LINE_KERNEL");
        if (e && std::strcmp(e, "reg") == 0) return 1;
        if (e && std::strcmp(e, "shared") == 0) return 2;
        if (e && std::strcmp(e, "half") == 0) return 3;
        return 0;
    }();
    return v;
}

int launch_lines(const DevicePlan& p, int path, const void* f, void* out, const LineSet& ls, unsigned* status,
                 cudaStream_t s) {
    if (ls.nlines <= 0) return PS_OK;
    const OpDef& d = p.host().def;
    if (d.zero || d.identity) {
        const int th = 128;
        const long bl = (ls.nlines + th - 1) / th;
        if (path == PATH_FP32)
            k_trivial<float><<<(unsigned)bl, th, 0, s>>>(d.zero, d.nout, (const float*)f, (float*)out, ls);
        else
            k_trivial<double><<<(unsigned)bl, th, 0, s>>>(d.zero, d.nout, (const double*)f, (double*)out, ls);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    if (path == PATH_NATIVE) {
        const int th = 128;
        const long bl = (ls.nlines + th - 1) / th;
        k_seq<<<(unsigned)bl, th, 0, s>>>(p.view_d(), (const double*)f, (double*)out, ls);
        return cudaGetLastError() == cudaSuccess ? PS_OK : PS_ECUDA;
    }
    if (!p.chunk_ok()) return PS_ENOTSUP;
    const auto& h = p.chunk_host();
    if (path == PATH_DF) {
        const int sh = p.line_shape();
        const bool tri = sh == SHAPE_T2A || sh == SHAPE_T2S || sh >= SHAPE_T2A_E2C;
        const int choice = line_kernel_choice();
        if ((choice == 0 || choice == 3) && sh >= SHAPE_T2A && sh <= SHAPE_P4S && p.half_band_params()) {
            const int rc = launch_line_half_band(sh, *p.half_band_params(), f, out, ls, status, s);
            if (rc != PS_ENOTSUP) return rc;
        }
        if ((choice == 0 || choice == 3) && sh >= SHAPE_T2A && sh <= SHAPE_T2S_C2E) {
            const StencilParams* h16 = p.half16_params();
            const StencilParams* h32 = p.half32_params();
            const StencilParams* hc = &p.line_params();
            if (h16 && half_chunk_choice() == 16) hc = h16;
            if (h32 && half_chunk_choice() == 32) hc = h32;
            const int rc = launch_line_half(sh, *hc, f, out, ls, status, s);
            if (rc != PS_ENOTSUP) return rc;
        }
        if (p.reg_ok() && (choice == 1 || (choice == 0 && tri && ls.fp != 1))) {
            const int rc = launch_line_reg(sh, p.reg_params(), 0, f, out, ls, status, s);
            if (rc != PS_ENOTSUP) return rc;
        }
        if (sh != SHAPE_NONE) {
            return launch_line(sh, p.line_params(), f, out, ls, status, s);
        }
        return h.M == 16 ? launch_chunk_m<ArDF, 16>(h, p.chunk_df(), f, out, ls, status, s)
                         : launch_chunk_m<ArDF, 32>(h, p.chunk_df(), f, out, ls, status, s);
    }
    if (path == PATH_FP32) {
        if (p.reg_ok() && line_kernel_choice() != 2 && p.line_shape() < SHAPE_T2A_E2C) {
            const int rc = launch_line_reg(p.line_shape(), p.reg_params(), 1, f, out, ls, status, s);
            if (rc != PS_ENOTSUP) return rc;
        }
        if (p.line_shape() != SHAPE_NONE && p.line_shape() < SHAPE_T2A_E2C)
            return launch_line_f32(p.line_shape(), p.line_params(), f, out, ls, status, s);
        return h.M == 16 ? launch_chunk_m<ArF32, 16>(h, p.chunk_f32(), f, out, ls, status, s)
                         : launch_chunk_m<ArF32, 32>(h, p.chunk_f32(), f, out, ls, status, s);
    }
    return PS_EINVAL;
}

}  // namespace pade
