// Chunked line-engine plan construction (see chunkplan.h).
#include "chunkplan.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>

namespace pade {
namespace {

using LD = long double;
using Mat = std::array<LD, 4>;  // 2x2 row-major

Mat eye() { return {1.0L, 0.0L, 0.0L, 1.0L}; }
Mat mul(const Mat& a, const Mat& b) {
    return {a[0] * b[0] + a[1] * b[2], a[0] * b[1] + a[1] * b[3], a[2] * b[0] + a[3] * b[2],
            a[2] * b[1] + a[3] * b[3]};
}
Mat inv(const Mat& a) {
    LD det = a[0] * a[3] - a[1] * a[2];
    return {a[3] / det, -a[1] / det, -a[2] / det, a[0] / det};
}
Mat sub(const Mat& a, const Mat& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]}; }

bool circulant(const OpDef& d) {
    if (!d.cyclic) return false;
    const auto& r0 = d.lhs[0];
    for (int i = 0; i < d.ns; i++)
        for (int k = 0; k < 5; k++)
            if (d.lhs[i][k] != r0[k]) return false;
    return r0[0] == r0[4] && r0[1] == r0[3];
}

// Symmetric spectral factorisation of the circulant symbol
//   a2 z^-2 + a1 z^-1 + d + a1 z + a2 z^2 = c (1 + l1 z^-1 + l2 z^-2)(1 + l1 z + l2 z^2)
// with the zeros of 1 + l1 z + l2 z^2 outside the unit circle.
bool factor_symbol(LD d, LD a1, LD a2, LD& c, LD& l1, LD& l2) {
    using C = std::complex<LD>;
    if (a2 == 0.0L) {
        l2 = 0.0L;
        if (a1 == 0.0L) { l1 = 0.0L; c = d; return d != 0.0L; }
        LD disc = d * d - 4.0L * a1 * a1;
        if (disc <= 0.0L) return false;
        l1 = (d - std::sqrt(disc)) / (2.0L * a1);
        c = a1 / l1;
        return std::fabs(l1) < 1.0L;
    }
    // w = z + 1/z solves a2 w^2 + a1 w + (d - 2 a2) = 0
    C disc = C(a1 * a1 - 4.0L * a2 * (d - 2.0L * a2), 0.0L);
    C sq = std::sqrt(disc);
    C w[2] = {(-C(a1) + sq) / C(2.0L * a2), (-C(a1) - sq) / C(2.0L * a2)};
    C z[2];
    for (int k = 0; k < 2; k++) {
        C s = std::sqrt(w[k] * w[k] - C(4.0L));
        C z1 = (w[k] + s) / C(2.0L), z2 = (w[k] - s) / C(2.0L);
        z[k] = std::abs(z1) > std::abs(z2) ? z1 : z2;
        if (!(std::abs(z[k]) > 1.0L)) return false;
    }
    C L1 = -(C(1.0L) / z[0] + C(1.0L) / z[1]);
    C L2 = C(1.0L) / (z[0] * z[1]);
    l1 = L1.real();
    l2 = L2.real();
    if (std::fabs(L1.imag()) > 1e-12L * (1 + std::fabs(l1)) || std::fabs(L2.imag()) > 1e-12L * (1 + std::fabs(l2)))
        return false;
    c = a2 / l2;
    // verify the factorisation reproduces the symbol
    LD e0 = c * (1.0L + l1 * l1 + l2 * l2) - d, e1 = c * (l1 + l1 * l2) - a1;
    return std::fabs(e0) < 1e-15L * std::fabs(d) + 1e-30L && std::fabs(e1) < 1e-15L * (std::fabs(a1) + 1.0L);
}

int pos_of(int p, int M) { return p + p / M; }

}  // namespace

int build_chunk_plan(const HostPlan& hp, int M, ChunkPlanHost& cp) {
    cp = ChunkPlanHost();
    const OpDef& d = hp.def;
    if (d.zero || d.identity) return PS_OK;
    cp.m = d.m;
    cp.nout = d.nout;
    cp.ns = d.ns;
    cp.resid = d.resid ? 1 : 0;
    cp.Q = d.q;
    cp.M = M;
    cp.P = (d.ns + M - 1) / M;
    if (cp.P > kMaxLanes) return PS_ENOTSUP;
    cp.Pp = 1;
    while (cp.Pp < cp.P) cp.Pp *= 2;
    cp.nsteps = 0;
    while ((1 << cp.nsteps) < cp.Pp) cp.nsteps++;
    cp.L = std::max(1, 256 / cp.Pp);
    // smem positions: chunk padding plus an odd line stride (conflict-free lanes)
    int maxp = std::max(d.m, d.nout);
    cp.LS = pos_of(maxp - 1, M) + 1;
    if (cp.LS % 2 == 0) cp.LS++;

    // interior stencil: detect a centre and antisymmetric / symmetric pairs
    cp.ntap = hp.ntap;
    for (int t = 0; t < hp.ntap; t++) { cp.io[t] = hp.io[t]; cp.ic[t] = hp.ic[t]; }
    {
        int lo = 1 << 30, hi = -(1 << 30);
        for (int t = 0; t < hp.ntap; t++) { lo = std::min(lo, hp.io[t]); hi = std::max(hi, hp.io[t]); }
        int c2 = lo + hi;  // twice the centre
        std::vector<char> used(hp.ntap, 0);
        bool ok = hp.ntap > 0;
        int np = 0;
        for (int t = 0; t < hp.ntap && ok; t++) {
            if (used[t]) continue;
            int o = hp.io[t];
            if (2 * o == c2) {  // centre tap
                if (cp.has_center) { ok = false; break; }
                cp.has_center = 1;
                cp.center_off = o;
                cp.center_c = hp.ic[t];
                used[t] = 1;
                continue;
            }
            int partner = -1;
            for (int u = 0; u < hp.ntap; u++)
                if (!used[u] && u != t && hp.io[u] == c2 - o) partner = u;
            if (partner < 0 || np >= kMaxPairs) { ok = false; break; }
            int tp = o > hp.io[partner] ? t : partner, tm = o > hp.io[partner] ? partner : t;
            double cpv = hp.ic[tp], cmv = hp.ic[tm];
            int sign;
            if (cmv == -cpv) sign = -1;
            else if (cmv == cpv) sign = 1;
            else { ok = false; break; }
            cp.pair_op[np] = hp.io[tp];
            cp.pair_om[np] = hp.io[tm];
            cp.pair_sign[np] = sign;
            cp.pair_c[np] = cpv;
            used[t] = used[partner] = 1;
            np++;
        }
        cp.npair = np;
        cp.use_pairs = ok ? 1 : 0;
    }

    // edge rows (explicit)
    cp.nlo = hp.nlo;
    cp.nhi = hp.nhi;
    cp.tw = hp.tw;
    cp.tidx = hp.tidx;
    cp.tc = hp.tc;

    if (d.q == 0) { cp.ok = 1; return PS_OK; }

    // ---- recurrence coefficients ----
    const int ns = d.ns;
    std::vector<std::array<LD, 5>> rc(ns);  // g, a1, a2, b1, b2
    if (d.cyclic) {
        if (!circulant(d)) return PS_ENOTSUP;
        LD c, l1, l2;
        if (!factor_symbol(d.lhs[0][2], d.lhs[0][3], d.lhs[0][4], c, l1, l2)) return PS_ENOTSUP;
        cp.circ = 1;
        cp.cg = (double)(1.0L / c);
        cp.ca1 = (double)l1;
        cp.ca2 = (double)l2;
        for (int i = 0; i < ns; i++) rc[i] = {1.0L / c, l1, l2, l1, l2};
    } else {
        // no-pivot band LU of A (long double), folded as described in chunkplan.h
        std::vector<std::array<LD, 5>> U(ns);
        for (int i = 0; i < ns; i++)
            for (int o = -2; o <= 2; o++) {
                int j = i + o;
                U[i][o + 2] = (j >= 0 && j < ns && std::abs(o) <= d.q) ? (LD)d.lhs[i][o + 2] : 0.0L;
            }
        std::vector<std::array<LD, 2>> Lm(ns, {0.0L, 0.0L});
        for (int k = 0; k < ns; k++) {
            LD piv = U[k][2];
            if (piv == 0.0L) return PS_EINVAL;
            for (int r = k + 1; r <= std::min(k + d.q, ns - 1); r++) {
                LD a = U[r][k - r + 2];
                if (a == 0.0L) continue;
                LD l = a / piv;
                Lm[r][r - k - 1] = l;
                for (int cc = k; cc <= std::min(k + d.q, ns - 1); cc++) U[r][cc - r + 2] -= l * U[k][cc - k + 2];
            }
        }
        for (int i = 0; i < ns; i++) {
            LD di = U[i][2];
            LD g = 1.0L / di;
            LD a1 = i >= 1 ? Lm[i][0] * U[i - 1][2] / di : 0.0L;
            LD a2 = i >= 2 ? Lm[i][1] * U[i - 2][2] / di : 0.0L;
            LD b1 = i + 1 < ns ? U[i][3] / di : 0.0L;
            LD b2 = i + 2 < ns ? U[i][4] / di : 0.0L;
            rc[i] = {g, a1, a2, b1, b2};
        }
    }
    cp.rc.resize((size_t)ns * 5);
    for (int i = 0; i < ns; i++)
        for (int k = 0; k < 5; k++) cp.rc[(size_t)i * 5 + k] = (double)rc[i][k];

    // ---- chunk transfers ----
    const int P = cp.P, Pp = cp.Pp;
    std::vector<Mat> Phi(Pp, eye()), The(Pp, eye());
    for (int t = 0; t < P; t++) {
        int s = t * M, e = std::min(ns, s + M);
        Mat F = eye();
        for (int i = s; i < e; i++) {
            Mat Ci = {-rc[i][1], -rc[i][2], 1.0L, 0.0L};
            F = mul(Ci, F);
        }
        Phi[t] = F;
        Mat B = eye();
        for (int i = e - 1; i >= s; i--) {
            Mat Di = {-rc[i][3], -rc[i][4], 1.0L, 0.0L};
            B = mul(Di, B);
        }
        The[t] = B;
    }
    const int K = cp.nsteps;
    cp.fscan.assign((size_t)Pp * kMaxSteps * 4, 0.0);
    cp.bscan.assign((size_t)Pp * kMaxSteps * 4, 0.0);
    for (int t = 0; t < Pp; t++)
        for (int k = 0; k < K; k++) {
            int w = 1 << k;
            Mat F = eye();
            if (t >= w)
                for (int u = t - w + 1; u <= t; u++) F = mul(Phi[u], F);
            Mat B = eye();
            if (t + w < Pp)
                for (int u = t + w - 1; u >= t; u--) B = mul(The[u], B);
            for (int x = 0; x < 4; x++) {
                cp.fscan[((size_t)t * kMaxSteps + k) * 4 + x] = (double)F[x];
                cp.bscan[((size_t)t * kMaxSteps + k) * 4 + x] = (double)B[x];
            }
        }
    // fundamental solutions within chunks
    if (cp.circ) {
        cp.phf.assign((size_t)M * 2, 0.0);
        cp.phb.assign((size_t)M * 2, 0.0);
        Mat F = eye(), B = eye();
        for (int j = 0; j < M; j++) {
            Mat Ci = {-rc[0][1], -rc[0][2], 1.0L, 0.0L};
            F = mul(Ci, F);
            cp.phf[(size_t)j * 2] = (double)F[0];
            cp.phf[(size_t)j * 2 + 1] = (double)F[1];
            Mat Di = {-rc[0][3], -rc[0][4], 1.0L, 0.0L};
            B = mul(Di, B);
            cp.phb[(size_t)j * 2] = (double)B[0];
            cp.phb[(size_t)j * 2 + 1] = (double)B[1];
        }
    } else {
        cp.phf.assign((size_t)ns * 2, 0.0);
        cp.phb.assign((size_t)ns * 2, 0.0);
        for (int t = 0; t < P; t++) {
            int s0 = t * M, e0 = std::min(ns, s0 + M);
            Mat F = eye();
            for (int i = s0; i < e0; i++) {
                Mat Ci = {-rc[i][1], -rc[i][2], 1.0L, 0.0L};
                F = mul(Ci, F);
                cp.phf[(size_t)i * 2] = (double)F[0];
                cp.phf[(size_t)i * 2 + 1] = (double)F[1];
            }
            Mat B = eye();
            for (int i = e0 - 1; i >= s0; i--) {
                Mat Di = {-rc[i][3], -rc[i][4], 1.0L, 0.0L};
                B = mul(Di, B);
                cp.phb[(size_t)i * 2] = (double)B[0];
                cp.phb[(size_t)i * 2 + 1] = (double)B[1];
            }
        }
    }
    cp.fwrap.assign((size_t)Pp * 4, 0.0);
    cp.bwrap.assign((size_t)Pp * 4, 0.0);
    if (cp.circ) {
        Mat Pi = eye(), Pi2 = eye();
        for (int t = 0; t < P; t++) Pi = mul(Phi[t], Pi);        // Phi_{P-1} ... Phi_0
        for (int t = P - 1; t >= 0; t--) Pi2 = mul(The[t], Pi2);  // Theta_0 ... Theta_{P-1}
        Mat Wf = inv(sub(eye(), Pi)), Wb = inv(sub(eye(), Pi2));
        Mat acc = eye();
        for (int t = 0; t < P; t++) {
            Mat Ps = mul(acc, Wf);
            for (int x = 0; x < 4; x++) cp.fwrap[(size_t)t * 4 + x] = (double)Ps[x];
            acc = mul(Phi[t], acc);
        }
        acc = eye();
        for (int t = P - 1; t >= 0; t--) {
            Mat Ps = mul(acc, Wb);
            for (int x = 0; x < 4; x++) cp.bwrap[(size_t)t * 4 + x] = (double)Ps[x];
            acc = mul(The[t], acc);
        }
    }
    cp.ok = 1;
    return PS_OK;
}

}  // namespace pade
