// Device-plan construction for compact line operators (see plan.h).
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <map>

namespace pade {
namespace {

using LD = long double;

std::vector<std::pair<int, double>> canon(const LinForm& a) {
    std::map<int, double> m;
    for (auto& p : a.t) m[p.first] += p.second;
    std::vector<std::pair<int, double>> r;
    for (auto& p : m)
        if (p.second != 0.0) r.push_back(p);
    return r;
}

bool close(double a, double b) { return std::fabs(a - b) <= 4e-16 * std::max(std::fabs(a), std::fabs(b)); }

// stencil row i with direct indices; false if any tap leaves [0, m)
bool stencil_direct(const HostPlan& p, int i, std::vector<std::pair<int, double>>& out) {
    std::map<int, double> m;
    for (int t = 0; t < p.ntap; t++) {
        int j = i + p.io[t];
        if (j < 0 || j >= p.def.m) return false;
        m[j] += p.ic[t];
    }
    out.clear();
    for (auto& q : m)
        if (q.second != 0.0) out.push_back(q);
    return true;
}

bool same_row(const std::vector<std::pair<int, double>>& a, const std::vector<std::pair<int, double>>& b) {
    if (a.size() != b.size()) return false;
    for (size_t k = 0; k < a.size(); k++)
        if (a[k].first != b[k].first || !close(a[k].second, b[k].second)) return false;
    return true;
}

}  // namespace

int build_plan(const OpDef& d, HostPlan& p) {
    p = HostPlan();
    p.def = d;
    if (d.zero || d.identity) return PS_OK;
    const int ns = d.ns, q = d.q;
    if ((int)d.io.size() > kMaxTap || d.io.size() != d.ic.size()) return PS_EINVAL;
    p.ntap = (int)d.io.size();
    p.io = d.io;
    p.ic = d.ic;
    std::vector<LinForm> rhs = d.rhs;
    if (d.resid) {
        // residual form: rows of R = A - B and the interior stencil of A - B
        if (d.m != ns || d.nout != ns) return PS_EINVAL;
        for (int i = 0; i < ns; i++) {
            LinForm a;
            for (int o = -2; o <= 2; o++) {
                double v = d.lhs[i][o + 2];
                if (v == 0.0) continue;
                int j = i + o;
                if (d.cyclic) j = ((j % ns) + ns) % ns;
                else if (j < 0 || j >= ns) continue;
                a = a + LinForm(j, v);
            }
            rhs[i] = a - d.rhs[i];
        }
        const auto& mid = d.lhs[ns / 2];
        std::map<int, double> st;
        for (int t = 0; t < p.ntap; t++) st[d.io[t]] -= d.ic[t];
        for (int o = -2; o <= 2; o++)
            if (mid[o + 2] != 0.0) st[o] += mid[o + 2];
        p.io.clear();
        p.ic.clear();
        for (auto& kv : st) {
            p.io.push_back(kv.first);
            p.ic.push_back(kv.second);
        }
        p.ntap = (int)p.io.size();
        if (p.ntap > kMaxTap) return PS_EINVAL;
    }

    // ---- RHS: which rows follow the interior stencil with direct indexing ----
    std::vector<char> reg(ns, 0);
    std::vector<std::vector<std::pair<int, double>>> rows(ns);
    std::vector<std::pair<int, double>> st;
    for (int i = 0; i < ns; i++) {
        rows[i] = canon(rhs[i]);
        reg[i] = stencil_direct(p, i, st) && same_row(rows[i], st);
    }
    int first = -1, last = -1;
    for (int i = 0; i < ns; i++)
        if (reg[i]) { if (first < 0) first = i; last = i; }
    bool contiguous = first >= 0;
    for (int i = first; contiguous && i <= last; i++) contiguous = reg[i];
    if (contiguous) { p.nlo = first; p.nhi = ns - 1 - last; }
    else { p.nlo = ns; p.nhi = 0; }
    int nt = p.nlo + p.nhi;
    p.tw = 1;
    auto trow = [&](int t) { return t < p.nlo ? t : ns - p.nhi + (t - p.nlo); };
    for (int t = 0; t < nt; t++) p.tw = std::max<int>(p.tw, (int)rows[trow(t)].size());
    p.tidx.assign((size_t)std::max(nt, 1) * p.tw, 0);
    p.tc.assign((size_t)std::max(nt, 1) * p.tw, 0.0);
    for (int t = 0; t < nt; t++) {
        auto& r = rows[trow(t)];
        for (size_t k = 0; k < r.size(); k++) {
            p.tidx[(size_t)t * p.tw + k] = r[k].first;
            p.tc[(size_t)t * p.tw + k] = r[k].second;
        }
    }

    // ---- LHS: no-pivot band LU of the non-cyclic part A0 ----
    p.lu.assign((size_t)ns * 5, 0.0);
    if (q == 0) {
        for (int i = 0; i < ns; i++) p.lu[(size_t)i * 5 + 4] = 1.0;
        return PS_OK;
    }
    // band storage U[i][o+2] for o in -2..2 (entries of A0)
    std::vector<std::array<LD, 5>> U(ns);
    for (int i = 0; i < ns; i++)
        for (int o = -2; o <= 2; o++) {
            int j = i + o;
            U[i][o + 2] = (j >= 0 && j < ns && std::abs(o) <= q) ? (LD)d.lhs[i][o + 2] : 0.0L;
        }
    std::vector<std::array<LD, 2>> Lm(ns, {0.0L, 0.0L});
    for (int k = 0; k < ns; k++) {
        LD piv = U[k][2];
        if (piv == 0.0L) return PS_EINVAL;
        for (int r = k + 1; r <= std::min(k + q, ns - 1); r++) {
            LD a = U[r][k - r + 2];
            if (a == 0.0L) continue;
            LD l = a / piv;
            Lm[r][r - k - 1] = l;
            for (int c = k; c <= std::min(k + q, ns - 1); c++) U[r][c - r + 2] -= l * U[k][c - k + 2];
        }
    }
    for (int i = 0; i < ns; i++) {
        p.lu[(size_t)i * 5 + 0] = (double)Lm[i][0];
        p.lu[(size_t)i * 5 + 1] = (double)Lm[i][1];
        p.lu[(size_t)i * 5 + 2] = (double)U[i][3];
        p.lu[(size_t)i * 5 + 3] = (double)U[i][4];
        p.lu[(size_t)i * 5 + 4] = (double)(1.0L / U[i][2]);
    }
    if (!d.cyclic) return PS_OK;

    // ---- cyclic corners: A = A0 + E W^T, Woodbury with Z = A0^-1 E ----
    std::vector<int> crow;
    for (int i = 0; i < ns; i++) {
        bool wraps = false;
        for (int o = -q; o <= q; o++) {
            int j = i + o;
            if ((j < 0 || j >= ns) && d.lhs[i][o + 2] != 0.0) wraps = true;
        }
        if (wraps) crow.push_back(i);
    }
    p.nc = (int)crow.size();
    if (p.nc > kMaxNc) return PS_EINVAL;
    p.wcol.assign((size_t)std::max(p.nc, 1) * q, 0);
    p.wc.assign((size_t)std::max(p.nc, 1) * q, 0.0);
    for (int c = 0; c < p.nc; c++) {
        int i = crow[c], t = 0;
        for (int o = -q; o <= q; o++) {
            int j = i + o;
            if ((j < 0 || j >= ns) && d.lhs[i][o + 2] != 0.0) {
                p.wcol[(size_t)c * q + t] = ((j % ns) + ns) % ns;
                p.wc[(size_t)c * q + t] = d.lhs[i][o + 2];
                t++;
            }
        }
    }
    // solve A0 z = e_{crow[c]} in long double with the factors above
    std::vector<LD> Zl((size_t)ns * p.nc);
    for (int c = 0; c < p.nc; c++) {
        std::vector<LD> y(ns, 0.0L);
        y[crow[c]] = 1.0L;
        for (int i = 0; i < ns; i++) {
            LD v = y[i];
            if (i >= 1) v -= Lm[i][0] * y[i - 1];
            if (i >= 2) v -= Lm[i][1] * y[i - 2];
            y[i] = v;
        }
        for (int i = ns - 1; i >= 0; i--) {
            LD v = y[i];
            if (i + 1 < ns) v -= U[i][3] * y[i + 1];
            if (i + 2 < ns) v -= U[i][4] * y[i + 2];
            y[i] = v / U[i][2];
        }
        for (int i = 0; i < ns; i++) Zl[(size_t)i * p.nc + c] = y[i];
    }
    // capacitance C = I + W^T Z and its inverse (Gauss-Jordan with partial pivoting)
    const int nc = p.nc;
    std::vector<LD> C((size_t)nc * nc, 0.0L), Ci((size_t)nc * nc, 0.0L);
    for (int a = 0; a < nc; a++) {
        Ci[(size_t)a * nc + a] = 1.0L;
        for (int b = 0; b < nc; b++) {
            LD s = (a == b) ? 1.0L : 0.0L;
            for (int t = 0; t < q; t++) s += (LD)p.wc[(size_t)a * q + t] * Zl[(size_t)p.wcol[(size_t)a * q + t] * nc + b];
            C[(size_t)a * nc + b] = s;
        }
    }
    for (int c = 0; c < nc; c++) {
        int pv = c;
        for (int r = c + 1; r < nc; r++)
            if (fabsl(C[(size_t)r * nc + c]) > fabsl(C[(size_t)pv * nc + c])) pv = r;
        if (C[(size_t)pv * nc + c] == 0.0L) return PS_EINVAL;
        for (int j = 0; j < nc; j++) {
            std::swap(C[(size_t)pv * nc + j], C[(size_t)c * nc + j]);
            std::swap(Ci[(size_t)pv * nc + j], Ci[(size_t)c * nc + j]);
        }
        LD inv = 1.0L / C[(size_t)c * nc + c];
        for (int j = 0; j < nc; j++) { C[(size_t)c * nc + j] *= inv; Ci[(size_t)c * nc + j] *= inv; }
        for (int r = 0; r < nc; r++) {
            if (r == c) continue;
            LD l = C[(size_t)r * nc + c];
            for (int j = 0; j < nc; j++) { C[(size_t)r * nc + j] -= l * C[(size_t)c * nc + j]; Ci[(size_t)r * nc + j] -= l * Ci[(size_t)c * nc + j]; }
        }
    }
    p.Z.resize(Zl.size());
    for (size_t k = 0; k < Zl.size(); k++) p.Z[k] = (double)Zl[k];
    p.Cinv.resize(Ci.size());
    for (size_t k = 0; k < Ci.size(); k++) p.Cinv[k] = (double)Ci[k];
    return PS_OK;
}

void host_apply_line(const HostPlan& p, const double* f, long fs, double* out, long os) {
    const OpDef& d = p.def;
    if (d.zero) { for (int i = 0; i < d.nout; i++) out[i * os] = 0.0; return; }
    if (d.identity) { for (int i = 0; i < d.nout; i++) out[i * os] = f[i * fs]; return; }
    const int ns = d.ns;
    for (int i = 0; i < ns; i++) {
        double r = 0.0;
        if (i < p.nlo || i >= ns - p.nhi) {
            int t = i < p.nlo ? i : p.nlo + (i - (ns - p.nhi));
            for (int k = 0; k < p.tw; k++) r += p.tc[(size_t)t * p.tw + k] * f[p.tidx[(size_t)t * p.tw + k] * fs];
        } else {
            for (int k = 0; k < p.ntap; k++) r += p.ic[k] * f[(i + p.io[k]) * fs];
        }
        out[i * os] = r;
    }
    if (d.q > 0) {
        for (int i = 1; i < ns; i++) {
            double v = out[i * os] - p.lu[i * 5 + 0] * out[(i - 1) * os];
            if (i >= 2) v -= p.lu[i * 5 + 1] * out[(i - 2) * os];
            out[i * os] = v;
        }
        for (int i = ns - 1; i >= 0; i--) {
            double v = out[i * os];
            if (i + 1 < ns) v -= p.lu[i * 5 + 2] * out[(i + 1) * os];
            if (i + 2 < ns) v -= p.lu[i * 5 + 3] * out[(i + 2) * os];
            out[i * os] = v * p.lu[i * 5 + 4];
        }
        if (p.nc) {
            double g[kMaxNc], h[kMaxNc];
            for (int c = 0; c < p.nc; c++) {
                g[c] = 0.0;
                for (int t = 0; t < d.q; t++) g[c] += p.wc[c * d.q + t] * out[p.wcol[c * d.q + t] * os];
            }
            for (int a = 0; a < p.nc; a++) {
                h[a] = 0.0;
                for (int b = 0; b < p.nc; b++) h[a] += p.Cinv[a * p.nc + b] * g[b];
            }
            for (int i = 0; i < ns; i++) {
                double v = out[i * os];
                for (int c = 0; c < p.nc; c++) v -= p.Z[(size_t)i * p.nc + c] * h[c];
                out[i * os] = v;
            }
        }
    }
    if (d.resid)
        for (int i = 0; i < ns; i++) out[i * os] = f[i * fs] - out[i * os];
    for (int i = ns; i < d.nout; i++) out[i * os] = out[(i - ns) * os];
}

}  // namespace pade
