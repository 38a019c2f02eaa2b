// Code generator: turns a PDF tree into one CUDA source holding a fused
// kernel set, compiled at run time for sm_103a.
//
// This replaces the reference's per-event pointer chase (MetricTaker ->
// callFunction -> d_function_table, src/PDFs/MetricTaker.cu:17-44,
// src/PDFs/GooPdf.cu:398-400) with straight-line code for the whole tree,
// and carries forward-mode derivatives for the parameters marked in the
// gradient mask (the adjoint of the NLL sum is a plain sum of per-event
// derivatives, so a forward tangent per parameter is exact and cheap).
//
// Kernels per tree and per variant (_g with gradient, _n without):
//   gf_conv_*  ConvolutionPdf workspaces + table T[k] = sum_m M[m] R[m+off-k]
//              (device_ConvolvePdfs, src/PDFs/combine/ConvolutionPdf.cu:27-75,
//              whose value depends on x only through k(x))
//   gf_grid_*  numeric normalisation grid sums (GooPdf::reduce_with_bins,
//              src/PDFs/GooPdf.cu:83-108), one CTA row per numeric node
//   gf_evt_*   event pass: per-event -log(P*norm), FP64 block reduction and a
//              last-CTA finish per toy (GooPdf::reduce_with_metric,
//              src/PDFs/GooPdf.cu:45-78, calculateNLL src/PDFs/MetricPointer.cu:13-16)
//   gf_val_n   per-event metric values (GooPdf::evaluate_with_metric,
//              src/PDFs/GooPdf.cu:112-173)
#include "tree.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <functional>
#include <map>
#include <sstream>
#include <stdexcept>

namespace gf {

namespace {

std::string lit(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%.17g", v);
    std::string s(b);
    if(s.find_first_of(".eEn") == std::string::npos)
        s += ".0";
    return s;
}

struct Val {
    std::string v;
    std::map<int, std::string> g; // gradient slot -> expression (a variable name)
};

struct Ctx {
    std::ostream &os;
    const Tree &T;
    bool grad;
    bool event; // event context: norms of non-forced nodes are live variables
    std::function<std::string(int)> x;           // observable -> expression
    std::function<std::string(int)> k;           // conv index -> int expression
    std::function<std::string(int, int)> tab;    // conv index, component -> expression
    std::vector<int> *xused;
    std::function<std::string(int, int)> amp; // amplitude node, amplitude -> R2 amplitude expression
    std::function<std::string(int)> ampcol;   // amplitude / derivative column -> R2 expression
    bool lohi = false;                        // normalisation factors as FP32 hi + lo pairs
    bool single = false;                      // R is FP32 (mixed engine): divisions by parameters become products
    // the root, when it is an amplitude PDF: |T|^2 = tr^2 + ti^2 and, per gradient slot, the inner term
    // d|T|^2/dp / 2 (its gradient divided by the value needs no efficiency)
    bool ampRoot = false;
    std::string ampTr, ampTi;
    std::map<int, std::string> ampInner;
    int uid = 0;
    std::string tmp(const char *p) { return std::string(p) + std::to_string(uid++); }
};

std::string P(int j) { return "p" + std::to_string(j); }

std::string normExpr(Ctx &c, int i) {
    if(c.T.nk[i] == NK_ONE)
        return "";
    if(!c.event)
        throw std::runtime_error("codegen: non-unit norm referenced outside the event pass");
    return "N" + std::to_string(i);
}
// x times the normalisation factor of node i (x itself for unit factors): x * (hi + lo) with one rounding
std::string normMul(Ctx &c, int i, const std::string &x) {
    std::string ne = normExpr(c, i);
    if(ne.empty())
        return x;
    if(c.lohi)
        return "gf_nm(" + x + ", N" + std::to_string(i) + ", NL" + std::to_string(i) + ")";
    return "(" + x + " * " + ne + ")";
}
std::string dnormExpr(Ctx &c, int i, int s) {
    const auto &d = c.T.dep_norm[i];
    if(std::find(d.begin(), d.end(), s) == d.end())
        return "";
    return "dN" + std::to_string(i) + "_" + std::to_string(s);
}

void gadd(Ctx &c, Val &v, int s, const std::string &e) {
    if(s < 0 || !c.grad)
        return;
    auto it = v.g.find(s);
    if(it == v.g.end())
        v.g[s] = "(" + e + ")";
    else
        it->second = "(" + it->second + " + " + e + ")";
}

int slot(Ctx &c, int param) { return c.T.gslot[param]; }

// Finalises gradient expressions into named registers.
void materialise(Ctx &c, Val &v) {
    if(!c.grad)
        return;
    for(auto &kv : v.g) {
        std::string n = c.tmp("g");
        c.os << "    const R " << n << " = " << kv.second << ";\n";
        kv.second = n;
    }
}

// x^n for small integer n >= 0 by repeated multiplication.
std::string powi(Ctx &c, const std::string &x, int n) {
    if(n == 0)
        return "R(1)";
    std::string r = x;
    for(int i = 1; i < n; ++i)
        r = "(" + r + " * " + x + ")";
    return r;
}

Val emit(Ctx &c, int i) {
    const TNode &n = c.T.nodes[i];
    Val out;
    std::ostream &os = c.os;
    switch(n.op) {
    case GF_OP_EXP: {
        std::string x = c.x(n.obs[0]), v = c.tmp("v");
        os << "    const R " << v << " = GF_EXP(" << P(n.params[0]) << " * " << x << ");\n";
        out.v = v;
        gadd(c, out, slot(c, n.params[0]), x + " * " + v);
        break;
    }
    case GF_OP_EXP_OFFSET: {
        std::string x = c.x(n.obs[0]), d = c.tmp("d"), v = c.tmp("v");
        os << "    const R " << d << " = " << x << " - " << P(n.params[0]) << ";\n";
        os << "    const R " << v << " = GF_EXP(" << P(n.params[1]) << " * " << d << ");\n";
        out.v = v;
        gadd(c, out, slot(c, n.params[1]), d + " * " + v);
        gadd(c, out, slot(c, n.params[0]), "-" + P(n.params[1]) + " * " + v);
        break;
    }
    case GF_OP_EXP_POLY:
    case GF_OP_EXP_POLY_OFFSET: {
        bool off      = n.op == GF_OP_EXP_POLY_OFFSET;
        size_t first  = off ? 1 : 0;
        std::string x = c.x(n.obs[0]), d = c.tmp("d"), a = c.tmp("a"), v = c.tmp("v");
        if(off)
            os << "    const R " << d << " = " << x << " - " << P(n.params[0]) << ";\n";
        else
            os << "    const R " << d << " = " << x << ";\n";
        os << "    R " << a << " = R(0);\n";
        std::vector<std::string> pw;
        for(size_t k = 0; k < n.params.size(); ++k) {
            std::string q = c.tmp("q");
            os << "    const R " << q << " = " << powi(c, d, (int)k) << ";\n";
            pw.push_back(q);
            if(k >= first)
                os << "    " << a << " += " << q << " * " << P(n.params[k]) << ";\n";
        }
        os << "    const R " << v << " = GF_EXP(" << a << ");\n";
        out.v = v;
        for(size_t k = first; k < n.params.size(); ++k)
            gadd(c, out, slot(c, n.params[k]), pw[k] + " * " + v);
        if(off && slot(c, n.params[0]) >= 0) {
            std::string s = "R(0)";
            for(size_t k = 1; k < n.params.size(); ++k)
                s += " + R(" + std::to_string(k) + ") * " + P(n.params[k]) + " * " + pw[k - 1];
            gadd(c, out, slot(c, n.params[0]), "-" + v + " * (" + s + ")");
        }
        break;
    }
    case GF_OP_GAUSSIAN: {
        std::string x = c.x(n.obs[0]), d = c.tmp("d"), s = c.tmp("s"), v = c.tmp("v");
        os << "    const R " << d << " = " << x << " - " << P(n.params[0]) << ";\n";
        os << "    const R " << s << " = " << P(n.params[1]) << ";\n";
        if(c.single) {
            // single precision: the reciprocals of sigma^2 and sigma^3 depend on the parameter only, so that a
            // loop over bins or events hoists them and multiplies (three IEEE divisions per value made the
            // convolution's resolution staging the longest step of a one-launch FCN)
            const std::string iq = c.tmp("iq"), iqs = c.tmp("iqs");
            os << "    const R " << iq << " = R(1) / (" << s << " * " << s << ");\n";
            os << "    const R " << iqs << " = " << iq << " / " << s << ";\n";
            os << "    const R " << v << " = GF_EXP(R(-0.5) * " << d << " * " << d << " * " << iq << ");\n";
            out.v = v;
            gadd(c, out, slot(c, n.params[0]), v + " * " + d + " * " + iq);
            gadd(c, out, slot(c, n.params[1]), v + " * " + d + " * " + d + " * " + iqs);
        } else {
            os << "    const R " << v << " = GF_EXP(R(-0.5) * " << d << " * " << d << " / (" << s << " * " << s
               << "));\n";
            out.v = v;
            gadd(c, out, slot(c, n.params[0]), v + " * " + d + " / (" + s + " * " + s + ")");
            gadd(c, out, slot(c, n.params[1]), v + " * " + d + " * " + d + " / (" + s + " * " + s + " * " + s + ")");
        }
        break;
    }
    case GF_OP_POLYNOMIAL:
    case GF_OP_POLYNOMIAL_OFFSET: {
        bool off  = n.op == GF_OP_POLYNOMIAL_OFFSET;
        int L     = (int)n.consts[0];
        size_t k0 = off ? 2 : 0;
        std::string v = c.tmp("v");
        os << "    R " << v << " = R(0);\n";
        bool needX = false;
        for(size_t k = k0; k < n.params.size(); ++k)
            needX |= (L + (int)(k - k0)) != 0;
        std::string x = needX ? c.x(n.obs[0]) : "";
        for(size_t k = k0; k < n.params.size(); ++k) {
            int e         = L + (int)(k - k0);
            std::string q = c.tmp("q");
            os << "    const R " << q << " = " << powi(c, x, e) << ";\n";
            os << "    " << v << " += " << P(n.params[k]) << " * " << q << ";\n";
            gadd(c, out, slot(c, n.params[k]), q);
        }
        out.v = v;
        break;
    }
    case GF_OP_ADD:
    case GF_OP_ADD_EXT: {
        bool ext = n.op == GF_OP_ADD_EXT;
        std::vector<Val> ch;
        for(int cidx : n.children)
            ch.push_back(emit(c, cidx));
        std::string tw = c.tmp("tw"), v = c.tmp("v");
        os << "    R " << tw << " = R(0);\n";
        for(size_t k = 0; k < n.params.size(); ++k)
            os << "    " << tw << " += " << P(n.params[k]) << ";\n";
        std::vector<std::string> u; // weight-free normalised child values v_c * N_c
        for(size_t k = 0; k < ch.size(); ++k)
            u.push_back(normMul(c, n.children[k], ch[k].v));
        os << "    R " << v << " = R(0);\n";
        size_t nw = ext ? ch.size() : ch.size() - 1;
        for(size_t k = 0; k < nw; ++k)
            os << "    " << v << " += " << normMul(c, n.children[k], "(" + P(n.params[k]) + " * " + ch[k].v + ")")
               << ";\n";
        if(!ext) {
            os << "    " << v << " += "
               << normMul(c, n.children.back(), "((R(1) - " + tw + ") * " + ch.back().v + ")") << ";\n";
        } else {
            os << "    " << v << " /= " << tw << ";\n";
        }
        out.v = v;
        if(c.grad) {
            // derivative of child k's normalised value for slot s
            auto du = [&](size_t k, int s) -> std::string {
                int cn = n.children[k];
                std::string r;
                auto it = ch[k].g.find(s);
                std::string ne = normExpr(c, cn), dn = dnormExpr(c, cn, s);
                if(it != ch[k].g.end())
                    r = ne.empty() ? it->second : it->second + " * " + ne;
                if(!dn.empty())
                    r += (r.empty() ? "" : " + ") + ch[k].v + " * " + dn;
                return r;
            };
            for(int s : c.T.dep_val[i]) {
                std::string e;
                for(size_t k = 0; k < ch.size(); ++k) {
                    std::string d = du(k, s);
                    if(d.empty())
                        continue;
                    std::string w;
                    if(k < nw)
                        w = P(n.params[k]);
                    else
                        w = "(R(1) - " + tw + ")";
                    e += (e.empty() ? "" : " + ") + w + " * (" + d + ")";
                }
                if(ext && !e.empty())
                    e = "(" + e + ") / " + tw;
                if(!e.empty())
                    gadd(c, out, s, e);
            }
            for(size_t k = 0; k < n.params.size(); ++k) {
                int s = slot(c, n.params[k]);
                if(s < 0)
                    continue;
                if(ext)
                    gadd(c, out, s, "(" + u[k] + " - " + v + ") / " + tw);
                else
                    gadd(c, out, s, u[k] + " - " + u.back());
            }
        }
        break;
    }
    case GF_OP_PROD: {
        std::vector<Val> ch;
        for(int cidx : n.children)
            ch.push_back(emit(c, cidx));
        std::vector<std::string> u;
        for(size_t k = 0; k < ch.size(); ++k) {
            std::string un = c.tmp("u");
            os << "    const R " << un << " = " << normMul(c, n.children[k], ch[k].v) << ";\n";
            u.push_back(un);
        }
        std::string v = c.tmp("v");
        os << "    R " << v << " = R(1);\n";
        for(auto &un : u)
            os << "    " << v << " *= " << un << ";\n";
        out.v = v;
        if(c.grad)
            for(int s : c.T.dep_val[i]) {
                std::string e;
                for(size_t k = 0; k < ch.size(); ++k) {
                    int cn = n.children[k];
                    std::string d;
                    auto it = ch[k].g.find(s);
                    std::string ne = normExpr(c, cn), dn = dnormExpr(c, cn, s);
                    if(it != ch[k].g.end())
                        d = ne.empty() ? it->second : it->second + " * " + ne;
                    if(!dn.empty())
                        d += (d.empty() ? "" : " + ") + ch[k].v + " * " + dn;
                    if(d.empty())
                        continue;
                    std::string rest;
                    for(size_t j = 0; j < u.size(); ++j)
                        if(j != k)
                            rest += " * " + u[j];
                    e += (e.empty() ? "" : " + ") + std::string("(") + d + ")" + rest;
                }
                if(!e.empty())
                    gadd(c, out, s, e);
            }
        break;
    }
    case GF_OP_CONVOLUTION: {
        int ci = c.T.conv_of[i];
        std::string v = c.tmp("v");
        os << "    const R " << v << " = " << c.tab(ci, 0) << ";\n";
        out.v = v;
        if(c.grad) {
            const auto &dep = c.T.convs[ci].dep;
            for(size_t j = 0; j < dep.size(); ++j)
                gadd(c, out, dep[j], c.tab(ci, 1 + (int)j));
        }
        break;
    }
    case GF_OP_MULTIPOLYNOMIAL: {
        // device_MultiPolynomial (src/PDFs/basic/PolynomialPdf.cu:46-107): sum over the monomials of total
        // degree <= maxDegree, coefficients in the order the box index enumerates them
        const int nO = (int)n.obs.size(), deg = (int)n.consts[0] + 1;
        std::vector<std::string> d(nO);
        for(int j = 0; j < nO; ++j) {
            // x_j is read only when some monomial has a positive power of it
            bool used   = false;
            int64_t bx  = 1;
            for(int k = 0; k < nO; ++k)
                bx *= deg;
            for(int64_t b = 1; b < bx && !used; ++b) {
                int64_t ci = b;
                int sum = 0, pj = 0;
                for(int k = 0; k < nO; ++k) {
                    const int pk = (int)(ci % deg);
                    ci /= deg;
                    sum += pk;
                    if(k == j)
                        pj = pk;
                }
                used = sum < deg && pj > 0;
            }
            if(!used)
                continue;
            d[j] = c.tmp("d");
            os << "    const R " << d[j] << " = " << c.x(n.obs[j]) << " - " << P(n.params[j]) << ";\n";
        }
        std::string v = c.tmp("v");
        os << "    R " << v << " = " << P(n.params[nO]) << ";\n";
        gadd(c, out, slot(c, n.params[nO]), "R(1)");
        int64_t boxes = 1;
        for(int j = 0; j < nO; ++j)
            boxes *= deg;
        int coeff = nO + 1;
        for(int64_t b = 1; b < boxes; ++b) {
            std::vector<int> pw(nO);
            int64_t ci = b;
            int sum    = 0;
            for(int j = 0; j < nO; ++j) {
                pw[j] = (int)(ci % deg);
                ci /= deg;
                sum += pw[j];
            }
            if(sum >= deg)
                continue;
            auto term = [&](int skip) {
                std::string e;
                for(int j = 0; j < nO; ++j) {
                    int q = pw[j] - (j == skip ? 1 : 0);
                    if(q > 0)
                        e += (e.empty() ? "" : " * ") + powi(c, d[j], q);
                }
                return e.empty() ? std::string("R(1)") : e;
            };
            std::string t = c.tmp("t");
            os << "    const R " << t << " = " << term(-1) << ";\n";
            os << "    " << v << " += " << P(n.params[coeff]) << " * " << t << ";\n";
            gadd(c, out, slot(c, n.params[coeff]), t);
            for(int j = 0; j < nO; ++j)
                if(pw[j] > 0)
                    gadd(c, out, slot(c, n.params[j]),
                         "-R(" + std::to_string(pw[j]) + ") * " + P(n.params[coeff]) + " * " + term(j));
            ++coeff;
        }
        out.v = v;
        break;
    }
    case GF_OP_AMP3BODY:
    case GF_OP_AMP4BODY: {
        // device_DalitzPlot (src/PDFs/physics/Amp3Body.cu:60-122) and device_DP
        // (src/PDFs/physics/Amp4Body.cu:53-90): |sum_r c_r B_r|^2 * efficiency, with the amplitudes B_r
        // read from the per-event cache
        if(!c.amp)
            throw std::runtime_error("codegen: amplitude PDF outside the event pass");
        const int ai   = c.T.amp_index(i);
        const int nRes = c.T.amp_count(ai);
        Val ev         = emit(c, n.children.back());
        std::string tr = c.tmp("tr"), ti = c.tmp("ti"), v = c.tmp("v");
        os << "    R " << tr << " = R(0), " << ti << " = R(0);\n";
        for(int r = 0; r < nRes; ++r) {
            std::string b = c.amp(ai, r), cr = P(n.params[2 * r]), cim = P(n.params[2 * r + 1]);
            os << "    " << tr << " += " << cr << " * " << b << ".x - " << cim << " * " << b << ".y;\n";
            os << "    " << ti << " += " << cr << " * " << b << ".y + " << cim << " * " << b << ".x;\n";
        }
        os << "    const R " << v << " = (" << tr << " * " << tr << " + " << ti << " * " << ti << ") * " << ev.v << ";\n";
        out.v = v;
        auto inner = [&](int s, const std::string &e) {
            if(s < 0 || !c.grad || i != 0)
                return;
            auto it = c.ampInner.find(s);
            c.ampInner[s] = it == c.ampInner.end() ? "(" + e + ")" : "(" + it->second + " + " + e + ")";
        };
        if(i == 0) {
            c.ampRoot = true;
            c.ampTr   = tr;
            c.ampTi   = ti;
        }
        for(int r = 0; r < nRes; ++r) {
            std::string b = c.amp(ai, r);
            gadd(c, out, slot(c, n.params[2 * r]),
                 "R(2) * (" + tr + " * " + b + ".x + " + ti + " * " + b + ".y) * " + ev.v);
            gadd(c, out, slot(c, n.params[2 * r + 1]),
                 "R(2) * (" + ti + " * " + b + ".x - " + tr + " * " + b + ".y) * " + ev.v);
            inner(slot(c, n.params[2 * r]), tr + " * " + b + ".x + " + ti + " * " + b + ".y");
            inner(slot(c, n.params[2 * r + 1]), ti + " * " + b + ".x - " + tr + " * " + b + ".y");
        }
        // resonance / line-shape parameters: d|T|^2/dt = 2 Re(conj(T) sum_a c_a dA_a/dt)
        if(c.grad && c.ampcol)
            for(const AmpTheta &t : c.T.amp_theta(ai)) {
                std::string dr = c.tmp("dr"), di = c.tmp("di");
                os << "    R " << dr << " = R(0), " << di << " = R(0);\n";
                for(size_t j = 0; j < t.amps.size(); ++j) {
                    const int a = t.amps[j];
                    std::string d = c.ampcol(t.col0 + (int)j), cr = P(n.params[2 * a]), cim = P(n.params[2 * a + 1]);
                    os << "    " << dr << " += " << cr << " * " << d << ".x - " << cim << " * " << d << ".y;\n";
                    os << "    " << di << " += " << cr << " * " << d << ".y + " << cim << " * " << d << ".x;\n";
                }
                gadd(c, out, t.slot, "R(2) * (" + tr + " * " + dr + " + " + ti + " * " + di + ") * " + ev.v);
                inner(t.slot, tr + " * " + dr + " + " + ti + " * " + di);
            }
        break;
    }
    case GF_OP_RES_RBW:
    case GF_OP_RES_NONRES:
    case GF_OP_AMPLITUDE:
    case GF_OP_LS_RBW:
    case GF_OP_LS_SBW:
    case GF_OP_SPINFACTOR: throw std::runtime_error("codegen: amplitude components are evaluated by the amplitude kernels only");
    default: throw std::runtime_error("codegen: unsupported operator");
    }
    materialise(c, out);
    return out;
}

const char *kPrelude = R"CUDA(
typedef long long i64;
struct GfArgs {
    const double *P;
    const int *active;
    const void *const *col;
    const int *const *kcol;
    void *ctab;
    const int *kgrid;
    double *gsum;
    double *gpartial;
    unsigned *gcounter;
    double *partial;
    unsigned *counter;
    double *out;
    const i64 *chunks;
    const int *toy_chunk0;
    const int *toy_nchunks;
    const i64 *toy_nevents;
    double *vals;
    const void *Pr;  /* [toy][npr] R: parameters, then host-computed analytic factors */
    void *Nq;        /* [toy][nq] R: numeric factors from the grid kernel */
    int *qflag;      /* [toy] bit 1 NaN, bit 2 non-positive numeric integral */
    const void *const *acol;   /* [toy][amplitude column] R2 cached resonance amplitudes */
    const double *const *dcol; /* [toy][observable] FP64 event columns (Dalitz variables) */
    const unsigned *dgrid;     /* in-Dalitz normalisation bins of every Amp3Body, b12 | b13 << 16 */
    double *gram;              /* integral partials [toy][tile][CTA][2 * pairs] */
    const int *dirty;          /* [toy] amplitude caches to rebuild */
    const double *const *nevt; /* per Amp4Body: normalisation events, SoA 5 x nnorm */
    const i64 *nnorm;
    void *const *nscr;         /* per amplitude node: normalisation-point columns of toy gtoy */
    int n_chunks;
    int n_toys;
    int metric;
    int gtoy;                  /* toy of the normalisation pass */
    i64 chunk;                 /* events per chunk */
    i64 nevt0;                 /* events of toy 0 */
    unsigned *gbar;            /* grid barrier of the one-launch evaluation: [arrivals, unused, error] */
    unsigned long long bar_ns; /* longest wait at that barrier (%globaltimer ns) before the kernel gives up */
    int rec_n;                 /* one-launch evaluation: the toy's record passed by value in rec (R values) */
    int stage_off;             /* one-launch evaluation: shared-memory offset of the CTA's staged events */
    unsigned stage_cap;        /* and the bytes available there (0: events are read from global memory) */
    unsigned bar_target;       /* the arrival count at which this launch's grid barrier opens */
    double *hpart;             /* one-launch evaluation: per chunk [components..., status] in page-locked host memory */
    const int *ksort;          /* one-launch tabulated path: toy 0's bin offsets sorted by bin (null: read kcol) */
    alignas(16) unsigned char rec[512];
    const void *p0[192];       /* one toy: its observable, bin-offset and amplitude columns, no table lookup */
};

// chunk ch of the event list: with one toy its bounds follow from the chunk size, else from the table
// pairwise sum of 8 values: exact when they are equal, three roundings on any path otherwise
__device__ __forceinline__ R gf_tree8(const R *v) {
    return ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
}
__device__ __forceinline__ void gf_chunk(const GfArgs &a, int ch, int &toy, i64 &b0, i64 &e0) {
    if(a.n_toys == 1) {
        toy = 0;
        b0  = (i64)ch * a.chunk;
        e0  = b0 + a.chunk < a.nevt0 ? b0 + a.chunk : a.nevt0;
    } else {
        const i64 *cd = a.chunks + 3 * (i64)ch;
        toy = (int)cd[0];
        b0  = cd[1];
        e0  = cd[2];
    }
}

__device__ __forceinline__ double gf_warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// The toy records the kernels read their parameters from: the argument block's (host-written) records in
// the kernels, a shared-memory copy in the bodies the one-launch kernel calls.
#define GF_PR a.Pr

// Programmatic dependent launch: let the next kernel of the evaluation start its independent prologue,
// and wait for the previous kernel's results (both are no-ops without a programmatic dependency).
__device__ __forceinline__ void gf_pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void gf_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Barrier over all CTAs of a cooperative launch (every CTA resident), bounded in time: thread 0 of each CTA
// arrives on bar[0]; the last to arrive resets it and advances the generation bar[1]; the others wait for
// the generation to move, at most `limit` ns of %globaltimer.  A wait that runs out sets bar[2] and makes
// every thread of the CTA see false, so that the CTA stops (the host then reports the evaluation as failed
// and clears the barrier words); no CTA gets past a barrier that not every CTA reached.
__device__ __forceinline__ unsigned long long gf_globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __noinline__ bool gf_grid_sync(unsigned *bar, unsigned target, unsigned long long limit) {
    __shared__ int ok;
    __syncthreads();
    if(threadIdx.x == 0) {
        int good = 1;
        // The arrival counter only grows: launch e of the engine opens at e x (CTAs) arrivals (modulo 2^32),
        // so an arriving CTA adds without reading and every CTA waits for the count itself (one trip to the
        // counter, no second word written by a last arrival).  The arrival releases the CTA's writes (ordered
        // before it by the __syncthreads above); the waiter's acquire of a count that includes every
        // arrival synchronises with all of them (each later addition extends the earlier ones' release
        // sequences), so every CTA sees every CTA's writes from before the barrier.
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" :: "l"(bar) : "memory");
        const unsigned long long t0 = gf_globaltimer();
        for(;;) {
            unsigned c;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(bar) : "memory");
            if((int)(c - target) >= 0)
                break;
            if(gf_globaltimer() - t0 > limit) {
                atomicOr(bar + 2, 1u);
                good = 0;
                break;
            }
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Shared-memory mbarrier of a bulk copy (cp.async.bulk, the TMA unit): a wait that gives up after `limit` ns.
__device__ __forceinline__ bool gf_mbar_wait(unsigned long long *mbar, unsigned parity, unsigned long long limit) {
    const unsigned addr = (unsigned)__cvta_generic_to_shared(mbar);
    const unsigned long long t0 = gf_globaltimer();
    for(;;) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n" : "=r"(done) : "r"(addr), "r"(parity) : "memory");
        if(done)
            return true;
        if(gf_globaltimer() - t0 > limit)
            return false;
    }
}

// Bin centre lo + w (b + 1/2) with w = (hi - lo) / n from the host: the binned MetricTaker's
// arithmetic (src/PDFs/MetricTaker.cu:76-82) with its two roundings kept separate.
__device__ __forceinline__ double gf_centre(double lo, double w, int b) {
    return __dadd_rn(__dmul_rn(w, (double)b + 0.5), lo);
}
)CUDA";

// FP32 lane reductions with a two-sum compensation term (error of the sum ~ one rounding of the total).
const char *kPreludeF32 = R"CUDA(
__device__ __forceinline__ void gf_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ float gf_group_sum(float v, int width) {
    float hi = v, lo = 0.f;
    for(int o = width >> 1; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o, width);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o, width);
        float s, e;
        gf_two_sum(hi, h2, s, e);
        hi = s;
        lo += l2 + e;
    }
    return hi + lo;
}
// The width lanes' pairs v + c summed as pairs: the total as a normalised pair (hi, lo) in every lane
__device__ __forceinline__ float2 gf_group_sum2(float v, float c, int width) {
    float hi = v, lo = c;
    for(int o = width >> 1; o > 0; o >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o, width);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o, width);
        float s, e;
        gf_two_sum(hi, h2, s, e);
        hi = s;
        lo += l2 + e;
    }
    const float h = hi + lo;
    return make_float2(h, lo - (h - hi));
}
// s + c += v with a two-sum correction term c.
__device__ __forceinline__ void gf_comp_add(float &s, float &c, float v) {
    float t, e;
    gf_two_sum(s, v, t, e);
    s = t;
    c += e;
}
// Partial sums as an unevaluated pair hi + lo of FP32 values (about 48 significant bits).
typedef float2 ACC;
__device__ __forceinline__ ACC acc_zero() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ ACC acc_of(float v) { return make_float2(v, 0.f); }
__device__ __forceinline__ ACC acc_pair(float hi, float lo) { return make_float2(hi, lo); }
// a b as an unevaluated pair (the product and its exact rounding error)
__device__ __forceinline__ ACC gf_two_prod(float a, float b) { const float p = a * b; return make_float2(p, fmaf(a, b, -p)); }
// 1/x: the hardware reciprocal approximation refined by one Newton-Raphson step r + r (1 - x r); not
// guaranteed to be correctly rounded (the generated kernels use it where 1/P feeds gradient sums)
__device__ __forceinline__ float gf_rcp(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}
// -log of a product of event probabilities: x = m 2^e with m in [0.75, 1.5) (exact bit operations), the
// mantissas multiplied into lm (8 of them stay within [0.1, 26)) and the exponents added into le; zero,
// subnormal, infinite and NaN x are added to av directly.  The caller adds -(log lm + le ln 2), with ln 2
// split after Cody and Waite into GF_LN2_HI (13 significant bits: le * GF_LN2_HI is exact for |le| < 2^11)
// and GF_LN2_LO = ln 2 - GF_LN2_HI.
#define GF_LN2_HI 0.693115234375f
#define GF_LN2_LO 3.1946183e-05f
__device__ __forceinline__ void gf_log_acc(float x, float &lm, int &le, float &av) {
    const int b = __float_as_int(x);
    if((unsigned)(b - 0x00800000) < 0x7F000000u) {
        const int e = (b - 0x3F400000) >> 23;
        lm *= __int_as_float(b - (e << 23));
        le += e;
    } else
        av -= logf(x);
}
__device__ __forceinline__ ACC acc_add(ACC a, ACC b) {
    float s, e;
    gf_two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    const float hi = s + e;
    const float lo = e - (hi - s);
    return make_float2(hi, lo);
}
__device__ __forceinline__ ACC warp_acc(float v) {
    ACC a = acc_of(v);
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) {
        ACC b;
        b.x = __shfl_down_sync(0xffffffffu, a.x, o);
        b.y = __shfl_down_sync(0xffffffffu, a.y, o);
        a   = acc_add(a, b);
    }
    return a;
}
__device__ __forceinline__ ACC warp_acc2(ACC a) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) {
        ACC b;
        b.x = __shfl_down_sync(0xffffffffu, a.x, o);
        b.y = __shfl_down_sync(0xffffffffu, a.y, o);
        a   = acc_add(a, b);
    }
    return a;
}
__device__ __forceinline__ ACC acc_shfl_xor(ACC a, int o) {
    return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
__device__ __forceinline__ ACC acc_shfl(ACC a, int src) {
    return make_float2(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
}
__device__ __forceinline__ double acc_value(ACC a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float acc_r(ACC a) { return a.x + a.y; }
// x * (h + l) for a normalisation factor kept as an FP32 pair: one rounding, no bias from rounding the factor
__device__ __forceinline__ float gf_nm(float x, float h, float l) { return fmaf(x, h, x * l); }
#define GF_CENTRE(lo, w, b) ((float)(lo) + (float)(w) * ((float)(b) + 0.5f))
)CUDA";

// Unevaluated FP32 pairs h + l (about 44 significant bits) for the per-bin terms of the tabulated event pass.
// There the event function and -log P of each bin offset are evaluated once and then added once per event,
// so a rounding of a bin's term in single precision would be repeated by every event of that bin and would
// move the NLL in steps as the parameters change.  The arithmetic is the classic double-single one (Dekker's
// exact products through fma, Knuth's two-sum); the logarithm reduces x = (m + ml) 2^e with
// m in [1/sqrt 2, sqrt 2) around c = 1 + j/32 and sums ln 2^e + ln c + 2 atanh(s), s = (m + ml - c) / (m + ml + c),
// |s| < 0.011, with the series 2 s + 2 s^3 / 3 + 2 s^5 / 5 + 2 s^7 / 7 (the first term as a pair).
const char *kPreludeDF = R"CUDA(
struct gf_df {
    float h, l;
    __device__ __forceinline__ gf_df() : h(0.f), l(0.f) {}
    __device__ __forceinline__ gf_df(float x) : h(x), l(0.f) {}
    __device__ __forceinline__ gf_df(int x) : h((float)x), l(0.f) {}
    __device__ __forceinline__ gf_df(float hi, float lo) : h(hi), l(lo) {}
};
__device__ __forceinline__ gf_df gf_df_fast(float a, float b) { const float s = a + b; return gf_df(s, b - (s - a)); }
__device__ __forceinline__ gf_df operator+(gf_df a, gf_df b) {
    float s, e;
    gf_two_sum(a.h, b.h, s, e);
    e += a.l + b.l;
    return gf_df_fast(s, e);
}
__device__ __forceinline__ gf_df operator-(gf_df a) { return gf_df(-a.h, -a.l); }
__device__ __forceinline__ gf_df operator-(gf_df a, gf_df b) { return a + (-b); }
__device__ __forceinline__ gf_df operator*(gf_df a, gf_df b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
    return gf_df_fast(p, e);
}
// a / b: a first quotient, the exact residual a - q1 b, and its quotient (each quotient to a few ulps suffices:
// the second corrects the first, and its own error is 2^-23 of a term 2^-22 smaller than the first)
__device__ __forceinline__ gf_df operator/(gf_df a, gf_df b) {
    const float q1 = __fdividef(a.h, b.h);
    const float p = q1 * b.h, pe = fmaf(q1, b.h, -p);
    float s, e;
    gf_two_sum(a.h, -p, s, e);
    e += a.l - pe - q1 * b.l;
    return gf_df_fast(q1, __fdividef(s + e, b.h));
}
__device__ __forceinline__ gf_df &operator+=(gf_df &a, gf_df b) { a = a + b; return a; }
__device__ __forceinline__ gf_df &operator-=(gf_df &a, gf_df b) { a = a - b; return a; }
__device__ __forceinline__ gf_df &operator*=(gf_df &a, gf_df b) { a = a * b; return a; }
__device__ __forceinline__ gf_df &operator/=(gf_df &a, gf_df b) { a = a / b; return a; }
__device__ __forceinline__ bool operator>(gf_df a, gf_df b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ bool operator<(gf_df a, gf_df b) { return b > a; }
// x * (h + l) for a normalisation factor kept as an FP32 pair
__device__ __forceinline__ gf_df gf_nm(gf_df x, float h, float l) { return x * gf_df(h, l); }
#define GF_LN2_DH 0.693147182f
#define GF_LN2_DL -1.90465421e-09f
// ln x; single precision for x <= 0, NaN and infinity
__device__ __forceinline__ gf_df gf_df_log(gf_df x) {
    if(!(x.h > 0.f) || isinf(x.h))
        return gf_df(logf(x.h));
    int e;
    float m = frexpf(x.h, &e);
    if(m < 0.707106769f) {
        m *= 2.f;
        e -= 1;
    }
    const float ml = ldexpf(x.l, -e);
    const int j    = __float2int_rn((m - 1.f) * 32.f);
    const float c  = fmaf((float)j, 0.03125f, 1.f);
    float uh, ul;
    gf_two_sum(m - c, ml, uh, ul);
    const gf_df u(uh, ul);
    const gf_df s = u / (gf_df(2.f * c) + u);
    const float s2   = s.h * s.h;
    const float tail = s.h * s2 * fmaf(s2, fmaf(s2, 0.285714298f, 0.4f), 0.666666687f);
    gf_df r = gf_df(2.f * s.h, 2.f * s.l) + gf_df(tail);
    r += gf_df(gf_lnc_h[j + 9], gf_lnc_l[j + 9]);
    const float fe = (float)e;
    const float p  = fe * GF_LN2_DH;
    r += gf_df_fast(p, fmaf(fe, GF_LN2_DL, fmaf(fe, GF_LN2_DH, -p)));
    return r;
}
)CUDA";

// ln(1 + j/32), j = -9 .. 13, as FP32 pairs for gf_df_log (from the host's FP64 logarithm)
std::string dfLogTable() {
    std::string h = "__device__ const float gf_lnc_h[23] = {", l = "__device__ const float gf_lnc_l[23] = {";
    char buf[64];
    for(int j = -9; j <= 13; ++j) {
        const double v  = std::log1p(j / 32.0);
        const float vh  = (float)v;
        const float vl  = (float)(v - (double)vh);
        std::snprintf(buf, sizeof buf, "%s%.9ef", j > -9 ? ", " : "", (double)vh);
        h += buf;
        std::snprintf(buf, sizeof buf, "%s%.9ef", j > -9 ? ", " : "", (double)vl);
        l += buf;
    }
    return h + "};\n" + l + "};\n";
}

const char *kPreludeF64 = R"CUDA(
__device__ __forceinline__ double gf_group_sum(double v, int width) {
    for(int o = width >> 1; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o, width);
    return v;
}
__device__ __forceinline__ void gf_comp_add(double &s, double &c, double v) { s += v; }
typedef double ACC;
__device__ __forceinline__ ACC acc_zero() { return 0.0; }
__device__ __forceinline__ ACC acc_of(double v) { return v; }
__device__ __forceinline__ ACC acc_pair(double hi, double lo) { return hi + lo; }
__device__ __forceinline__ double gf_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ ACC gf_two_prod(double a, double b) { return a * b; }
__device__ __forceinline__ ACC acc_add(ACC a, ACC b) { return a + b; }
__device__ __forceinline__ ACC warp_acc(double v) { return gf_warp_sum(v); }
__device__ __forceinline__ ACC warp_acc2(ACC a) { return gf_warp_sum(a); }
__device__ __forceinline__ ACC acc_shfl_xor(ACC a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
__device__ __forceinline__ ACC acc_shfl(ACC a, int src) { return __shfl_sync(0xffffffffu, a, src); }
__device__ __forceinline__ double acc_value(ACC a) { return a; }
__device__ __forceinline__ double acc_r(ACC a) { return a; }
__device__ __forceinline__ double gf_nm(double x, double h, double l) { return x * h; }
#define GF_CENTRE(lo, w, b) gf_centre(lo, w, b)
)CUDA";

// Dalitz-plot helpers: the kinematic boundary in FP64 with every rounding explicit (no contraction, as the
// host restatement compiles it), and the relativistic Breit-Wigner of src/PDFs/physics/resonances/RBW.cu:9-86
// with its helpers (src/PDFs/physics/resonances/Resonance.cu:48-155).  The amplitude works in R; the squared
// masses and their differences with the resonance mass come in FP64, so that an FP32 amplitude loses nothing
// to cancellation near the pole.
const char *kPreludeAmp = R"CUDA(
__device__ __forceinline__ bool gf_in_dalitz(double m12, double m13, double M, double m1, double m2, double m3) {
    const double dm1pdm2 = __dadd_rn(m1, m2), bigMmdm3 = __dsub_rn(M, m3), bigMmdm1 = __dsub_rn(M, m1);
    const double MM = __dmul_rn(M, M), m11 = __dmul_rn(m1, m1), m22 = __dmul_rn(m2, m2), m33 = __dmul_rn(m3, m3);
    const double m23 = __dsub_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(MM, m11), m22), m33), m12), m13);
    if(m23 < 0. || m23 > __dmul_rn(bigMmdm1, bigMmdm1))
        return false;
    const bool a = !(m12 < __dmul_rn(dm1pdm2, dm1pdm2)), b = !(m12 > __dmul_rn(bigMmdm3, bigMmdm3));
    const double rt = __dsqrt_rn(m12);
    const double e1 = __ddiv_rn(__dmul_rn(0.5, __dadd_rn(__dsub_rn(m12, m22), m11)), rt);
    const double e3 = __ddiv_rn(__dmul_rn(0.5, __dsub_rn(__dsub_rn(MM, m12), m33)), rt);
    const double p1 = __dsqrt_rn(__dsub_rn(__dmul_rn(e1, e1), m11));
    const double p3 = __dsqrt_rn(__dsub_rn(__dmul_rn(e3, e3), m33));
    const double s = __dadd_rn(e1, e3), u = __dadd_rn(p1, p3), w = __dsub_rn(p1, p3);
    const double lo = __dsub_rn(__dmul_rn(s, s), __dmul_rn(u, u)), hi = __dsub_rn(__dmul_rn(s, s), __dmul_rn(w, w));
    return a && b && !(m13 < lo) && !(m13 > hi);
}
__device__ __forceinline__ double gf_m23(double m12, double m13, double M, double m1, double m2, double m3) {
    return __dsub_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(M, M), __dmul_rn(m1, m1)), __dmul_rn(m2, m2)),
                                          __dmul_rn(m3, m3)), m12), m13);
}
__device__ __forceinline__ R gf_tb_mom(R s, R a, R b) {
    R k1 = R(1) - (a + b) * (a + b) / s;
    k1   = k1 >= R(0) ? sqrt(k1) : R(1);
    R k2 = R(1) - (a - b) * (a - b) / s;
    k2   = k2 >= R(0) ? sqrt(k2) : R(1);
    return R(0.5) * sqrt(s) * k1 * k2;
}
__device__ __forceinline__ R gf_tb_mom_mother(R s, R M, R c) {
    R k1 = R(1) - (M + c) * (M + c) / s;
    k1   = k1 >= R(0) ? sqrt(k1) : R(1);
    R k2 = R(1) - (M - c) * (M - c) / s;
    k2   = k2 >= R(0) ? sqrt(k2) : R(1);
    return R(0.5) * s * k1 * k2 / M;
}
__device__ __forceinline__ R gf_damp2(R p, int spin, R r) {
    const R sq = r * r * p * p;
    return spin == 2 ? R(13) * sq / ((sq - R(3)) * (sq - R(3))) + R(9) * sq * sq : R(2) * sq;
}
__device__ __forceinline__ R gf_damp2n(R p, int spin, R r) {
    const R sq = r * r * p * p;
    const R d  = R(1) + sq;
    return spin == 2 ? d + R(8) + R(2) * sq + sq * sq : d;
}
// Zemach spin factor (Resonance.cu spinFactor); the event-dependent differences are formed in FP64.
__device__ __forceinline__ R gf_spin(int spin, double M, double m1, double m2, double m3, double m12, double m13,
                                     double m23, int cyc) {
    if(spin == 0)
        return R(1);
    const double mA = cyc == 0 ? m1 : (cyc == 1 ? m3 : m2), mB = cyc == 0 ? m2 : (cyc == 1 ? m1 : m3);
    const double mC = cyc == 0 ? m3 : (cyc == 1 ? m2 : m1);
    const double mAC = cyc == 0 ? m13 : (cyc == 1 ? m23 : m12), mBC = cyc == 0 ? m23 : (cyc == 1 ? m12 : m13);
    const double mAB = cyc == 0 ? m12 : (cyc == 1 ? m13 : m23);
    const R massFactor = R(1) / (R)mAB;
    const R MC = (R)(M * M - mC * mC), AB = (R)(mA * mA - mB * mB);
    R sf = -((R)(mBC - mAC) + massFactor * MC * AB);
    if(spin == 2) {
        sf *= sf;
        R ex = ((R)(mAB - 2 * M * M - 2 * mC * mC) + massFactor * MC * MC);
        ex *= ((R)(mAB - 2 * mA * mA - 2 * mB * mB) + massFactor * AB * AB);
        ex /= R(3);
        sf -= ex;
    }
    return sf;
}
template <int I>
__device__ __forceinline__ R2 gf_rbw(double m12, double m13, double m23, double mass, double width, int spin, int cyc,
                                     bool norm, double M, double m1, double m2, double m3, double rr, double rmm) {
    R re = R(0), im = R(0);
    const double rm2 = mass * mass;
    const R rs = (R)rm2, r = (R)rr, rm = (R)rmm;
#pragma unroll
    for(int it = 0; it < I; ++it) {
        const double sq = cyc == 0 ? m12 : (cyc == 1 ? m13 : m23);
        const R d1 = (R)(cyc == 2 ? m2 : m1), d2 = (R)(cyc == 0 ? m2 : m3);
        const R bach = (R)(cyc == 0 ? m3 : (cyc == 1 ? m2 : m1));
        const R s = (R)sq;
        R fr = R(1), frM = R(1);
        const R pm = gf_tb_mom(s, d1, d2), pn = gf_tb_mom(rs, d1, d2);
        R pmM, pnM = R(0);
        if(norm) {
            pmM = gf_tb_mom_mother(s, (R)M, bach);
            pnM = gf_tb_mom_mother(rs, (R)M, bach);
        } else
            pmM = gf_tb_mom((R)(M * M), sqrt(s), bach);
        if(spin != 0) {
            if(norm) {
                fr  = gf_damp2n(pn, spin, r) / gf_damp2n(pm, spin, r);
                frM = gf_damp2n(pnM, spin, rm) / gf_damp2n(pmM, spin, rm);
            } else {
                fr  = gf_damp2(pm, spin, r);
                frM = gf_damp2(pmM, spin, rm);
            }
        }
        const R A = (R)(rm2 - sq);
        const R q = pm / pn;
        R qp      = q;
        for(int k = 0; k < 2 * spin; ++k)
            qp *= q;
        const R B = rs * (R)width * qp * fr / sqrt(s);
        const R C = R(1) / (A * A + B * B);
        R xr = A * C, xi = B * C;
        const R f1 = sqrt(fr), f2 = sqrt(frM), sf = gf_spin(spin, M, m1, m2, m3, m12, m13, m23, cyc);
        xr *= f1;
        xi *= f1;
        xr *= f2;
        xi *= f2;
        xr *= sf;
        xi *= sf;
        re += xr;
        im += xi;
        if(I > 1)
            cyc = (cyc + 1) % 3;
    }
    R2 o;
    o.x = re;
    o.y = im;
    return o;
}
)CUDA";

// 4-body amplitude helpers in FP64: daughter 4-vectors from the five variables (get4Vecs,
// src/PDFs/physics/DalitzPlotHelpers.cu:77-156), invariant masses of daughter combinations (getmass,
// :158-232), the Zemach spin-factor algebra (include/goofit/PDFs/physics/detail/SpinHelper.h), the spin
// factors (src/PDFs/physics/SpinFactors.cu:83-568) and the BW / SBW line shapes with their Blatt-Weisskopf
// factors (src/PDFs/physics/lineshapes/BW.cu:14-110, Common.cu:8-51).  Vectors are (x, y, z, E).
const char *kPreludeAmp4 = R"CUDA(
struct GfLV { double x, y, z, e; };
__device__ __forceinline__ GfLV lv(double x, double y, double z, double e) { GfLV v; v.x = x; v.y = y; v.z = z; v.e = e; return v; }
__device__ __forceinline__ GfLV operator+(GfLV a, GfLV b) { return lv(a.x + b.x, a.y + b.y, a.z + b.z, a.e + b.e); }
__device__ __forceinline__ GfLV operator-(GfLV a, GfLV b) { return lv(a.x - b.x, a.y - b.y, a.z - b.z, a.e - b.e); }
__device__ __forceinline__ GfLV operator*(GfLV a, double s) { return lv(a.x * s, a.y * s, a.z * s, a.e * s); }
__device__ __forceinline__ GfLV operator*(double s, GfLV a) { return lv(a.x * s, a.y * s, a.z * s, a.e * s); }
__device__ __forceinline__ double ldot(GfLV a, GfLV b) { return a.e * b.e - a.x * b.x - a.y * b.y - a.z * b.z; }
__device__ __forceinline__ double lmass(GfLV a) { return sqrt(ldot(a, a)); }
// spin-1 Zemach tensor q - (q.p) p / mR^2 and the spin sum of a vector, -v + p (p.v) / mR^2
__device__ __forceinline__ GfLV zt1(GfLV q, GfLV p, double mR) { return q - ldot(q, p) * p * (1. / (mR * mR)); }
__device__ __forceinline__ GfLV ssv(GfLV p, double mR, GfLV v) { return -1.0 * v + p * (ldot(p, v) / (mR * mR)); }
__device__ __forceinline__ double ssvs(GfLV p, double mR, GfLV l, GfLV r) { return ldot(l, ssv(p, mR, r)); }
__device__ __forceinline__ double ssts(GfLV p, double mR, GfLV lm, GfLV ln, GfLV ra, GfLV rb) {
    const double manb = ssvs(p, mR, lm, ra) * ssvs(p, mR, ln, rb);
    const double mbna = ssvs(p, mR, lm, rb) * ssvs(p, mR, ln, ra);
    const double mnab = ssvs(p, mR, lm, ln) * ssvs(p, mR, ra, rb);
    return (1. / 2.) * (manb + mbna) - (1. / 3.) * mnab;
}
// spin-2 Zemach tensor contracted with a vector: T(q, p) . v with T = t t - |t|^2 / 3 (g - p p / mR^2)
__device__ __forceinline__ GfLV zt2c(GfLV q, GfLV p, double mR, GfLV v) {
    const GfLV t = zt1(q, p, mR);
    const double f = (1. / 3.) * ldot(t, t), iu = 1. / (mR * mR);
    const double tc[4] = {t.x, t.y, t.z, t.e}, pc[4] = {p.x, p.y, p.z, p.e};
    const double g[4][4] = {{-1, 0, 0, 0}, {0, -1, 0, 0}, {0, 0, -1, 0}, {0, 0, 0, 1}};
    GfLV row[4];
#pragma unroll
    for(int i = 0; i < 4; ++i) {
        double r[4];
#pragma unroll
        for(int j = 0; j < 4; ++j)
            r[j] = tc[i] * tc[j] - f * (g[i][j] - pc[i] * pc[j] * iu);
        row[i] = lv(r[0], r[1], r[2], r[3]);
    }
    return v.e * row[3] - v.x * row[0] - v.y * row[1] - v.z * row[2];
}
__device__ __forceinline__ GfLV leps3(GfLV a, GfLV b, GfLV c) {
    GfLV v;
    v.e = -1. * a.x * (b.y * c.z - b.z * c.y) - a.y * (b.z * c.x - b.x * c.z) - a.z * (b.x * c.y - b.y * c.x);
    v.z = a.x * (b.e * c.y - b.y * c.e) + a.y * (b.x * c.e - b.e * c.x) + a.e * (b.y * c.x - b.x * c.y);
    v.y = a.x * (b.z * c.e - b.e * c.z) + a.z * (b.e * c.x - b.x * c.e) + a.e * (b.x * c.z - b.z * c.x);
    v.x = a.y * (b.e * c.z - b.z * c.e) + a.z * (b.y * c.e - b.e * c.y) + a.e * (b.z * c.y - b.y * c.z);
    return v;
}
__device__ __forceinline__ void gf_get4vecs(GfLV *P, double m12, double m34, double cos12, double cos34, double phi,
                                            double M, double m1, double m2, double m3, double m4) {
    const double E1 = (m12 * m12 + m1 * m1 - m2 * m2) / (2 * m12), E2 = (m12 * m12 - m1 * m1 + m2 * m2) / (2 * m12);
    const double E3 = (m34 * m34 + m3 * m3 - m4 * m4) / (2 * m34), E4 = (m34 * m34 - m3 * m3 + m4 * m4) / (2 * m34);
    const double p1 = sqrt(E1 * E1 - m1 * m1), p3 = sqrt(E3 * E3 - m3 * m3);
    const double sin12 = sqrt(1 - cos12 * cos12), sin34 = sqrt(1 - cos34 * cos34);
    const double ED1 = (M * M + m12 * m12 - m34 * m34) / (2 * m12), PD1 = sqrt(ED1 * ED1 - M * M);
    const double beta1 = PD1 / ED1, gamma1 = 1.0 / sqrt(1 - beta1 * beta1);
    const double ED2 = (M * M - m12 * m12 + m34 * m34) / (2 * m34), PD2 = sqrt(ED2 * ED2 - M * M);
    const double beta2 = -PD2 / ED2, gamma2 = 1.0 / sqrt(1 - beta2 * beta2);
    const double x[4] = {cos12 * p1, -cos12 * p1, -cos34 * p3, cos34 * p3};
    const double y[4] = {sin12 * p1, -sin12 * p1, -sin34 * p3, sin34 * p3};
    const double E[4] = {E1, E2, E3, E4};
    const double cp = cos(phi), sp = sin(phi);
#pragma unroll
    for(int k = 0; k < 4; ++k) {
        const double g = k < 2 ? gamma1 : gamma2, b = k < 2 ? beta1 : beta2;
        P[k].e = g * (E[k] + b * x[k]);
        P[k].x = g * (x[k] + b * E[k]);
        P[k].z = k < 2 ? sp * y[k] : 0.0;
        P[k].y = k < 2 ? cp * y[k] : y[k];
    }
}
// invariant mass of a daughter combination (DP4Pair code) and the masses it decays to
__device__ __forceinline__ double gf_pairmass(int pair, const GfLV *P, double m1, double m2, double m3, double m4,
                                              double &d1, double &d2) {
    switch(pair) {
    case 0: d1 = m1; d2 = m2; return lmass(P[0] + P[1]);
    case 1: d1 = m3; d2 = m4; return lmass(P[2] + P[3]);
    case 2: d1 = m1; d2 = m3; return lmass(P[0] + P[2]);
    case 3: d1 = m1; d2 = m4; return lmass(P[0] + P[3]);
    case 4: d1 = m2; d2 = m3; return lmass(P[1] + P[2]);
    case 5: d1 = m2; d2 = m4; return lmass(P[1] + P[3]);
    case 6: d1 = lmass(P[0] + P[1]); d2 = m3; return lmass(P[0] + P[1] + P[2]);
    case 7: d1 = lmass(P[0] + P[2]); d2 = m2; return lmass(P[0] + P[1] + P[2]);
    case 8: d1 = lmass(P[1] + P[2]); d2 = m1; return lmass(P[0] + P[1] + P[2]);
    case 9: d1 = lmass(P[0] + P[1]); d2 = m4; return lmass(P[0] + P[1] + P[3]);
    case 10: d1 = lmass(P[0] + P[3]); d2 = m2; return lmass(P[0] + P[1] + P[3]);
    case 11: d1 = lmass(P[1] + P[3]); d2 = m1; return lmass(P[0] + P[1] + P[3]);
    case 12: d1 = lmass(P[0] + P[2]); d2 = m4; return lmass(P[0] + P[2] + P[3]);
    case 13: d1 = lmass(P[0] + P[3]); d2 = m3; return lmass(P[0] + P[2] + P[3]);
    case 14: d1 = lmass(P[2] + P[3]); d2 = m1; return lmass(P[0] + P[2] + P[3]);
    case 15: d1 = lmass(P[1] + P[2]); d2 = m4; return lmass(P[1] + P[2] + P[3]);
    case 16: d1 = lmass(P[1] + P[3]); d2 = m3; return lmass(P[1] + P[2] + P[3]);
    default: d1 = lmass(P[2] + P[3]); d2 = m2; return lmass(P[1] + P[2] + P[3]);
    }
}
__device__ __forceinline__ double gf_spinfactor(int kind, double mD0, GfLV P1, GfLV P2, GfLV P3, GfLV P4) {
    switch(kind) {
    case 1: { const GfLV pV = P3 + P4, qV = P3 - P4, pP = pV + P2, qP = pV - P2;
              return ldot(zt1(qP, pP, lmass(pP)), zt1(qV, pV, lmass(pV))); }
    case 2: { const GfLV pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4;
              const double MV1 = sqrt(ldot(pV1, pV1)), MV2 = sqrt(ldot(pV2, pV2));
              return (ldot(qV1, qV2) - ldot(qV1, pV1) * ldot(pV1, qV2) / (MV1 * MV1) -
                      ldot(qV1, pV2) * ldot(pV2, qV2) / (MV2 * MV2) +
                      ldot(qV1, pV1) * ldot(pV1, pV2) * ldot(pV2, qV2) / (MV1 * MV1 * MV2 * MV2)); }
    case 3: { const GfLV pV1 = P1 + P2, qV1 = P2 - P1, pV2 = P3 + P4, qV2 = P4 - P3, pD = pV1 + pV2, qD = pV1 - pV2;
              const double MV1 = sqrt(ldot(pV1, pV1)), MV2 = sqrt(ldot(pV2, pV2));
              return -ldot(leps3(pD, zt1(qD, pD, lmass(pD)), zt1(qV1, pV1, MV1)), zt1(qV2, pV2, MV2)); }
    case 4: { const GfLV pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4, pD = pV1 + pV2, qD = pV1 - pV2;
              return ldot(zt1(qV1, pV1, lmass(pV1)), zt2c(qD, pD, lmass(pD), zt1(qV2, pV2, lmass(pV2)))); }
    case 5: { const GfLV pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, pD = P1 + pA, qD = pA - P1;
              return -ldot(zt1(qD, pD, lmass(pD)), ssv(pA, lmass(pA), zt1(qV, pV, lmass(pV)))); }
    case 6: { const GfLV pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, qA = P2 - pV, pD = P1 + pA, qD = pA - P1;
              return ldot(zt1(qD, pD, lmass(pD)), zt2c(qA, pA, lmass(pA), zt1(qV, pV, lmass(pV)))); }
    case 7: { const GfLV pS = P3 + P4, pV = P1 + P2, qV = P1 - P2, pD = pV + pS, qD = pV - pS;
              return ldot(zt1(qD, pD, lmass(pD)), zt1(qV, pV, lmass(pV))); }
    case 8: { const GfLV pV1 = P2 + P3 + P4, pV2 = P3 + P4, qV1 = (P3 + P4) - P2, qV2 = P3 - P4;
              const double MV1 = lmass(pV1), MV2 = lmass(pV2);
              const GfLV pD = pV1 + P1, qD = pV1 - P1;
              return ldot(leps3(pV1, zt1(qV1, pV1, MV1), zt1(qV2, pV2, MV2)), ssv(pV1, MV1, zt1(qD, pD, lmass(pD)))); }
    case 9: { const GfLV pS = P3 + P4, pA = P2 + pS, qA = pS - P2, pD = pA + P1, qD = pA - P1;
              return ldot(zt1(qD, pD, lmass(pD)), zt1(qA, pA, lmass(pA))); }
    case 10: { const GfLV pV = P3 + P4, qV = P3 - P4, pT = P2 + pV, qT = pV - P2, pD = P1 + pT, qD = pT - P1;
               const double mT = lmass(pT);
               const GfLV tV = zt1(qV, pV, lmass(pV)), tD = zt1(qD, pD, lmass(pD)), t1T = zt1(qT, pT, mT);
               const GfLV tmp = leps3(t1T, pT, ssv(pT, mT, tV));
               return ssts(pT, mT, tD, tD, tmp, t1T) + 1. / 3. * ldot(tD, tD) / ldot(pT, pT) * ssts(pT, mT, pD, pD, tmp, t1T); }
    case 11: case 12: case 13: case 14: {
        const bool l12 = kind == 11 || kind == 12;
        const double a = l12 ? ldot(P1 + P2, P1 + P2) : ldot(P1 + P2 + P3, P1 + P2 + P3);
        const double b = l12 ? ldot(P3 + P4, P3 + P4) : ldot(P4, P4);
        const GfLV T = P1 + P2 + P3 + P4;
        const double s = ldot(T, T);
        const double q2 = s / 4. - (a + b) / 2. + (a - b) * (a - b) / (4 * s);
        const double z2 = q2 * mD0 * mD0;
        const double ff = (kind == 11 || kind == 13) ? 1.0 / (1 + z2) : 1.0 / (z2 * z2 + 3 * z2 + 9);
        return sqrt(ff); }
    default: return 1.0; // DtoPP1_PtoSP2_StoP3P4 and ONE
    }
}
__device__ __forceinline__ double gf_blp(double z2, double z02, int L) {
    return L == 0 ? 1.0 : (L == 1 ? (1 + z02) / (1 + z2) : (z02 * z02 + 3 * z02 + 9) / (z2 * z2 + 3 * z2 + 9));
}
__device__ __forceinline__ double gf_bl(double z2, int L) {
    return L == 0 ? 1.0 : (L == 1 ? 2 * z2 / (1 + z2) : (13 * z2 * z2) / (z2 * z2 + 3 * z2 + 9));
}
__device__ __forceinline__ double gf_bl2(double z2, int L) {
    return L == 0 ? 1.0 : (L == 1 ? 1.0 / (1 + z2) : 1.0 / (z2 * z2 + 3 * z2 + 9));
}
// BW (RBW, with mass-dependent width) or SBW (constant width) line shape; the body is gf_lineshape_t
__device__ __forceinline__ double2 gf_lineshape(bool sbw, double Mpair, double m1, double m2, double mass, double width,
                                                int orbital, int FF, double radius);
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
)CUDA";

// FP32 arithmetic of the 4-body amplitudes for the mixed-precision engine: the kinematic inversion, pair
// masses, spin factors, line shapes and products.  Same formulas and order as the FP64 functions above.
const char *kPreludeAmp4F = R"CUDA(
struct GfLVf { float x, y, z, e; };
__device__ __forceinline__ GfLVf lvf(float x, float y, float z, float e) { GfLVf v; v.x = x; v.y = y; v.z = z; v.e = e; return v; }
__device__ __forceinline__ GfLVf lvf(GfLV a) { return lvf((float)a.x, (float)a.y, (float)a.z, (float)a.e); }
__device__ __forceinline__ GfLVf operator+(GfLVf a, GfLVf b) { return lvf(a.x + b.x, a.y + b.y, a.z + b.z, a.e + b.e); }
__device__ __forceinline__ GfLVf operator-(GfLVf a, GfLVf b) { return lvf(a.x - b.x, a.y - b.y, a.z - b.z, a.e - b.e); }
__device__ __forceinline__ GfLVf operator*(GfLVf a, float s) { return lvf(a.x * s, a.y * s, a.z * s, a.e * s); }
__device__ __forceinline__ GfLVf operator*(float s, GfLVf a) { return lvf(a.x * s, a.y * s, a.z * s, a.e * s); }
__device__ __forceinline__ float ldot(GfLVf a, GfLVf b) { return a.e * b.e - a.x * b.x - a.y * b.y - a.z * b.z; }
__device__ __forceinline__ float lmass(GfLVf a) { return sqrtf(ldot(a, a)); }
__device__ __forceinline__ GfLVf zt1(GfLVf q, GfLVf p, float mR) { return q - ldot(q, p) * p * (1.f / (mR * mR)); }
__device__ __forceinline__ GfLVf ssv(GfLVf p, float mR, GfLVf v) { return -1.0f * v + p * (ldot(p, v) / (mR * mR)); }
__device__ __forceinline__ float ssvs(GfLVf p, float mR, GfLVf l, GfLVf r) { return ldot(l, ssv(p, mR, r)); }
__device__ __forceinline__ float ssts(GfLVf p, float mR, GfLVf lm, GfLVf ln, GfLVf ra, GfLVf rb) {
    const float manb = ssvs(p, mR, lm, ra) * ssvs(p, mR, ln, rb);
    const float mbna = ssvs(p, mR, lm, rb) * ssvs(p, mR, ln, ra);
    const float mnab = ssvs(p, mR, lm, ln) * ssvs(p, mR, ra, rb);
    return 0.5f * (manb + mbna) - (1.f / 3.f) * mnab;
}
__device__ __forceinline__ GfLVf zt2c(GfLVf q, GfLVf p, float mR, GfLVf v) {
    const GfLVf t = zt1(q, p, mR);
    const float f = (1.f / 3.f) * ldot(t, t), iu = 1.f / (mR * mR);
    const float tc[4] = {t.x, t.y, t.z, t.e}, pc[4] = {p.x, p.y, p.z, p.e};
    const float g[4][4] = {{-1, 0, 0, 0}, {0, -1, 0, 0}, {0, 0, -1, 0}, {0, 0, 0, 1}};
    GfLVf row[4];
#pragma unroll
    for(int i = 0; i < 4; ++i) {
        float r[4];
#pragma unroll
        for(int j = 0; j < 4; ++j)
            r[j] = tc[i] * tc[j] - f * (g[i][j] - pc[i] * pc[j] * iu);
        row[i] = lvf(r[0], r[1], r[2], r[3]);
    }
    return v.e * row[3] - v.x * row[0] - v.y * row[1] - v.z * row[2];
}
__device__ __forceinline__ GfLVf leps3(GfLVf a, GfLVf b, GfLVf c) {
    GfLVf v;
    v.e = -1.f * a.x * (b.y * c.z - b.z * c.y) - a.y * (b.z * c.x - b.x * c.z) - a.z * (b.x * c.y - b.y * c.x);
    v.z = a.x * (b.e * c.y - b.y * c.e) + a.y * (b.x * c.e - b.e * c.x) + a.e * (b.y * c.x - b.x * c.y);
    v.y = a.x * (b.z * c.e - b.e * c.z) + a.z * (b.e * c.x - b.x * c.e) + a.e * (b.x * c.z - b.z * c.x);
    v.x = a.y * (b.e * c.z - b.z * c.e) + a.z * (b.y * c.e - b.e * c.y) + a.e * (b.z * c.y - b.y * c.z);
    return v;
}
__device__ __forceinline__ float gf_spinfactor_f(int kind, float mD0, GfLVf P1, GfLVf P2, GfLVf P3, GfLVf P4) {
    switch(kind) {
    case 1: { const GfLVf pV = P3 + P4, qV = P3 - P4, pP = pV + P2, qP = pV - P2;
              return ldot(zt1(qP, pP, lmass(pP)), zt1(qV, pV, lmass(pV))); }
    case 2: { const GfLVf pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4;
              const float MV1 = sqrtf(ldot(pV1, pV1)), MV2 = sqrtf(ldot(pV2, pV2));
              return (ldot(qV1, qV2) - ldot(qV1, pV1) * ldot(pV1, qV2) / (MV1 * MV1) -
                      ldot(qV1, pV2) * ldot(pV2, qV2) / (MV2 * MV2) +
                      ldot(qV1, pV1) * ldot(pV1, pV2) * ldot(pV2, qV2) / (MV1 * MV1 * MV2 * MV2)); }
    case 3: { const GfLVf pV1 = P1 + P2, qV1 = P2 - P1, pV2 = P3 + P4, qV2 = P4 - P3, pD = pV1 + pV2, qD = pV1 - pV2;
              const float MV1 = sqrtf(ldot(pV1, pV1)), MV2 = sqrtf(ldot(pV2, pV2));
              return -ldot(leps3(pD, zt1(qD, pD, lmass(pD)), zt1(qV1, pV1, MV1)), zt1(qV2, pV2, MV2)); }
    case 4: { const GfLVf pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4, pD = pV1 + pV2, qD = pV1 - pV2;
              return ldot(zt1(qV1, pV1, lmass(pV1)), zt2c(qD, pD, lmass(pD), zt1(qV2, pV2, lmass(pV2)))); }
    case 5: { const GfLVf pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, pD = P1 + pA, qD = pA - P1;
              return -ldot(zt1(qD, pD, lmass(pD)), ssv(pA, lmass(pA), zt1(qV, pV, lmass(pV)))); }
    case 6: { const GfLVf pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, qA = P2 - pV, pD = P1 + pA, qD = pA - P1;
              return ldot(zt1(qD, pD, lmass(pD)), zt2c(qA, pA, lmass(pA), zt1(qV, pV, lmass(pV)))); }
    case 7: { const GfLVf pS = P3 + P4, pV = P1 + P2, qV = P1 - P2, pD = pV + pS, qD = pV - pS;
              return ldot(zt1(qD, pD, lmass(pD)), zt1(qV, pV, lmass(pV))); }
    case 8: { const GfLVf pV1 = P2 + P3 + P4, pV2 = P3 + P4, qV1 = (P3 + P4) - P2, qV2 = P3 - P4;
              const float MV1 = lmass(pV1), MV2 = lmass(pV2);
              const GfLVf pD = pV1 + P1, qD = pV1 - P1;
              return ldot(leps3(pV1, zt1(qV1, pV1, MV1), zt1(qV2, pV2, MV2)), ssv(pV1, MV1, zt1(qD, pD, lmass(pD)))); }
    case 9: { const GfLVf pS = P3 + P4, pA = P2 + pS, qA = pS - P2, pD = pA + P1, qD = pA - P1;
              return ldot(zt1(qD, pD, lmass(pD)), zt1(qA, pA, lmass(pA))); }
    case 10: { const GfLVf pV = P3 + P4, qV = P3 - P4, pT = P2 + pV, qT = pV - P2, pD = P1 + pT, qD = pT - P1;
               const float mT = lmass(pT);
               const GfLVf tV = zt1(qV, pV, lmass(pV)), tD = zt1(qD, pD, lmass(pD)), t1T = zt1(qT, pT, mT);
               const GfLVf tmp = leps3(t1T, pT, ssv(pT, mT, tV));
               return ssts(pT, mT, tD, tD, tmp, t1T) + (1.f / 3.f) * ldot(tD, tD) / ldot(pT, pT) * ssts(pT, mT, pD, pD, tmp, t1T); }
    case 11: case 12: case 13: case 14: {
        const bool l12 = kind == 11 || kind == 12;
        const float a = l12 ? ldot(P1 + P2, P1 + P2) : ldot(P1 + P2 + P3, P1 + P2 + P3);
        const float b = l12 ? ldot(P3 + P4, P3 + P4) : ldot(P4, P4);
        const GfLVf T = P1 + P2 + P3 + P4;
        const float s = ldot(T, T);
        const float q2 = s / 4.f - (a + b) / 2.f + (a - b) * (a - b) / (4 * s);
        const float z2 = q2 * mD0 * mD0;
        const float ff = (kind == 11 || kind == 13) ? 1.0f / (1 + z2) : 1.0f / (z2 * z2 + 3 * z2 + 9);
        return sqrtf(ff); }
    default: return 1.0f;
    }
}
__device__ __forceinline__ float gf_blp_f(float z2, float z02, int L) {
    return L == 0 ? 1.0f : (L == 1 ? (1 + z02) / (1 + z2) : (z02 * z02 + 3 * z02 + 9) / (z2 * z2 + 3 * z2 + 9));
}
__device__ __forceinline__ float gf_bl_f(float z2, int L) {
    return L == 0 ? 1.0f : (L == 1 ? 2 * z2 / (1 + z2) : (13 * z2 * z2) / (z2 * z2 + 3 * z2 + 9));
}
__device__ __forceinline__ float gf_bl2_f(float z2, int L) {
    return L == 0 ? 1.0f : (L == 1 ? 1.0f / (1 + z2) : 1.0f / (z2 * z2 + 3 * z2 + 9));
}
// FP32 throughout: the pair mass comes from FP32 four-vectors, so an FP64 threshold or pole difference would
// not recover precision; the pole term's absolute error (~5e-8) is far below the width term m Gamma(m)
__device__ __forceinline__ float2 gf_lineshape_f(bool sbw, float Mpair, float m1, float m2, float mass, float width,
                                                 int orbital, int FF, float radius) {
    const float mr2 = Mpair * Mpair;
    const float mpsq = (m1 + m2) * (m1 + m2), mmsq = (m1 - m2) * (m1 - m2);
    const float ms2 = mass * mass;
    const float pABSq = (mr2 - mpsq) * (mr2 - mmsq) / (4 * mr2);
    float prSq        = (ms2 - mpsq) * (ms2 - mmsq) / (4 * ms2);
    const float prSq2 = prSq < 0 ? 0.0f : prSq;
    prSq              = fabsf(prSq);
    const float r2    = radius * radius;
    float fr          = 1.0f;
    if(0 != orbital && 0 != FF) {
        fr = (FF == 1 ? gf_bl_f(pABSq * r2, orbital) : gf_blp_f(pABSq * r2, prSq2 * r2, orbital));
        fr = (FF == 3 ? gf_bl2_f(pABSq * r2, orbital) : fr);
    }
    const float m = mass, w = width;
    float GofM, k;
    if(!sbw) {
        const float pratio = sqrtf(pABSq / prSq);
        float pj           = 1.0f;
        for(int i = 0; i < 2 * orbital + 1; i++)
            pj = pj * pratio;
        GofM = w * pj * (m / Mpair) * gf_blp_f(pABSq * r2, prSq * r2, orbital);
        const float gamma = m * sqrtf((m * m + w * w));
        k = 0.90031631615710606f * m * w * gamma / sqrtf(m * m + gamma); // 2 sqrt(2) / pi
    } else {
        GofM = w;
        const float gamma = sqrtf(m * m * (m * m + w * w));
        k = m * w * gamma / sqrtf(m * m + gamma);
    }
    const float dm2 = ms2 - mr2;
    const float den = dm2 * dm2 + m * GofM * m * GofM;
    const float f   = sqrtf(k * fr) / den;
    return make_float2(f * dm2, f * (m * GofM));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// get4Vecs (the FP64 gf_get4vecs above, same formulas and order) in FP32
__device__ __forceinline__ void gf_get4vecs_f(GfLVf *P, float m12, float m34, float cos12, float cos34, float phi,
                                              float M, float m1, float m2, float m3, float m4) {
    const float E1 = (m12 * m12 + m1 * m1 - m2 * m2) / (2 * m12), E2 = (m12 * m12 - m1 * m1 + m2 * m2) / (2 * m12);
    const float E3 = (m34 * m34 + m3 * m3 - m4 * m4) / (2 * m34), E4 = (m34 * m34 - m3 * m3 + m4 * m4) / (2 * m34);
    const float p1 = sqrtf(fmaxf(E1 * E1 - m1 * m1, 0.f)), p3 = sqrtf(fmaxf(E3 * E3 - m3 * m3, 0.f));
    const float sin12 = sqrtf(fmaxf(1 - cos12 * cos12, 0.f)), sin34 = sqrtf(fmaxf(1 - cos34 * cos34, 0.f));
    const float ED1 = (M * M + m12 * m12 - m34 * m34) / (2 * m12), PD1 = sqrtf(fmaxf(ED1 * ED1 - M * M, 0.f));
    const float beta1 = PD1 / ED1, gamma1 = 1.0f / sqrtf(1 - beta1 * beta1);
    const float ED2 = (M * M - m12 * m12 + m34 * m34) / (2 * m34), PD2 = sqrtf(fmaxf(ED2 * ED2 - M * M, 0.f));
    const float beta2 = -PD2 / ED2, gamma2 = 1.0f / sqrtf(1 - beta2 * beta2);
    const float x[4] = {cos12 * p1, -cos12 * p1, -cos34 * p3, cos34 * p3};
    const float y[4] = {sin12 * p1, -sin12 * p1, -sin34 * p3, sin34 * p3};
    const float E[4] = {E1, E2, E3, E4};
    float sp, cp;
    sincosf(phi, &sp, &cp);
#pragma unroll
    for(int k = 0; k < 4; ++k) {
        const float g = k < 2 ? gamma1 : gamma2, b = k < 2 ? beta1 : beta2;
        P[k].e = g * (E[k] + b * x[k]);
        P[k].x = g * (x[k] + b * E[k]);
        P[k].z = k < 2 ? sp * y[k] : 0.0f;
        P[k].y = k < 2 ? cp * y[k] : y[k];
    }
}
// the pair / triple invariant masses of gf_pairmass in FP32
__device__ __forceinline__ float gf_pairmass_f(int pair, const GfLVf *P, float m1, float m2, float m3, float m4,
                                               float &d1, float &d2) {
    switch(pair) {
    case 0: d1 = m1; d2 = m2; return lmass(P[0] + P[1]);
    case 1: d1 = m3; d2 = m4; return lmass(P[2] + P[3]);
    case 2: d1 = m1; d2 = m3; return lmass(P[0] + P[2]);
    case 3: d1 = m1; d2 = m4; return lmass(P[0] + P[3]);
    case 4: d1 = m2; d2 = m3; return lmass(P[1] + P[2]);
    case 5: d1 = m2; d2 = m4; return lmass(P[1] + P[3]);
    case 6: d1 = lmass(P[0] + P[1]); d2 = m3; return lmass(P[0] + P[1] + P[2]);
    case 7: d1 = lmass(P[0] + P[2]); d2 = m2; return lmass(P[0] + P[1] + P[2]);
    case 8: d1 = lmass(P[1] + P[2]); d2 = m1; return lmass(P[0] + P[1] + P[2]);
    case 9: d1 = lmass(P[0] + P[1]); d2 = m4; return lmass(P[0] + P[1] + P[3]);
    case 10: d1 = lmass(P[0] + P[3]); d2 = m2; return lmass(P[0] + P[1] + P[3]);
    case 11: d1 = lmass(P[1] + P[3]); d2 = m1; return lmass(P[0] + P[1] + P[3]);
    case 12: d1 = lmass(P[0] + P[2]); d2 = m4; return lmass(P[0] + P[2] + P[3]);
    case 13: d1 = lmass(P[0] + P[3]); d2 = m3; return lmass(P[0] + P[2] + P[3]);
    case 14: d1 = lmass(P[2] + P[3]); d2 = m1; return lmass(P[0] + P[2] + P[3]);
    case 15: d1 = lmass(P[1] + P[2]); d2 = m4; return lmass(P[1] + P[2] + P[3]);
    case 16: d1 = lmass(P[1] + P[3]); d2 = m3; return lmass(P[1] + P[2] + P[3]);
    default: d1 = lmass(P[2] + P[3]); d2 = m2; return lmass(P[1] + P[2] + P[3]);
    }
}
)CUDA";

// The 4-body line shapes for double or dual mass / width (the value path uses T = double).
const char *kPreludeAmp4T = R"CUDA(
template <typename T>
__device__ __forceinline__ T gf_blp_t(T z2, T z02, int L) {
    return L == 0 ? T(1.0) : (L == 1 ? (1 + z02) / (1 + z2) : (z02 * z02 + 3 * z02 + 9) / (z2 * z2 + 3 * z2 + 9));
}
template <typename T>
__device__ __forceinline__ void gf_lineshape_t(bool sbw, double Mpair, double m1, double m2, T mass, T width,
                                               int orbital, int FF, double radius, T &re, T &im) {
    const double mr2 = Mpair * Mpair;
    const double mpsq = (m1 + m2) * (m1 + m2), mmsq = (m1 - m2) * (m1 - m2);
    const double num = (mr2 - mpsq) * (mr2 - mmsq);
    const T num2 = (mass * mass - mpsq) * (mass * mass - mmsq);
    const double pABSq = num / (4 * mr2);
    T prSq = num2 / (4 * mass * mass);
    const T prSq2 = dval(prSq) < 0 ? T(0.0) : prSq;
    prSq = fabs(prSq);
    const double r2 = radius * radius;
    T fr = T(1.0);
    if(0 != orbital && 0 != FF) {
        fr = (FF == 1 ? T(gf_bl(pABSq * r2, orbital)) : gf_blp_t<T>(T(pABSq * r2), prSq2 * r2, orbital));
        fr = (FF == 3 ? T(gf_bl2(pABSq * r2, orbital)) : fr);
    }
    T GofM, k;
    if(!sbw) {
        const T pratio = sqrt(pABSq / prSq);
        T pj = T(1.0);
        for(int i = 0; i < 2 * orbital + 1; i++)
            pj = pj * pratio;
        GofM = width * pj * (mass / Mpair) * gf_blp_t<T>(T(pABSq * r2), prSq * r2, orbital);
        const T gamma = mass * sqrt((mass * mass + width * width));
        k = (2.0 * sqrt(2.0) / 3.14159265358979323846) * mass * width * gamma / sqrt(mass * mass + gamma);
    } else {
        GofM = width;
        const T gamma = sqrt(mass * mass * (mass * mass + width * width));
        k = mass * width * gamma / sqrt(mass * mass + gamma);
    }
    const T den = (mass * mass - mr2) * (mass * mass - mr2) + mass * GofM * mass * GofM;
    const T f = sqrt(k * fr) / den;
    re = f * (mass * mass - mr2);
    im = f * (mass * GofM);
}
)CUDA";

// The 3-body relativistic Breit-Wigner for double or dual mass / width, FP64 (the derivative path).
const char *kPreludeAmp3T = R"CUDA(
template <typename T>
__device__ __forceinline__ T gf_tb_mom_t(T s, double a, double b) {
    T k1 = 1.0 - (a + b) * (a + b) / s;
    k1   = dval(k1) >= 0 ? sqrt(k1) : T(1.0);
    T k2 = 1.0 - (a - b) * (a - b) / s;
    k2   = dval(k2) >= 0 ? sqrt(k2) : T(1.0);
    return 0.5 * sqrt(s) * k1 * k2;
}
template <typename T>
__device__ __forceinline__ T gf_tb_mom_mother_t(T s, double M, double c) {
    T k1 = 1.0 - (M + c) * (M + c) / s;
    k1   = dval(k1) >= 0 ? sqrt(k1) : T(1.0);
    T k2 = 1.0 - (M - c) * (M - c) / s;
    k2   = dval(k2) >= 0 ? sqrt(k2) : T(1.0);
    return 0.5 * s * k1 * k2 / M;
}
template <typename T>
__device__ __forceinline__ T gf_damp2_t(T p, int spin, double r) {
    const T sq = r * r * p * p;
    return spin == 2 ? 13.0 * sq / ((sq - 3.0) * (sq - 3.0)) + 9.0 * sq * sq : 2.0 * sq;
}
template <typename T>
__device__ __forceinline__ T gf_damp2n_t(T p, int spin, double r) {
    const T sq = r * r * p * p;
    const T d  = 1.0 + sq;
    return spin == 2 ? d + 8.0 + 2.0 * sq + sq * sq : d;
}
__device__ __forceinline__ double gf_spin_d(int spin, double M, double m1, double m2, double m3, double m12, double m13,
                                            double m23, int cyc) {
    if(spin == 0)
        return 1.0;
    const double mA = cyc == 0 ? m1 : (cyc == 1 ? m3 : m2), mB = cyc == 0 ? m2 : (cyc == 1 ? m1 : m3);
    const double mC = cyc == 0 ? m3 : (cyc == 1 ? m2 : m1);
    const double mAC = cyc == 0 ? m13 : (cyc == 1 ? m23 : m12), mBC = cyc == 0 ? m23 : (cyc == 1 ? m12 : m13);
    const double mAB = cyc == 0 ? m12 : (cyc == 1 ? m13 : m23);
    const double massFactor = 1.0 / mAB;
    const double MC = M * M - mC * mC, AB = mA * mA - mB * mB;
    double sf = -((mBC - mAC) + massFactor * MC * AB);
    if(spin == 2) {
        sf *= sf;
        double ex = ((mAB - 2 * M * M - 2 * mC * mC) + massFactor * MC * MC);
        ex *= ((mAB - 2 * mA * mA - 2 * mB * mB) + massFactor * AB * AB);
        ex /= 3;
        sf -= ex;
    }
    return sf;
}
template <int I, typename T>
__device__ __forceinline__ void gf_rbw_t(double m12, double m13, double m23, T mass, T width, int spin, int cyc,
                                         bool norm, double M, double m1, double m2, double m3, double r, double rm,
                                         T &re, T &im) {
    re = T(0.0);
    im = T(0.0);
    const T rm2 = mass * mass;
#pragma unroll
    for(int it = 0; it < I; ++it) {
        const double sq = cyc == 0 ? m12 : (cyc == 1 ? m13 : m23);
        const double d1 = cyc == 2 ? m2 : m1, d2 = cyc == 0 ? m2 : m3;
        const double bach = cyc == 0 ? m3 : (cyc == 1 ? m2 : m1);
        T fr = T(1.0), frM = T(1.0);
        const double pm = gf_tb_mom_t<double>(sq, d1, d2);
        const T pn      = gf_tb_mom_t<T>(rm2, d1, d2);
        double pmM;
        T pnM = T(0.0);
        if(norm) {
            pmM = gf_tb_mom_mother_t<double>(sq, M, bach);
            pnM = gf_tb_mom_mother_t<T>(rm2, M, bach);
        } else
            pmM = gf_tb_mom_t<double>(M * M, sqrt(sq), bach);
        if(spin != 0) {
            if(norm) {
                fr  = gf_damp2n_t<T>(pn, spin, r) / gf_damp2n_t<double>(pm, spin, r);
                frM = gf_damp2n_t<T>(pnM, spin, rm) / gf_damp2n_t<double>(pmM, spin, rm);
            } else {
                fr  = T(gf_damp2_t<double>(pm, spin, r));
                frM = T(gf_damp2_t<double>(pmM, spin, rm));
            }
        }
        const T A = rm2 - sq;
        const T q = pm / pn;
        T qp      = q;
        for(int k = 0; k < 2 * spin; ++k)
            qp = qp * q;
        const T B = rm2 * width * qp * fr / sqrt(sq);
        const T C = 1.0 / (A * A + B * B);
        T xr = A * C, xi = B * C;
        const T f1 = sqrt(fr), f2 = sqrt(frM);
        const double sf = gf_spin_d(spin, M, m1, m2, m3, m12, m13, m23, cyc);
        xr = xr * f1 * f2 * sf;
        xi = xi * f1 * f2 * sf;
        re = re + xr;
        im = im + xi;
        if(I > 1)
            cyc = (cyc + 1) % 3;
    }
}
)CUDA";

// Forward-mode dual numbers (value and the derivatives with respect to a resonance's mass and width) for the
// analytic gradient of the cached amplitudes, and the relativistic Breit-Wigner of the 3-body path written
// once for double and for duals (FP64 throughout: it runs only when those parameters change).
const char *kPreludeDual = R"CUDA(
struct GfDual {
    double v, a, b;
    __device__ __forceinline__ GfDual(double v_ = 0, double a_ = 0, double b_ = 0) : v(v_), a(a_), b(b_) {}
};
__device__ __forceinline__ double dval(double x) { return x; }
__device__ __forceinline__ double dval(const GfDual &x) { return x.v; }
__device__ __forceinline__ GfDual operator+(GfDual x, GfDual y) { return GfDual(x.v + y.v, x.a + y.a, x.b + y.b); }
__device__ __forceinline__ GfDual operator-(GfDual x, GfDual y) { return GfDual(x.v - y.v, x.a - y.a, x.b - y.b); }
__device__ __forceinline__ GfDual operator-(GfDual x) { return GfDual(-x.v, -x.a, -x.b); }
__device__ __forceinline__ GfDual operator*(GfDual x, GfDual y) {
    return GfDual(x.v * y.v, x.a * y.v + x.v * y.a, x.b * y.v + x.v * y.b);
}
__device__ __forceinline__ GfDual operator/(GfDual x, GfDual y) {
    const double q = x.v / y.v;
    return GfDual(q, (x.a - q * y.a) / y.v, (x.b - q * y.b) / y.v);
}
__device__ __forceinline__ GfDual operator+(GfDual x, double y) { return GfDual(x.v + y, x.a, x.b); }
__device__ __forceinline__ GfDual operator+(double y, GfDual x) { return GfDual(x.v + y, x.a, x.b); }
__device__ __forceinline__ GfDual operator-(GfDual x, double y) { return GfDual(x.v - y, x.a, x.b); }
__device__ __forceinline__ GfDual operator-(double y, GfDual x) { return GfDual(y - x.v, -x.a, -x.b); }
__device__ __forceinline__ GfDual operator*(GfDual x, double y) { return GfDual(x.v * y, x.a * y, x.b * y); }
__device__ __forceinline__ GfDual operator*(double y, GfDual x) { return GfDual(x.v * y, x.a * y, x.b * y); }
__device__ __forceinline__ GfDual operator/(GfDual x, double y) { return GfDual(x.v / y, x.a / y, x.b / y); }
__device__ __forceinline__ GfDual operator/(double y, GfDual x) {
    const double q = y / x.v;
    return GfDual(q, -q * x.a / x.v, -q * x.b / x.v);
}
__device__ __forceinline__ GfDual sqrt(GfDual x) {
    const double r = sqrt(x.v);
    return GfDual(r, x.a / (2 * r), x.b / (2 * r));
}
__device__ __forceinline__ GfDual fabs(GfDual x) { return x.v < 0 ? -x : x; }
// Single precision (the mixed engine's floated line shapes): sums and differences with an FP64 operand are
// formed in FP64 and rounded once (the pole difference mass^2 - m^2 cancels near the pole), every other
// operation is FP32.
struct GfDualF {
    float v, a, b;
    __device__ __forceinline__ GfDualF(float v_ = 0.f, float a_ = 0.f, float b_ = 0.f) : v(v_), a(a_), b(b_) {}
    __device__ __forceinline__ GfDualF(double v_) : v((float)v_), a(0.f), b(0.f) {}
    __device__ __forceinline__ GfDualF(int v_) : v((float)v_), a(0.f), b(0.f) {}
};
__device__ __forceinline__ float dval(const GfDualF &x) { return x.v; }
__device__ __forceinline__ GfDualF operator+(GfDualF x, GfDualF y) { return GfDualF(x.v + y.v, x.a + y.a, x.b + y.b); }
__device__ __forceinline__ GfDualF operator-(GfDualF x, GfDualF y) { return GfDualF(x.v - y.v, x.a - y.a, x.b - y.b); }
__device__ __forceinline__ GfDualF operator-(GfDualF x) { return GfDualF(-x.v, -x.a, -x.b); }
__device__ __forceinline__ GfDualF operator*(GfDualF x, GfDualF y) {
    return GfDualF(x.v * y.v, x.a * y.v + x.v * y.a, x.b * y.v + x.v * y.b);
}
__device__ __forceinline__ GfDualF operator/(GfDualF x, GfDualF y) {
    const float q = x.v / y.v;
    return GfDualF(q, (x.a - q * y.a) / y.v, (x.b - q * y.b) / y.v);
}
__device__ __forceinline__ GfDualF operator+(GfDualF x, double y) { return GfDualF((float)((double)x.v + y), x.a, x.b); }
__device__ __forceinline__ GfDualF operator+(double y, GfDualF x) { return GfDualF((float)((double)x.v + y), x.a, x.b); }
__device__ __forceinline__ GfDualF operator-(GfDualF x, double y) { return GfDualF((float)((double)x.v - y), x.a, x.b); }
__device__ __forceinline__ GfDualF operator-(double y, GfDualF x) { return GfDualF((float)(y - (double)x.v), -x.a, -x.b); }
__device__ __forceinline__ GfDualF operator*(GfDualF x, double y) {
    const float f = (float)y;
    return GfDualF(x.v * f, x.a * f, x.b * f);
}
__device__ __forceinline__ GfDualF operator*(double y, GfDualF x) { return x * y; }
__device__ __forceinline__ GfDualF operator/(GfDualF x, double y) {
    const float f = (float)y;
    return GfDualF(x.v / f, x.a / f, x.b / f);
}
__device__ __forceinline__ GfDualF operator/(double y, GfDualF x) {
    const float q = (float)y / x.v;
    return GfDualF(q, -q * x.a / x.v, -q * x.b / x.v);
}
__device__ __forceinline__ GfDualF sqrt(GfDualF x) {
    const float r = sqrtf(x.v);
    return GfDualF(r, x.a / (2.f * r), x.b / (2.f * r));
}
__device__ __forceinline__ GfDualF fabs(GfDualF x) { return x.v < 0 ? -x : x; }
)CUDA";

// Where every normalisation factor is kept (see NormLayout in tree.h).
NormLayout computeNormLayout(const Tree &T) {
    NormLayout nl;
    nl.npr = T.n_params;
    for(size_t i = 0; i < T.nodes.size(); ++i) {
        if(T.nk[i] != NK_EXP && T.nk[i] != NK_GAUSS && T.nk[i] != NK_AMP3 && T.nk[i] != NK_AMP4)
            continue;
        NormLayout::Analytic a;
        a.node   = (int)i;
        a.kind   = T.nk[i];
        a.slotN  = nl.npr++;
        a.slotNL = nl.npr++;
        for(int s : T.dep_norm[i])
            a.dN.push_back({s, nl.npr++});
        nl.analytic.push_back(a);
    }
    nl.qN.assign(T.nums.size(), -1);
    nl.qNL.assign(T.nums.size(), -1);
    nl.qdN.assign(T.nums.size(), {});
    for(size_t q = 0; q < T.nums.size(); ++q) {
        int i     = T.nums[q].node;
        nl.qN[q]  = nl.nq++;
        nl.qNL[q] = nl.nq++;
        for(int s : T.dep_norm[i])
            nl.qdN[q].push_back({s, nl.nq++});
    }
    return nl;
}

// Parameters (type R) of the toy from its record.
void emitParamsR(std::ostream &os, const Tree &T, const NormLayout &nl, const char *ind) {
    os << ind << "const R *Pr = reinterpret_cast<const R *>(GF_PR) + (i64)toy * " << nl.npr << "; (void)Pr;\n";
    for(int j = 0; j < T.n_params; ++j)
        os << ind << "const R p" << j << " = Pr[" << j << "]; (void)p" << j << ";\n";
}

// Normalisation factors used by the event pass: analytic ones from the record, numeric ones from Nq.
void emitNormReads(std::ostream &os, const Tree &T, bool grad, const NormLayout &nl, const char *ind) {
    if(nl.nq > 0)
        os << ind << "const R *Nq = reinterpret_cast<const R *>(a.Nq) + (i64)toy * " << nl.nq << ";\n";
    for(auto &an : nl.analytic) {
        os << ind << "const R N" << an.node << " = Pr[" << an.slotN << "], NL" << an.node << " = Pr[" << an.slotNL
           << "]; (void)NL" << an.node << ";\n";
        if(grad)
            for(auto &d : an.dN)
                os << ind << "const R dN" << an.node << "_" << d.first << " = Pr[" << d.second << "];\n";
    }
    for(size_t q = 0; q < T.nums.size(); ++q) {
        int i = T.nums[q].node;
        os << ind << "const R N" << i << " = Nq[" << nl.qN[q] << "], NL" << i << " = Nq[" << nl.qNL[q] << "]; (void)NL"
           << i << ";\n";
        if(grad)
            for(auto &d : nl.qdN[q])
                os << ind << "const R dN" << i << "_" << d.first << " = Nq[" << d.second << "];\n";
    }
}

int padComps(int c) { return c <= 1 ? 1 : c <= 2 ? 2 : (c + 3) / 4 * 4; }

// Sums K per-thread values (ACC expressions) over a warp into red[wid][0..K) by a transposed butterfly
// (recursive halving): at each of the five exchange steps a lane keeps one half of its values and sends the other half to its
// partner, so that a warp exchanges about K values instead of 5 K.  Components go in groups of at most 32;
// after the exchanges a lane holds one component, summed over the warp.  Ends with __syncthreads().
void emitCtaReduce(std::ostream &os, const std::vector<std::string> &vals, const std::string &ind) {
    const int K = (int)vals.size();
    for(int g0 = 0; g0 < K; g0 += 32) {
        const int k = std::min(32, K - g0);
        int kp      = 1;
        while(kp < k)
            kp <<= 1;
        os << ind << "{\n";
        for(int i = 0; i < kp; ++i)
            os << ind << "  ACC t" << i << " = " << (i < k ? vals[g0 + i] : std::string("acc_zero()")) << ";\n";
        int m = kp, dup = 0;
        std::vector<std::pair<int, int>> halves;
        for(int o = 16; o > 0; o >>= 1) {
            if(m >= 2) {
                const int h = m / 2;
                os << ind << "  { const bool b = (lane & " << o << ") != 0;\n";
                for(int i = 0; i < h; ++i)
                    os << ind << "    { const ACC s = b ? t" << i << " : t" << i + h << ", q = b ? t" << i + h << " : t"
                       << i << "; t" << i << " = acc_add(q, acc_shfl_xor(s, " << o << ")); }\n";
                os << ind << "  }\n";
                halves.push_back({o, h});
                m = h;
            } else {
                os << ind << "  t0 = acc_add(t0, acc_shfl_xor(t0, " << o << "));\n";
                dup |= o;
            }
        }
        os << ind << "  if((lane & " << dup << ") == 0) {\n";
        os << ind << "    const int c = " << g0;
        for(auto &hv : halves)
            os << " + ((lane & " << hv.first << ") ? " << hv.second << " : 0)";
        os << ";\n";
        os << ind << "    if(c < " << g0 + k << ") red[wid][c] = t0;\n";
        os << ind << "  }\n";
        os << ind << "}\n";
    }
    os << ind << "__syncthreads();\n";
}

// convolution tables in the event pass: staged in shared memory per CTA (default) or read through L1
// (GF_CTAB=l1)
// GF_EVT_TAB=0: the one-launch kernel evaluates the event function per event even where it could tabulate it
bool tabDisabled() {
    const char *v = std::getenv("GF_EVT_TAB");
    return v && v[0] == '0';
}

bool ctabThroughL1() {
    const char *v = std::getenv("GF_CTAB");
    return v && std::string(v) == "l1";
}

struct Gen {
    const Tree &T;
    bool mixed;
    int block;
    bool batch; // many toys per launch: fewer, larger CTAs for the tables and grids
    KernelPlan &plan;
    std::ostringstream os;
    const bool ctabL1 = ctabThroughL1();
    // amplitude trees with floated line-shape / resonance parameters: also emit the recompute-mode kernels
    // (gf_evt_gr, gf_gramr); `recompute` is set while the event pass of that mode is generated
    bool recomputeKernels = false;
    bool recompute        = false;
    Shapes shapes;
    bool countDecl = false; // the counting pass's shared variables have been declared
    // rows (bins) a CTA's events may span for the counting pass of the tabulated event pass
    static constexpr int kCountRows = 256;

    // per-toy column pointer i of table `tab` (n per toy); one toy: from the kernel arguments at p0[off + i]
    static std::string p0ptr(const char *tab, int n, int i, int off) {
        return "(a.n_toys == 1 ? a.p0[" + std::to_string(off + i) + "] : (const void *)" + tab + "[(i64)toy * " +
               std::to_string(n) + " + " + std::to_string(i) + "])";
    }

    int convComps(int ci, bool grad) const { return 1 + (grad ? (int)T.convs[ci].dep.size() : 0); }
    // Strides of the conv kernel's staged arrays: multiples of 4 elements (16-byte loads of 4 FP32 values),
    // congruent to 8 modulo 32 (successive arrays start 8 banks apart)
    static int convStride(int n) { return n + (((8 - n) % 32) + 32) % 32; }

    // Table layout per toy: for each conv, AoS [k][cp] with cp = padded component count (16-byte rows).
    // Counting pass of the tabulated event pass (events sorted by bin, staged in shared memory): every event's
    // bin offset is read once, 8 per thread and step, and each run of equal offsets records its start in
    // gf_rstart[bin - kr_lo]; the events of a bin are then the distance to the next run's start.  Emitted after
    // the table loads were issued and before their first use, so that it runs while they are in flight (it
    // holds no barrier, which would wait for them).  cnt_ok = 0 (the per-event loop instead) for unsorted or
    // unstaged events, and for a range over more than kCountRows bins.
    void emitCountPass(const ConvInfo &cv) {
        os << "  {\n";
        os << "    const i64 ee = (i64)ce * a.chunk < a.nevt0 ? (i64)ce * a.chunk : a.nevt0;\n";
        os << "    cnt_ok = a.ksort != nullptr && gf_st != nullptr && cb < ce && ee > gf_ib && cnt_nrows > 0 && cnt_nrows <= "
           << kCountRows << ";\n";
        os << "    if(cnt_ok) {\n";
        os << "      cnt_nev = (int)(ee - gf_ib);\n";
        os << "      const int *ks = reinterpret_cast<const int *>(gf_st + gf_soff[0]);\n";
        os << "      for(int i0 = 8 * tid; i0 < cnt_nev; i0 += " << 8 * block << ") {\n";
        os << "        const int4 u = *reinterpret_cast<const int4 *>(ks + i0), w = *reinterpret_cast<const int4 *>(ks + i0 + 4);\n";
        os << "        const int kv[8] = {u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w};\n";
        os << "        int prev = i0 > 0 ? ks[i0 - 1] : " << cv.kmin - 1 << ";\n";
        os << "#pragma unroll\n        for(int j = 0; j < 8; ++j) {\n";
        os << "          const int r = kv[j] - " << cv.kmin << " - kr_lo;\n";
        os << "          if(i0 + j < cnt_nev && kv[j] != prev && r >= 0 && r < cnt_nrows) gf_rstart[r] = i0 + j;\n";
        os << "          prev = kv[j];\n        }\n      }\n    }\n  }\n";
    }

    // The event function of the tabulated pass can be evaluated with gf_df: only sums, products and quotients
    // (AddPdf, ProdPdf, constant polynomials) above the convolution, whose model and resolution the table kernel
    // evaluates.
    bool dfEligible() const {
        std::vector<int> st{0};
        while(!st.empty()) {
            const TNode &n = T.nodes[st.back()];
            st.pop_back();
            switch(n.op) {
            case GF_OP_CONVOLUTION:
            case GF_OP_POLYNOMIAL:
            case GF_OP_POLYNOMIAL_OFFSET: break;
            case GF_OP_ADD:
            case GF_OP_ADD_EXT:
            case GF_OP_PROD:
                for(int ch : n.children)
                    st.push_back(ch);
                break;
            default: return false;
            }
        }
        return true;
    }
    void tableLayout(bool grad) {
        auto &off = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        off.clear();
        cps.clear();
        int64_t total = 0;
        for(size_t ci = 0; ci < T.convs.size(); ++ci) {
            int cp = padComps(convComps((int)ci, grad));
            total  = (total + 3) / 4 * 4;
            off.push_back(total);
            cps.push_back(cp);
            total += (int64_t)cp * T.convs[ci].nK;
        }
        total = (total + 3) / 4 * 4;
        int64_t &lo = grad ? plan.ctab_lo_off_grad : plan.ctab_lo_off_nograd;
        lo          = -1;
        if(mixed && !batch && !T.convs.empty()) {
            lo = total;
            total += (T.convs[0].nK + 3) / 4 * 4;
        }
        (grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd) = total;
    }

    // ---------------- numeric-normalisation plan ----------------
    struct ConvShape {
        int MS = 8, KT = 8, items = 0, KP = 1;
        std::vector<int> KB;
    };
    // m split across the 32 lanes of a warp for one toy when every table has at most 8 components (more
    // CTAs of fewer k each: one table is short and latency-bound); batches of toys, or more components: 8
    // lanes.  KB = table entries per CTA.
    ConvShape convShape(bool grad) const {
        ConvShape sh;
        int maxComps = 0;
        for(size_t ci = 0; ci < T.convs.size(); ++ci)
            maxComps = std::max(maxComps, convComps((int)ci, grad));
        sh.MS    = (!batch && maxComps <= block / 32) ? 32 : 8;
        // one toy: 4 entries per item tile, so that the table spreads over twice as many CTAs (its sums and lane
        // reductions halve per CTA; the launch has CTAs to spare, every one of which waits at the grid barrier)
        // (3 entries per item tile, 251 table CTAs for C2's 1501 entries, so that fewer SMs run two table CTAs:
        // the FCN took 19.1-19.3 us against 17.6-18.0 us at 4)
        sh.KT = batch ? 8 : 4;
        sh.items = block / sh.MS;
        // batches: each item covers KP k-tiles in turn, so that one CTA's staged model and resolution
        // arrays (whose evaluation is a third of the work at KP = 1) serve KP times the table entries;
        // 1024 toys of the composite model: KP 1 / 2 / 3 / 4 / 6 -> table kernel 0.58 / 0.51 / 0.48 /
        // 0.48 / 0.47 ms (GF_CONV_KP overrides)
        sh.KP = 1;
        if(batch) {
            const char *v = std::getenv("GF_CONV_KP");
            sh.KP = shapes.conv_kp > 0 ? std::min(8, shapes.conv_kp) : v ? std::max(1, std::min(8, std::atoi(v))) : 4;
        }
        plan.conv_kp = sh.KP;
        for(size_t ci = 0; ci < T.convs.size(); ++ci) {
            const int comps = convComps((int)ci, grad);
            if(comps > sh.items)
                throw std::runtime_error("codegen: too many convolution derivative components");
            sh.KB.push_back(sh.KT * (sh.items / comps) * sh.KP);
        }
        return sh;
    }
    void planNumerics() {
        const int NQ = (int)T.nums.size(), NC = (int)T.convs.size();
        const int BPB = plan.grid_bins_per_block;
        plan.grid_blocks.clear();
        plan.max_grid_blocks = 0;
        for(auto &g : T.nums) {
            const int nb = (int)((g.total + BPB - 1) / BPB);
            plan.grid_blocks.push_back(nb);
            plan.max_grid_blocks = std::max(plan.max_grid_blocks, nb);
        }
        plan.conv_fold_q.assign(NC, -1);
        plan.num_folded.assign(NQ, 0);
        plan.grid_needs_conv = false;
        for(int q = 0; q < NQ; ++q) {
            const NumInfo &g = T.nums[q];
            // one toy and batches: the one-launch evaluation then needs no barrier between tables and grids
            // (with separate launches for one toy the fold's finishing chain lengthens the table kernel by
            // about what the grid launch takes)
            bool fold = T.nodes[g.node].op == GF_OP_CONVOLUTION && g.obs.size() == 1 &&
                        g.convs.size() == 1 && g.convs[0] == T.conv_of[g.node] && plan.conv_fold_q[g.convs[0]] < 0;
            if(fold)
                for(auto &d : plan.nl.qdN[q]) {
                    const auto &dep = T.convs[g.convs[0]].dep;
                    if(std::find(dep.begin(), dep.end(), d.first) == dep.end())
                        fold = false;
                }
            if(!fold) {
                if(!g.convs.empty())
                    plan.grid_needs_conv = true;
                continue;
            }
            const int ci = g.convs[0];
            plan.conv_fold_q[ci] = q;
            plan.num_folded[q]   = 1;
            for(bool gr : {true, false}) {
                const int KB = convShape(gr).KB[ci];
                plan.max_grid_blocks = std::max(plan.max_grid_blocks, (T.convs[ci].nK + KB - 1) / KB);
            }
        }
    }
    // The normalisation factor of numeric node q (and its derivatives) from tot[0] = the grid sum and
    // tot[1 + s] = its derivative for gradient slot s (GooPdf::normalize numeric branch,
    // src/PDFs/GooPdf.cu:366-395), written to Nq; the grid sum to gsum; NaN / non-positive flags to qflag.
    void emitNumFinish(int q, bool grad, const std::string &ind) {
        const NumInfo &g  = T.nums[q];
        const int NQ      = (int)T.nums.size();
        const NormLayout &nl = plan.nl;
        // ((1 * volume) / bins), the reference's order of operations, evaluated on the host
        double c = 1.0;
        c *= g.volume;
        c /= (double)g.total;
        os << ind << "{\n";
        os << ind << "  R *Nq = reinterpret_cast<R *>(a.Nq) + (i64)toy * " << nl.nq << ";\n";
        os << ind << "  const double S = acc_value(tot[0]);\n";
        os << ind << "  a.gsum[(i64)toy * " << NQ << " + " << q << "] = S;\n";
        os << ind << "  if(isnan(S)) atomicOr(&a.qflag[toy], 1); else if(!(S > 0.0)) atomicOr(&a.qflag[toy], 2);\n";
        os << ind << "  const double I = " << lit(c) << " * S;\n";
        os << ind << "  const double Nd = 1.0 / I;\n";
        os << ind << "  const R N = (R)Nd;\n";
        os << ind << "  Nq[" << nl.qN[q] << "] = N;\n";
        os << ind << "  Nq[" << nl.qNL[q] << "] = (R)(Nd - (double)N);\n";
        if(grad)
            for(auto &d : nl.qdN[q])
                os << ind << "  Nq[" << d.second << "] = -N * N * (R)" << lit(c) << " * (R)acc_r(tot[" << 1 + d.first
                   << "]);\n";
        os << ind << "}\n";
    }

    // ---------------- convolution tables ----------------
    // T_c[k] = sum_m A_c[m] B_c[m + off - k] for k in [kmin, kmax].  One CTA covers KB consecutive k; a
    // thread owns KT consecutive k of one component over a contiguous slice of m (MS slices per k-tile),
    // keeping a sliding window of the resolution values in registers (KT FMAs per two shared loads).
    // The MS lane partials are combined with a compensated (two-sum) shuffle reduction.
    // Kernel header, or (body) the same code as a device function over a virtual block index, which the
    // one-launch evaluation kernel calls: blockIdx / gridDim stand for the function's arguments and the
    // record pointer for its shared-memory copy until endBody() closes it.
    void kernelHead(const std::string &name, const std::string &bounds, bool body, const std::string &extra = "") {
        if(!body) {
            os << "extern \"C\" __global__ void __launch_bounds__(" << bounds << ") " << name << "(const GfArgs a) {\n";
            return;
        }
        os << "#define blockIdx gf_bid\n#define gridDim gf_gdim\n#undef GF_PR\n#define GF_PR gf_pr\n";
        os << "__device__ __forceinline__ void " << name
           << "_body(const GfArgs &a, const uint3 gf_bid, const uint3 gf_gdim, const void *gf_pr" << extra << ") {\n";
    }
    void endBody(bool body) {
        if(body)
            os << "#undef blockIdx\n#undef gridDim\n#undef GF_PR\n#define GF_PR a.Pr\n";
    }

    // foldPartials: a folded grid sum leaves only its per-CTA partials (the one-launch kernel's CTAs sum
    // them after its barrier), without the completion counter and finishing CTA
    void convKernel(bool grad, bool body = false, bool foldPartials = false) {
        const char *sfx = grad ? "g" : "n";
        const int NC    = (int)T.convs.size();
        if(NC == 0)
            return;
        const ConvShape sh = convShape(grad);
        const int MS = sh.MS, KT = sh.KT, items = sh.items;
        auto &off       = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps       = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const int64_t total = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        size_t smem   = 0;
        int maxBlocks = 0;
        std::vector<int> KBs;
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            const int KB       = sh.KB[ci];
            KBs.push_back(KB);
            int mcomp = 1 + (grad ? (int)T.dep_val[cv.model].size() : 0);
            int rcomp = 1 + (grad ? (int)T.dep_val[cv.resol].size() : 0);
            size_t sm = (size_t)(mcomp * convStride(cv.nM) + rcomp * convStride(cv.nM + KB)) * (mixed ? 4 : 8);
            smem      = std::max(smem, sm);
            maxBlocks = std::max(maxBlocks, (cv.nK + KB - 1) / KB);
        }
        (grad ? plan.conv_smem_grad : plan.conv_smem_nograd) = smem;
        plan.conv_blocks = std::max(plan.conv_blocks, maxBlocks);

        if(grad && !body)
            for(int ci = 0; ci < NC; ++ci) {
                const int q = plan.conv_fold_q[ci];
                if(q < 0)
                    continue;
                // grid bins per table entry of the folded numeric node
                const ConvInfo &cv = T.convs[ci];
                const NumInfo &g   = T.nums[q];
                std::vector<int> cnt(cv.nK, 0);
                for(int lb = 0; lb < g.nbins[0]; ++lb) {
                    const int k = T.kgrid[g.kgrid_off[0] + lb];
                    if(k < cv.kmin || k > cv.kmax)
                        throw std::runtime_error("codegen: grid bin offset outside the convolution table");
                    ++cnt[k - cv.kmin];
                }
                os << "__device__ const int gf_kcount_" << ci << "[" << cv.nK << "] = {";
                for(int k = 0; k < cv.nK; ++k)
                    os << (k ? "," : "") << cnt[k];
                os << "};\n";
            }
        kernelHead(std::string("gf_conv_") + sfx, std::to_string(block), body);
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *sm = reinterpret_cast<R *>(smraw);\n";
        os << "  const int toy = blockIdx.y; const int ci = blockIdx.z; const int tid = threadIdx.x;\n";
        os << "  const int lane = tid & 31, wid = tid >> 5; (void)lane; (void)wid;\n";
        os << "  gf_pdl_trigger();\n";
        // launched after the grid kernel (which then needs no table), this kernel overlaps it and waits for
        // it only before it completes, so that the event kernel's wait on this one covers both
        os << "  if(a.active && !a.active[toy]) { gf_pdl_wait(); return; }\n";
        emitParamsR(os, T, plan.nl, "  ");
        os << "  R *ctab = reinterpret_cast<R *>(a.ctab) + (i64)toy * " << total << ";\n";
        os << "  switch(ci) {\n";
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            const int comps = convComps(ci, grad), KB = KBs[ci], ktiles = items / comps, cp = cps[ci];
            const auto &dm = T.dep_val[cv.model];
            const auto &dr = T.dep_val[cv.resol];
            const int mcomp = 1 + (grad ? (int)dm.size() : 0);
            const int W1    = cv.nM + KB; // window entries (one spare for the last shift)
            const int nMp = convStride(cv.nM), W1p = convStride(W1);
            os << "  case " << ci << ": {\n";
            os << "    const int k0 = " << cv.kmin << " + (int)blockIdx.x * " << KB << ";\n";
            os << "    if(k0 > " << cv.kmax << ") { gf_pdl_wait(); return; }\n";
            os << "    R *sM = sm; R *sR = sm + " << mcomp * nMp << ";\n";
            os << "    const int rbase = " << cv.offset << " - (k0 + " << KB - 1 << ");\n";
            // one pass of k-tiles per item: the lane that adds an item's entries to the folded grid sum (ms == 0)
            // loads their grid-bin counts into registers first, so that nothing waits for these loads before
            // the fold at the end
            const bool kcReg = plan.conv_fold_q[ci] >= 0 && sh.KP == 1;
            const bool kcPre = plan.conv_fold_q[ci] >= 0 && KB <= block && !kcReg;
            // kcReg: the counts are loaded after the support's barrier (below), because a barrier waits for the
            // warp's loads in flight (a DRAM miss after an L2 flush, ~1.3 us); the sums that follow have no
            // barrier and cover the load
            if(kcPre) {
                // the grid-bin count of one of this CTA's table entries per thread, loaded into a register now
                // and stored after the staging below, so that the load's latency overlaps the staging
                os << "    __shared__ R s_kc[" << KB << "];\n";
                // loaded as int by every thread at a clamped index (no predicate or select, which would stall the
                // warp on the load) and converted at the store after the staging
                os << "    const int kcv = gf_kcount_" << ci << "[min(k0 + min(tid, " << KB - 1 << "), " << cv.kmax << ") - "
                   << cv.kmin << "];\n";
            }
            const double wM = (cv.ic[1] - cv.ic[0]) / cv.nM, wR = (cv.ic[4] - cv.ic[3]) / cv.nR;
            // support of every staged array: the first and last index holding a nonzero value (products with
            // an exact zero factor add nothing, so each item sums only the m range where both factors can
            // be nonzero and splits that range over its lanes)
            const int NA = mcomp + 1 + (grad ? (int)dr.size() : 0);
            os << "    __shared__ int sup_lo[" << NA << "], sup_hi[" << NA << "];\n";
            os << "    if(tid < " << NA << ") { sup_lo[tid] = 1 << 30; sup_hi[tid] = -(1 << 30); }\n";
            os << "    int slo[" << NA << "], shi[" << NA << "];\n";
            os << "#pragma unroll\n    for(int c = 0; c < " << NA << "; ++c) { slo[c] = 1 << 30; shi[c] = -(1 << 30); }\n";
            for(int pass = 0; pass < 2; ++pass) {
                bool model = pass == 0;
                int sub    = model ? cv.model : cv.resol;
                const auto &dd = model ? dm : dr;
                int len        = model ? nMp : W1p; // array stride
                if(model)
                    os << "    for(int m = tid; m < " << cv.nM << "; m += " << block << ") {\n"
                       << "      const R wx = (R)GF_CENTRE(" << lit(cv.ic[0]) << ", " << lit(wM) << ", m);\n";
                else
                    os << "    for(int w = tid; w < " << W1 << "; w += " << block << ") {\n"
                       << "      const int r = rbase + w;\n"
                       << "      if(r < 0 || r >= " << cv.nR << ") {\n"
                       << "        for(int c = 0; c < " << 1 + (grad ? (int)dr.size() : 0) << "; ++c) sR[c * " << W1p
                       << " + w] = R(0);\n"
                       << "        continue;\n      }\n"
                       << "      const R wx = (R)GF_CENTRE(" << lit(cv.ic[3]) << ", " << lit(wR) << ", r);\n";
                std::ostringstream body;
                Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
                c.single = mixed;
                c.x   = [&](int) { return std::string("wx"); };
                c.k   = [&](int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.tab = [&](int, int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.uid = model ? 0 : 1000;
                Val v = emit(c, sub);
                std::string idx = model ? "m" : "w";
                auto store = [&](size_t slot, const std::string &expr) {
                    const int arr = model ? (int)slot : mcomp + (int)slot;
                    os << "      { const R sv = " << expr << "; " << (model ? "sM" : "sR") << "[" << slot * len
                       << " + " << idx << "] = sv; if(sv != R(0)) { slo[" << arr << "] = min(slo[" << arr << "], "
                       << idx << "); shi[" << arr << "] = max(shi[" << arr << "], " << idx << "); } }\n";
                };
                os << "      {\n" << body.str();
                store(0, v.v);
                if(grad)
                    for(size_t j = 0; j < dd.size(); ++j) {
                        auto it = v.g.find(dd[j]);
                        store(1 + j, it == v.g.end() ? std::string("R(0)") : it->second);
                    }
                os << "      }\n    }\n";
            }
            if(kcPre)
                os << "    if(tid < " << KB << ") s_kc[tid] = (R)kcv;\n";
            os << "    __syncthreads();\n";
            os << "#pragma unroll\n    for(int c = 0; c < " << NA << "; ++c) {\n";
            os << "      const int lo = __reduce_min_sync(0xffffffffu, slo[c]), hi = __reduce_max_sync(0xffffffffu, "
                  "shi[c]);\n";
            os << "      if(lane == 0) { atomicMin(&sup_lo[c], lo); atomicMax(&sup_hi[c], hi); }\n";
            os << "    }\n";
            os << "    __syncthreads();\n";
            const int fq = plan.conv_fold_q[ci];
            if(kcReg) {
                // every lane loads its item's counts at a clamped (valid) index, without a predicate or a select,
                // and keeps them as ints: nothing consumes them before the fold, which reads them only for
                // entries that exist
                os << "    int kcr[" << KT << "];\n    {\n";
                os << "      const int kt0_ = k0 + min((tid / " << MS << ") / " << comps << ", " << ktiles - 1 << ") * " << KT
                   << ";\n";
                os << "#pragma unroll\n      for(int j = 0; j < " << KT << "; ++j)\n";
                os << "        kcr[j] = gf_kcount_" << ci << "[min(kt0_ + j, " << cv.kmax << ") - " << cv.kmin << "];\n    }\n";
            }
            os << "    const int ms = tid % " << MS << ", item = tid / " << MS << ", comp = item % " << comps
               << ", ktb = item / " << comps << ";\n";
            os << "    const bool live = ktb < " << ktiles << ";\n";
            if(fq >= 0)
                os << "    ACC fs = acc_zero();\n";
            os << "    for(int kp = 0; kp < " << sh.KP << "; ++kp) {\n";
            os << "    const int kt = ktb + kp * " << ktiles << ";\n";
            os << "    const int kt0 = k0 + kt * " << KT << ";\n";
            os << "    const int c0 = " << KB - 1 << " - kt * " << KT << ";\n";
            os << "    R acc[" << KT << "], cmp[" << KT << "];\n#pragma unroll\n    for(int j = 0; j < " << KT
               << "; ++j) { acc[j] = R(0); cmp[j] = R(0); }\n";
            os << "    if(live) {\n";
            os << "      const R *mA[2] = {nullptr, nullptr}; const R *rA[2] = {nullptr, nullptr};\n";
            os << "      int ma[2] = {0, 0}, ra[2] = {" << mcomp << ", " << mcomp << "};\n";
            os << "      switch(comp) {\n";
            os << "      case 0: mA[0] = sM; rA[0] = sR; break;\n";
            if(grad)
                for(size_t j = 0; j < cv.dep.size(); ++j) {
                    int sl  = cv.dep[j];
                    auto im = std::find(dm.begin(), dm.end(), sl);
                    auto ir = std::find(dr.begin(), dr.end(), sl);
                    os << "      case " << 1 + j << ": ";
                    int t = 0;
                    if(im != dm.end()) {
                        os << "mA[" << t << "] = sM + " << (1 + (im - dm.begin())) * nMp << "; rA[" << t
                           << "] = sR; ma[" << t << "] = " << 1 + (im - dm.begin()) << "; ";
                        ++t;
                    }
                    if(ir != dr.end()) {
                        os << "mA[" << t << "] = sM; rA[" << t << "] = sR + " << (1 + (ir - dr.begin())) * W1p
                           << "; ra[" << t << "] = " << mcomp + 1 + (ir - dr.begin()) << "; ";
                        ++t;
                    }
                    os << "break;\n";
                }
            os << "      default: break;\n      }\n";
            os << "      for(int t = 0; t < 2; ++t) {\n";
            os << "        if(!mA[t]) break;\n";
            os << "        const R *M = mA[t]; const R *Rw = rA[t] + c0;\n";
            // m with M[m] != 0 and R[c0 + m - j] != 0 for some j of the tile, split evenly over the lanes
            os << "        const int s = max(max(sup_lo[ma[t]], sup_lo[ra[t]] - c0), 0);\n";
            os << "        const int e = min(min(sup_hi[ma[t]] + 1, sup_hi[ra[t]] - c0 + " << KT << "), " << cv.nM
               << ");\n";
            os << "        if(e <= s) continue;\n";
            // batches (8 lanes of long slices): blocks of 16 m, FP32 loads 16 bytes wide, lane slices
            // starting at multiples of 4 (extending the range down to s & ~3 only adds products with a zero
            // factor); one toy (32 lanes of short slices): blocks of 8 m, an even split
            const int BM = batch ? 16 : 8;
            const bool vec = batch && mixed;
            if(vec) {
                os << "        const int s4 = s & ~3, L = ((((e - s4 + " << MS - 1 << ") / " << MS << ") + 3) & ~7) + 4;\n";
                os << "        const int mlo = min(s4 + ms * L, e), mhi = min(mlo + L, e);\n";
            } else
                os << "        const int mlo = s + ((e - s) * ms) / " << MS << ", mhi = s + ((e - s) * (ms + 1)) / " << MS
                   << ";\n";
            os << "        R rv[" << KT << "];\n#pragma unroll\n        for(int j = 0; j < " << KT
               << "; ++j) rv[j] = Rw[mlo - j];\n";
            // blocks of BM products are summed plainly, blocks are added with a two-sum correction (mixed);
            // full blocks fully unrolled (the window shifts become register renames; batches in FP32: M and
            // the window read as float4, M + mb and Rw + mb + 1 being 16-byte aligned), the last partial
            // block stepwise; the same products in the same order either way
            os << "        for(int mb = mlo; mb < mhi; mb += " << BM << ") {\n";
            os << "          R bs[" << KT << "];\n#pragma unroll\n          for(int j = 0; j < " << KT << "; ++j) bs[j] = R(0);\n";
            os << "          if(mb + " << BM << " <= mhi) {\n";
            if(vec) {
                os << "            const float4 *M4 = reinterpret_cast<const float4 *>(M + mb);\n";
                os << "            const float4 *R4 = reinterpret_cast<const float4 *>(Rw + mb + 1);\n";
                os << "#pragma unroll\n            for(int q = 0; q < 4; ++q) {\n";
                os << "              const float4 mq = M4[q], rq = R4[q];\n";
                os << "              const float mvs[4] = {mq.x, mq.y, mq.z, mq.w}, rvs[4] = {rq.x, rq.y, rq.z, rq.w};\n";
                os << "#pragma unroll\n              for(int u = 0; u < 4; ++u) {\n";
                os << "                const R mv = mvs[u];\n";
                os << "#pragma unroll\n                for(int j = 0; j < " << KT << "; ++j) bs[j] = fma(mv, rv[j], bs[j]);\n";
                os << "#pragma unroll\n                for(int j = " << KT - 1 << "; j > 0; --j) rv[j] = rv[j - 1];\n";
                os << "                rv[0] = rvs[u];\n";
                os << "              }\n";
                os << "            }\n";
            } else {
                os << "#pragma unroll\n            for(int u = 0; u < " << BM << "; ++u) {\n";
                os << "              const R mv = M[mb + u];\n";
                os << "#pragma unroll\n              for(int j = 0; j < " << KT << "; ++j) bs[j] = fma(mv, rv[j], bs[j]);\n";
                os << "#pragma unroll\n              for(int j = " << KT - 1 << "; j > 0; --j) rv[j] = rv[j - 1];\n";
                os << "              rv[0] = Rw[mb + u + 1];\n";
                os << "            }\n";
            }
            os << "          } else {\n";
            os << "            for(int m = mb; m < mhi; ++m) {\n";
            os << "              const R mv = M[m];\n";
            os << "#pragma unroll\n              for(int j = 0; j < " << KT << "; ++j) bs[j] = fma(mv, rv[j], bs[j]);\n";
            os << "#pragma unroll\n              for(int j = " << KT - 1 << "; j > 0; --j) rv[j] = rv[j - 1];\n";
            os << "              rv[0] = Rw[m + 1];\n";
            os << "            }\n";
            os << "          }\n";
            os << "#pragma unroll\n          for(int j = 0; j < " << KT << "; ++j) gf_comp_add(acc[j], cmp[j], bs[j]);\n";
            os << "        }\n      }\n    }\n";
            // mixed precision: the lanes' compensated sums reduced as pairs; conv 0's values keep the pair's low
            // part (one toy), so that a value enters the per-bin terms and the folded grid sum unrounded
            const int64_t loOff = ci == 0 ? (grad ? plan.ctab_lo_off_grad : plan.ctab_lo_off_nograd) : -1;
            if(mixed) {
                os << "#pragma unroll\n    for(int j = 0; j < " << KT << "; ++j) {\n";
                os << "      const ACC tp = gf_group_sum2(acc[j], cmp[j], " << MS << ");\n";
                os << "      const R t = tp.x;\n";
            } else {
                os << "#pragma unroll\n    for(int j = 0; j < " << KT << "; ++j) acc[j] += cmp[j];\n";
                os << "#pragma unroll\n    for(int j = 0; j < " << KT << "; ++j) {\n";
                os << "      const R t = gf_group_sum(acc[j], " << MS << ");\n";
            }
            os << "      const int k = kt0 + j;\n";
            const std::string loStore = loOff >= 0 ? "        if(comp == 0) ctab[" + std::to_string(loOff) + " + (k - " +
                                                         std::to_string(cv.kmin) + ")] = tp.y;\n"
                                                   : "";
            if(fq < 0) {
                os << "      if(live && ms == 0 && k <= " << cv.kmax << ") {\n";
                os << "        ctab[" << off[ci] << " + (k - " << cv.kmin << ") * " << cp << " + comp] = t;\n" << loStore;
                os << "      }\n";
            } else {
                os << "      if(live && ms == 0 && k <= " << cv.kmax << ") {\n";
                os << "        ctab[" << off[ci] << " + (k - " << cv.kmin << ") * " << cp << " + comp] = t;\n" << loStore;
                const std::string kc = kcReg   ? "(R)kcr[j]"
                                       : kcPre ? "s_kc[k - k0]"
                                               : "(R)gf_kcount_" + std::to_string(ci) + "[k - " + std::to_string(cv.kmin) + "]";
                if(mixed)
                    os << "        { ACC pr = gf_two_prod(" << kc << ", t); pr.y = fmaf(" << kc << ", tp.y, pr.y); fs = acc_add(fs, pr); }\n";
                else
                    os << "        fs = acc_add(fs, gf_two_prod(" << kc << ", t));\n";
                os << "      }\n";
            }
            os << "    }\n";
            os << "    }\n"; // kp
            if(fq >= 0)
                emitConvFold(ci, fq, grad, comps, ktiles, MS, KB, foldPartials);
            os << "    break; }\n";
        }
        os << "  }\n";
        os << "  gf_pdl_wait();\n";
        os << "}\n\n";
        endBody(body);
    }

    // The folded grid sum of numeric node q in the conv kernel: the CTA's sums of n_k T_comp[k] into the
    // grid partials (component slot: 0 value, 1 + gradient slot), then the last CTA of (toy, q) sums the
    // partials and finishes the node's normalisation.
    void emitConvFold(int ci, int q, bool grad, int comps, int ktiles, int MS, int KB, bool partialsOnly = false) {
        const ConvInfo &cv = T.convs[ci];
        const int NQ = (int)T.nums.size(), NGs = 1 + T.NG, NGp = 1 + (grad ? T.NG : 0), NW = block / 32;
        const int MGB = plan.max_grid_blocks, nblk = (cv.nK + KB - 1) / KB;
        os << "    {\n";
        os << "      const int cs[" << comps << "] = {0";
        for(int j = 1; j < comps; ++j)
            os << ", " << 1 + cv.dep[j - 1];
        os << "};\n";
        os << "      __shared__ ACC fsh[" << (block / MS) << "];\n";
        os << "      __shared__ ACC tot[" << NGp << "];\n";
        os << "      __shared__ int flast;\n";
        os << "      if(ms == 0) fsh[item] = fs;\n";
        os << "      __syncthreads();\n";
        os << "      ACC *gp = reinterpret_cast<ACC *>(a.gpartial) + ((i64)toy * " << NQ << " + " << q << ") * " << NGs
           << " * " << MGB << ";\n";
        os << "      if(tid < " << comps << ") { ACC t = acc_zero(); for(int kk = 0; kk < " << ktiles
           << "; ++kk) t = acc_add(t, fsh[kk * " << comps << " + tid]); gp[(i64)cs[tid] * " << MGB
           << " + blockIdx.x] = t; }\n";
        if(partialsOnly) {
            os << "    }\n";
            return;
        }
        os << "      __threadfence();\n      __syncthreads();\n";
        os << "      if(tid == 0) { unsigned prev = atomicAdd(&a.gcounter[toy * " << NQ << " + " << q
           << "], 1u); flast = (prev == " << nblk - 1 << "u); }\n";
        os << "      __syncthreads();\n";
        os << "      if(flast) {\n";
        os << "        __threadfence();\n";
        os << "        for(int cc = wid; cc < " << comps << "; cc += " << NW << ") {\n";
        os << "          const ACC *pc = gp + (i64)cs[cc] * " << MGB << ";\n";
        os << "          ACC t = acc_zero();\n";
        os << "          for(int bi = lane; bi < " << nblk << "; bi += 32) t = acc_add(t, pc[bi]);\n";
        os << "          t = warp_acc2(t);\n";
        os << "          if(lane == 0) tot[cs[cc]] = t;\n";
        os << "        }\n";
        os << "        __syncthreads();\n";
        os << "        if(tid == 0) {\n";
        os << "          a.gcounter[toy * " << NQ << " + " << q << "] = 0u;\n";
        emitNumFinish(q, grad, "          ");
        os << "        }\n";
        os << "      }\n";
        os << "    }\n";
    }

    // ---------------- numeric grids ----------------
    // One CTA row per numeric node; the finishing CTA of a (toy, node) turns the grid sum into the node's
    // normalisation factor and its derivatives (GooPdf::normalize numeric branch,
    // src/PDFs/GooPdf.cu:366-395) and stores them for the event pass.
    void gridKernel(bool grad, bool body = false) {
        const char *sfx = grad ? "g" : "n";
        const int NQ    = (int)T.nums.size();
        if(NQ == 0)
            return;
        const int NGp = 1 + (grad ? T.NG : 0); // components reduced
        const int NGs = 1 + T.NG;              // buffer stride
        const int BPB = plan.grid_bins_per_block;
        const int NW  = block / 32;
        const int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        auto &off               = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps               = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const NormLayout &nl    = plan.nl;
        kernelHead(std::string("gf_grid_") + sfx, std::to_string(block), body);
        os << "  const int toy = blockIdx.y; const int q = blockIdx.z; const int tid = threadIdx.x;\n";
        os << "  const int lane = tid & 31, wid = tid >> 5;\n";
        os << "  gf_pdl_trigger();\n";
        os << "  gf_pdl_wait();\n";
        os << "  if(a.active && !a.active[toy]) return;\n";
        emitParamsR(os, T, nl, "  ");
        os << "  const R *ctab = reinterpret_cast<const R *>(a.ctab) + (i64)toy * " << ctabTotal << ";\n";
        os << "  (void)ctab;\n";
        os << "  R av = R(0);\n";
        for(int s = 0; s < NGp - 1; ++s)
            os << "  R ag" << s << " = R(0);\n";
        os << "  int nblk = 0;\n";
        os << "  switch(q) {\n";
        for(int q = 0; q < NQ; ++q) {
            const NumInfo &g = T.nums[q];
            if(plan.num_folded[q]) {
                os << "  case " << q << ": return; // folded into the convolution table kernel\n";
                continue;
            }
            os << "  case " << q << ": {\n";
            os << "    nblk = " << plan.grid_blocks[q] << ";\n";
            os << "    if((int)blockIdx.x >= nblk) return;\n";
            os << "    const i64 bend = min((i64)" << g.total << "LL, (i64)(blockIdx.x + 1) * " << BPB << ");\n";
            os << "#pragma unroll 4\n    for(i64 b = (i64)blockIdx.x * " << BPB << " + tid; b < bend; b += " << block << ") {\n";
            os << "      i64 bb = b;\n";
            for(size_t ax = 0; ax < g.obs.size(); ++ax) {
                const gf_observable &o = T.obs[g.obs[ax]];
                double w               = (o.hi - o.lo) / g.nbins[ax];
                os << "      const int lb" << ax << " = (int)(bb % " << g.nbins[ax] << "); bb /= " << g.nbins[ax]
                   << ";\n";
                os << "      const R gx" << g.obs[ax] << " = (R)GF_CENTRE(" << lit(o.lo) << ", " << lit(w) << ", lb"
                   << ax << ");\n";
            }
            std::ostringstream body;
            Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
            c.single = mixed;
            c.x = [&](int o) { return "gx" + std::to_string(o); };
            c.k = [&](int ci) -> std::string {
                for(size_t j = 0; j < g.convs.size(); ++j)
                    if(g.convs[j] == ci)
                        return "a.kgrid[" + std::to_string(g.kgrid_off[j]) + " + lb" + std::to_string(g.conv_axis[j]) +
                               "]";
                throw std::runtime_error("codegen: conv without grid k");
            };
            c.tab = [&](int ci, int comp) {
                const ConvInfo &cv = T.convs[ci];
                return "ctab[" + std::to_string(off[ci]) + " + (" + c.k(ci) + " - " + std::to_string(cv.kmin) + ") * " +
                       std::to_string(cps[ci]) + " + " + std::to_string(comp) + "]";
            };
            Val v = emit(c, g.node);
            os << "      {\n" << body.str();
            os << "      av += " << v.v << ";\n";
            if(grad)
                for(auto &kv : v.g)
                    os << "      ag" << kv.first << " += " << kv.second << ";\n";
            os << "      }\n";
            os << "    }\n";
            os << "    break; }\n";
        }
        os << "  default: return;\n  }\n";
        os << "  __shared__ ACC red[" << NW << "][" << NGp << "];\n";
        os << "  __shared__ ACC tot[" << NGp << "];\n";
        os << "  __shared__ int last;\n";
        {
            std::vector<std::string> comps{"acc_of(av)"};
            for(int s = 0; s < NGp - 1; ++s)
                comps.push_back("acc_of(ag" + std::to_string(s) + ")");
            emitCtaReduce(os, comps, "  ");
        }
        // a node covered by one CTA finishes from the CTA's sums (no partials, fence or counter)
        os << "  if(nblk == 1) {\n";
        os << "    __shared__ ACC tot1[" << NGp << "];\n";
        os << "    if(tid < " << NGp << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
           << "; ++w) t = acc_add(t, red[w][tid]); tot1[tid] = t; }\n";
        os << "    __syncthreads();\n";
        os << "    if(tid == 0) {\n";
        os << "      const ACC *tot = tot1;\n";
        os << "      switch(q) {\n";
        for(int q = 0; q < NQ; ++q) {
            if(plan.num_folded[q] || plan.grid_blocks[q] != 1)
                continue;
            os << "      case " << q << ":\n";
            emitNumFinish(q, grad, "        ");
            os << "        break;\n";
        }
        os << "      default: break;\n";
        os << "      }\n    }\n    return;\n  }\n";
        // block partials are component-major: gpartial[toy][q][comp][block]
        os << "  ACC *gp = reinterpret_cast<ACC *>(a.gpartial) + ((i64)toy * " << NQ << " + q) * " << NGs << " * "
           << plan.max_grid_blocks << ";\n";
        os << "  if(tid < " << NGp << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
           << "; ++w) t = acc_add(t, red[w][tid]); gp[(i64)tid * " << plan.max_grid_blocks << " + blockIdx.x] = t; }\n";
        os << "  __threadfence();\n  __syncthreads();\n";
        os << "  if(tid == 0) { unsigned prev = atomicAdd(&a.gcounter[toy * " << NQ
           << " + q], 1u); last = (prev == (unsigned)(nblk - 1)); }\n";
        os << "  __syncthreads();\n";
        os << "  if(!last) return;\n";
        os << "  __threadfence();\n";
        // one warp per component: contiguous loads of that component's block partials, then a warp reduction
        os << "  for(int comp = wid; comp < " << NGp << "; comp += " << NW << ") {\n";
        os << "    const ACC *pc = gp + (i64)comp * " << plan.max_grid_blocks << ";\n";
        os << "    ACC t = acc_zero();\n";
        os << "#pragma unroll 4\n    for(int bi = lane; bi < nblk; bi += 32) t = acc_add(t, pc[bi]);\n";
        os << "    t = warp_acc2(t);\n";
        os << "    if(lane == 0) tot[comp] = t;\n";
        os << "  }\n";
        os << "  __syncthreads();\n";
        os << "  if(tid == 0) {\n";
        os << "    a.gcounter[toy * " << NQ << " + q] = 0u;\n";
        os << "    switch(q) {\n";
        for(int q = 0; q < NQ; ++q) {
            if(plan.num_folded[q])
                continue;
            os << "    case " << q << ":\n";
            emitNumFinish(q, grad, "      ");
            os << "      break;\n";
        }
        os << "    default: break;\n";
        os << "    }\n  }\n}\n\n";
        endBody(body);
    }

    // ---------------- Amp3Body amplitude caches and integrals ----------------
    // Rebuilt only for toys flagged in a.dirty (the resonance or efficiency parameters changed), as
    // Amp3Body::normalize does with its per-resonance redoIntegral flags
    // (src/PDFs/physics/Amp3Body.cu:263-330).
    //   gf_amp   B_r(event) for every resonance into the R2 columns, zero outside the kinematic boundary
    //            (SpecialResonanceCalculator, src/PDFs/physics/detail/SpecialResonanceCalculator.cu:12-45)
    //   gf_gram  I_ij = sum over in-Dalitz bins of B_i conj(B_j) eff, i <= j, per-CTA FP64 partials
    //            (SpecialResonanceIntegrator, src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:7-121)
    std::string resCall(const Amp3Info &A, int r, const char *m12, const char *m13, const char *m23) {
        const TNode &rn = T.nodes[A.res[r]];
        if(rn.op == GF_OP_RES_NONRES)
            return mixed ? "make_float2(1.0f, 0.0f)" : "make_double2(1.0, 0.0)";
        const int I = (rn.consts.size() > 3 && rn.consts[3] != 0) ? 2 : 1;
        std::ostringstream o;
        o << "gf_rbw<" << I << ">(" << m12 << ", " << m13 << ", " << m23 << ", P[" << rn.params[0] << "], P["
          << rn.params[1] << "], " << (int)rn.consts[0] << ", " << (int)rn.consts[1] << ", "
          << (rn.consts[2] != 0 ? "true" : "false") << ", " << lit(A.M) << ", " << lit(A.m1) << ", " << lit(A.m2)
          << ", " << lit(A.m3) << ", " << lit(A.r) << ", " << lit(A.rm) << ")";
        return o.str();
    }
    std::string dalitzArgs(const Amp3Info &A) {
        return lit(A.M) + ", " + lit(A.m1) + ", " + lit(A.m2) + ", " + lit(A.m3);
    }

    // ---- amplitude nodes: values and derivative columns at one point ----
    int nDeriv(int k) const {
        int n = 0;
        for(auto &t : T.amp_theta(k))
            n += (int)t.amps.size();
        return n;
    }
    bool thetaParam(int k, int p) const {
        for(auto &t : T.amp_theta(k))
            if(t.param == p)
                return true;
        return false;
    }
    // d(component)/d(theta t) from the partials with respect to the component's mass (pm) and width (pw)
    std::string dPart(int t_param, int mass_p, int width_p, const std::string &dm, const std::string &dw,
                      const std::string &mk = "make_double2") {
        std::string e;
        if(mass_p == t_param)
            e = dm;
        if(width_p == t_param)
            e = e.empty() ? dw : mk + "(" + e + ".x + " + dw + ".x, " + e + ".y + " + dw + ".y)";
        return e;
    }

    // __device__ gf_ampv_<k>(point, P, A, dA): the amplitudes of amplitude node k (unified numbering) at one
    // point and, for every floated resonance / line-shape parameter t, dA_a/dt of the amplitudes depending on
    // it (in AmpTheta order).  Amp3Body: SpecialResonanceCalculator (zero outside the kinematic boundary);
    // Amp4Body: the line shapes and spin factors once, then AmpCalc's sum over permutations
    // (src/PDFs/physics/detail/AmpCalc.cu:29-56) and its derivatives by the product rule.
    void ampFunction(int k) {
        const int n3 = (int)T.amp3s.size();
        const auto &theta = T.amp_theta(k);
        const int ND = std::max(1, nDeriv(k));
        std::vector<int> toff;
        for(int t = 0, o = 0; t < (int)theta.size(); ++t) {
            toff.push_back(o);
            o += (int)theta[t].amps.size();
        }
        if(k < n3) {
            const Amp3Info &A = T.amp3s[k];
            os << "__device__ void gf_ampv_" << k << "(double m12, double m13, const double *P, R2 *A, R2 *dA) {\n";
            os << "  for(int q = 0; q < " << A.nRes << "; ++q) { A[q].x = R(0); A[q].y = R(0); }\n";
            os << "  for(int q = 0; q < " << ND << "; ++q) { dA[q].x = R(0); dA[q].y = R(0); }\n";
            os << "  if(!gf_in_dalitz(m12, m13, " << dalitzArgs(A) << ")) return;\n";
            os << "  const double m23 = gf_m23(m12, m13, " << dalitzArgs(A) << ");\n";
            for(int r = 0; r < A.nRes; ++r) {
                const TNode &rn = T.nodes[A.res[r]];
                const bool dep = rn.op == GF_OP_RES_RBW && (thetaParam(k, rn.params[0]) || thetaParam(k, rn.params[1]));
                if(!dep) {
                    os << "  A[" << r << "] = " << resCall(A, r, "m12", "m13", "m23") << ";\n";
                    continue;
                }
                const int I = (rn.consts.size() > 3 && rn.consts[3] != 0) ? 2 : 1;
                os << "  { GfDual re, im;\n";
                os << "    gf_rbw_t<" << I << ", GfDual>(m12, m13, m23, GfDual(P[" << rn.params[0] << "], 1.0, 0.0), GfDual(P["
                   << rn.params[1] << "], 0.0, 1.0), " << (int)rn.consts[0] << ", " << (int)rn.consts[1] << ", "
                   << (rn.consts[2] != 0 ? "true" : "false") << ", " << lit(A.M) << ", " << lit(A.m1) << ", " << lit(A.m2)
                   << ", " << lit(A.m3) << ", " << lit(A.r) << ", " << lit(A.rm) << ", re, im);\n";
                os << "    A[" << r << "].x = (R)re.v; A[" << r << "].y = (R)im.v;\n";
                os << "    const double2 dm = make_double2(re.a, im.a), dw = make_double2(re.b, im.b); (void)dm; (void)dw;\n";
                for(int t = 0; t < (int)theta.size(); ++t) {
                    auto it = std::find(theta[t].amps.begin(), theta[t].amps.end(), r);
                    if(it == theta[t].amps.end())
                        continue;
                    std::string e = dPart(theta[t].param, rn.params[0], rn.params[1], "dm", "dw");
                    const int idx = toff[t] + (int)(it - theta[t].amps.begin());
                    os << "    { const double2 d = " << e << "; dA[" << idx << "].x = (R)d.x; dA[" << idx
                       << "].y = (R)d.y; }\n";
                }
                os << "  }\n";
            }
            os << "}\n\n";
            return;
        }
        const Amp4Info &A = T.amp4s[k - n3];
        const double m1 = A.m[0], m2 = A.m[1], m3 = A.m[2], m4 = A.m[3];
        // mixed precision: FP64 kinematic inversion and pair masses, FP32 spin factors, line shapes and
        // products; FP64 engine: FP64 throughout
        const std::string C2 = mixed ? "float2" : "double2", MK = mixed ? "make_float2" : "make_double2";
        const std::string F = mixed ? "float" : "double";
        os << "__device__ void gf_ampv_" << k
           << "(double m12, double m34, double c12, double c34, double phi, const double *P, R2 *A, R2 *dA) {\n";
        os << "  for(int q = 0; q < " << ND << "; ++q) { dA[q].x = R(0); dA[q].y = R(0); }\n";
        // the mixed engine inverts the kinematics in FP32 unless a line shape's derivative column (dual
        // numbers, FP64) needs the FP64 pair masses
        bool anyDep = false;
        for(size_t u = 0; u < A.ls.size(); ++u) {
            const TNode &L = T.nodes[A.ls[u]];
            anyDep |= thetaParam(k, L.params[0]) || thetaParam(k, L.params[1]);
        }
        (void)anyDep;
        const bool kin32 = mixed; // floated line shapes: single-precision duals over the FP32 pair masses
        if(kin32) {
            os << "  GfLVf W[4];\n";
            os << "  gf_get4vecs_f(W, (float)m12, (float)m34, (float)c12, (float)c34, (float)phi, (float)" << lit(A.M)
               << ", (float)" << lit(m1) << ", (float)" << lit(m2) << ", (float)" << lit(m3) << ", (float)" << lit(m4)
               << ");\n";
            os << "  float d1f, d2f; (void)d1f; (void)d2f;\n";
        } else {
            os << "  GfLV V[4];\n";
            os << "  gf_get4vecs(V, m12, m34, c12, c34, phi, " << lit(A.M) << ", " << lit(m1) << ", " << lit(m2) << ", "
               << lit(m3) << ", " << lit(m4) << ");\n";
            if(mixed)
                os << "  const GfLVf W[4] = {lvf(V[0]), lvf(V[1]), lvf(V[2]), lvf(V[3])};\n";
        }
        const char *vv = mixed ? "W" : "V";
        os << "  double d1, d2, mp; (void)d1; (void)d2; (void)mp;\n";
        std::vector<int> lsDep(A.ls.size(), 0);
        for(size_t u = 0; u < A.ls.size(); ++u) {
            const TNode &L = T.nodes[A.ls[u]];
            const int pair = (int)L.consts[0];
            if(pair < 2)
                os << "  mp = " << (pair == 0 ? "m12" : "m34") << "; d1 = " << lit(pair == 0 ? m1 : m3) << "; d2 = "
                   << lit(pair == 0 ? m2 : m4) << ";\n";
            else if(kin32)
                os << "  mp = gf_pairmass_f(" << pair << ", W, (float)" << lit(m1) << ", (float)" << lit(m2) << ", (float)"
                   << lit(m3) << ", (float)" << lit(m4) << ", d1f, d2f); d1 = d1f; d2 = d2f;\n";  // exact widening
            else
                os << "  mp = gf_pairmass(" << pair << ", V, " << lit(m1) << ", " << lit(m2) << ", " << lit(m3) << ", "
                   << lit(m4) << ", d1, d2);\n";
            lsDep[u] = thetaParam(k, L.params[0]) || thetaParam(k, L.params[1]);
            const std::string sbw = L.op == GF_OP_LS_SBW ? "true" : "false";
            if(!lsDep[u]) {
                if(mixed)
                    os << "  const float2 L" << u << " = gf_lineshape_f(" << sbw << ", (float)mp, (float)d1, (float)d2, (float)P["
                       << L.params[0] << "], (float)P[" << L.params[1] << "], " << (int)L.consts[1] << ", "
                       << (int)L.consts[2] << ", (float)" << lit(L.consts[3]) << ");\n";
                else
                    os << "  const double2 L" << u << " = gf_lineshape(" << sbw << ", mp, d1, d2, P[" << L.params[0]
                       << "], P[" << L.params[1] << "], " << (int)L.consts[1] << ", " << (int)L.consts[2] << ", "
                       << lit(L.consts[3]) << ");\n";
            } else {
                // value and derivatives from the dual-number line shape (single precision in the mixed engine)
                const char *DT = mixed ? "GfDualF" : "GfDual";
                const std::string one = mixed ? "1.f, 0.f" : "1.0, 0.0", two = mixed ? "0.f, 1.f" : "0.0, 1.0";
                const std::string cv0 = mixed ? "(float)" : "";
                os << "  " << C2 << " L" << u << ", Lm" << u << ", Lw" << u << ";\n";
                os << "  { " << DT << " re, im;\n";
                os << "    gf_lineshape_t<" << DT << ">(" << sbw << ", mp, d1, d2, " << DT << "(" << cv0 << "P[" << L.params[0]
                   << "], " << one << "), " << DT << "(" << cv0 << "P[" << L.params[1] << "], " << two << "), "
                   << (int)L.consts[1] << ", " << (int)L.consts[2] << ", " << lit(L.consts[3]) << ", re, im);\n";
                os << "    L" << u << " = " << MK << "(re.v, im.v); Lm" << u << " = " << MK << "(re.a, im.a); Lw" << u
                   << " = " << MK << "(re.b, im.b); }\n";
            }
        }
        for(size_t u = 0; u < A.sf.size(); ++u) {
            const TNode &S = T.nodes[A.sf[u]];
            os << "  const " << F << " S" << u << " = " << (mixed ? "gf_spinfactor_f(" : "gf_spinfactor(")
               << (int)S.consts[0] << ", " << (mixed ? "(float)" : "") << lit(S.consts[1]) << ", " << vv << "["
               << (int)S.consts[2] << "], " << vv << "[" << (int)S.consts[3] << "], " << vv << "[" << (int)S.consts[4]
               << "], " << vv << "[" << (int)S.consts[5] << "]);\n";
        }
        // product of one permutation's factors, with factor `skip` (a line-shape position) replaced by `repl`
        auto product = [&](const Amp4Info::Amp &am, int p, int skip, const std::string &repl) {
            const int ls_step = (int)am.ls.size() / am.nPerm, sf_step = (int)am.sf.size() / am.nPerm;
            std::ostringstream o;
            o << "    { " << C2 << " r = " << MK << "(1.0, 0.0);\n";
            for(int j = p * ls_step; j < (p + 1) * ls_step; ++j)
                o << "      r = cmul(r, " << (j == skip ? repl : "L" + std::to_string(am.ls[j])) << ");\n";
            for(int j = p * sf_step; j < (p + 1) * sf_step; ++j)
                o << "      r.x *= S" << am.sf[j] << "; r.y *= S" << am.sf[j] << ";\n";
            o << "      r2.x += r.x; r2.y += r.y; }\n";
            return o.str();
        };
        auto norm = [&](int nPerm) {
            // 1 / sqrt(nPerm): evaluated in FP64 (FP64 engine, as the reference) or as an FP32 literal
            if(!mixed)
                return std::string("    const double f = 1 / sqrt((double)") + std::to_string(nPerm) + ");\n";
            return std::string("    const float f = (float)") + lit(1.0 / std::sqrt((double)nPerm)) + ";\n";
        };
        for(int a = 0; a < A.nAmp; ++a) {
            const Amp4Info::Amp &am = A.amps[a];
            os << "  {\n    " << C2 << " r2 = " << MK << "(0.0, 0.0);\n";
            for(int p = 0; p < am.nPerm; ++p)
                os << product(am, p, -1, "");
            os << norm(am.nPerm);
            os << "    A[" << a << "].x = (R)(r2.x * f); A[" << a << "].y = (R)(r2.y * f);\n  }\n";
        }
        for(int t = 0; t < (int)theta.size(); ++t)
            for(size_t j = 0; j < theta[t].amps.size(); ++j) {
                const int a = theta[t].amps[j];
                const Amp4Info::Amp &am = A.amps[a];
                const int ls_step = (int)am.ls.size() / am.nPerm;
                os << "  {\n    " << C2 << " r2 = " << MK << "(0.0, 0.0);\n";
                for(int p = 0; p < am.nPerm; ++p)
                    for(int pos = p * ls_step; pos < (p + 1) * ls_step; ++pos) {
                        const int u = am.ls[pos];
                        if(!lsDep[u])
                            continue;
                        const TNode &L = T.nodes[A.ls[u]];
                        std::string d = dPart(theta[t].param, L.params[0], L.params[1], "Lm" + std::to_string(u),
                                              "Lw" + std::to_string(u), MK);
                        if(d.empty())
                            continue;
                        os << product(am, p, pos, d);
                    }
                os << norm(am.nPerm);
                const int idx = toff[t] + (int)j;
                os << "    dA[" << idx << "].x = (R)(r2.x * f); dA[" << idx << "].y = (R)(r2.y * f);\n  }\n";
            }
        os << "}\n\n";
    }

    // Entries of the normalisation reduction of amplitude node k: the pairs i <= j of the Gram matrix
    // I_ij = sum_p A_i conj(A_j) e_p, then for every floated parameter t and dependent amplitude a the row
    // H_t,ab = sum_p dA_a/dt conj(A_b) e_p (e_p the efficiency at an Amp3Body bin, 1 for Amp4Body).
    struct Entry {
        bool h;
        int i, j; // value columns (pairs) or derivative index (i) and value column (j)
    };
    std::vector<Entry> entries(int k) {
        std::vector<Entry> e;
        const int n = T.amp_count(k);
        for(int i = 0; i < n; ++i)
            for(int j = i; j < n; ++j)
                e.push_back({false, i, j});
        int d = 0;
        for(auto &t : T.amp_theta(k))
            for(size_t q = 0; q < t.amps.size(); ++q, ++d)
                for(int b = 0; b < n; ++b)
                    e.push_back({true, d, b});
        return e;
    }

    // Declarations before the loop over the normalisation points of amplitude node k: npts (and the points'
    // stride nst), the Amp3Body bin list or the Amp4Body events.
    void normPointsHead(int k, std::ostream &o) {
        const int n3 = (int)T.amp3s.size();
        if(k < n3) {
            o << "    const i64 npts = " << (int64_t)T.amp3s[k].grid.size() << "LL, nst = (npts + 3) & ~3LL; (void)nst;\n";
            o << "    const unsigned *pts = a.dgrid + " << plan.dgrid_off.at(k) << "LL;\n";
        } else {
            o << "    const double *ne = a.nevt[" << k - n3 << "];\n";
            o << "    const i64 npts = a.nnorm[" << k - n3 << "], nst = (npts + 3) & ~3LL; (void)nst;\n";
        }
    }
    // Point p of node k's normalisation set: A and dA (declared by the caller) and its weight `const R e`, the
    // efficiency at an Amp3Body bin centre (the reference's fake event holds 2 in slot 0), 1 for Amp4Body.
    // Reads P (FP64 parameters) and the R parameter locals p<j>.
    void normPoint(int k, std::ostream &o) {
        const int n3 = (int)T.amp3s.size();
        if(k >= n3) {
            o << "      gf_ampv_" << k << "(ne[p], ne[npts + p], ne[2 * npts + p], ne[3 * npts + p], ne[4 * npts + p], P, A, dA);\n";
            o << "      const R e = R(1); (void)e;\n";
            return;
        }
        const Amp3Info &A = T.amp3s[k];
        const gf_observable &g12 = T.obs[A.o12], &g13 = T.obs[A.o13];
        double w12 = g12.hi - g12.lo;
        w12 /= A.nb12;
        double w13 = g13.hi - g13.lo;
        w13 /= A.nb13q;
        o << "      const unsigned q = pts[p];\n";
        o << "      const double c12 = gf_centre(" << lit(g12.lo) << ", " << lit(w12) << ", (int)(q & 0xffffu));\n";
        o << "      const double c13 = gf_centre(" << lit(g13.lo) << ", " << lit(w13) << ", (int)(q >> 16));\n";
        o << "      gf_ampv_" << k << "(c12, c13, P, A, dA);\n";
        std::ostringstream body;
        Ctx c{body, T, false, false, nullptr, nullptr, nullptr, nullptr};
        c.single = mixed;
        c.x = [&](int ob) -> std::string {
            if(ob == A.o12)
                return "((R)c12)";
            if(ob == A.o13)
                return "((R)c13)";
            return "R(2)";
        };
        c.k   = [&](int) -> std::string { throw std::runtime_error("codegen: convolution in an efficiency"); };
        c.tab = [&](int, int) -> std::string { throw std::runtime_error("codegen: convolution in an efficiency"); };
        Val ev = emit(c, A.eff);
        o << "      R e;\n      {\n" << body.str() << "      e = " << ev.v << ";\n      }\n";
    }

    void ampKernels() {
        const int NK = T.n_amp_nodes();
        if(NK == 0)
            return;
        for(int k = 0; k < NK; ++k)
            ampFunction(k);
        const int NA = T.n_amp_cols, NO = (int)T.obs.size(), np = std::max(1, T.n_params);
        const int n3 = (int)T.amp3s.size();

        // data events -> value and derivative columns of every dirty toy
        os << "extern \"C\" __global__ void __launch_bounds__(256) gf_amp(const GfArgs a) {\n";
        os << "  const int toy = blockIdx.y, k = blockIdx.z, tid = threadIdx.x;\n";
        os << "  if(!a.dirty[toy]) return;\n";
        os << "  const i64 n = a.toy_nevents[toy], npad = n < 8 ? 8 : (n + 7) / 8 * 8;\n";
        os << "  const double *P = a.P + (i64)toy * " << np << "; (void)P;\n";
        os << "  R2 *const *ac = reinterpret_cast<R2 *const *>(const_cast<void **>(a.acol)) + (i64)toy * " << NA << ";\n";
        os << "  switch(k) {\n";
        for(int k = 0; k < NK; ++k) {
            const int nAmp = T.amp_count(k), ND = std::max(1, nDeriv(k));
            const auto &theta = T.amp_theta(k);
            os << "  case " << k << ": {\n";
            const int nv = k < n3 ? 2 : 5;
            std::vector<int> ob;
            if(k < n3)
                ob = {T.amp3s[k].o12, T.amp3s[k].o13};
            else
                ob.assign(T.amp4s[k - n3].obs, T.amp4s[k - n3].obs + 5);
            for(int v = 0; v < nv; ++v)
                os << "    const double *x" << v << " = a.dcol[(i64)toy * " << NO << " + " << ob[v] << "];\n";
            os << "    R2 A[" << nAmp << "], dA[" << ND << "];\n";
            os << "    for(i64 i = (i64)blockIdx.x * 256 + tid; i < npad; i += (i64)gridDim.x * 256) {\n";
            os << "      if(i < n) gf_ampv_" << k << "(" << (k < n3 ? "x0[i], x1[i]" : "x0[i], x1[i], x2[i], x3[i], x4[i]")
               << ", P, A, dA);\n";
            os << "      else { for(int q = 0; q < " << nAmp << "; ++q) { A[q].x = R(0); A[q].y = R(0); }\n";
            os << "             for(int q = 0; q < " << ND << "; ++q) { dA[q].x = R(0); dA[q].y = R(0); } }\n";
            for(int q = 0; q < nAmp; ++q)
                os << "      ac[" << T.amp_col0(k) + q << "][i] = A[" << q << "];\n";
            for(int t = 0, d = 0; t < (int)theta.size(); ++t)
                for(size_t j = 0; j < theta[t].amps.size(); ++j, ++d)
                    os << "      if(ac[" << theta[t].col0 + (int)j << "]) ac[" << theta[t].col0 + (int)j << "][i] = dA[" << d
                       << "];\n";
            os << "    }\n    break; }\n";
        }
        os << "  default: break;\n  }\n}\n\n";

        // normalisation points of toy a.gtoy -> scratch columns [value | derivative][point], then the efficiency;
        // columns are nst = npts rounded up to 4 points apart, so that every column starts on 32 bytes
        os << "extern \"C\" __global__ void __launch_bounds__(256) gf_ampn(const GfArgs a) {\n";
        os << "  const int toy = a.gtoy, k = blockIdx.z, tid = threadIdx.x;\n";
        os << "  const double *P = a.P + (i64)toy * " << np << "; (void)P;\n";
        os << "  const R *Pr = reinterpret_cast<const R *>(a.Pr) + (i64)toy * " << plan.nl.npr << "; (void)Pr;\n";
        for(int j = 0; j < T.n_params; ++j)
            os << "  const R p" << j << " = Pr[" << j << "]; (void)p" << j << ";\n";
        os << "  switch(k) {\n";
        plan.dgrid_off.clear();
        int64_t goff = 0;
        for(int k = 0; k < NK; ++k) {
            const int nAmp = T.amp_count(k), ND = std::max(1, nDeriv(k)), NC = nAmp + nDeriv(k);
            os << "  case " << k << ": {\n";
            os << "    R2 *sc = reinterpret_cast<R2 *>(a.nscr[" << k << "]);\n";
            os << "    R2 A[" << nAmp << "], dA[" << ND << "];\n";
            if(k < n3) {
                plan.dgrid_off.push_back(goff);
                goff += (int64_t)T.amp3s[k].grid.size();
            }
            normPointsHead(k, os);
            os << "    R *se = reinterpret_cast<R *>(sc + " << NC << " * nst); (void)se;\n";
            os << "    for(i64 p = (i64)blockIdx.x * 256 + tid; p < npts; p += (i64)gridDim.x * 256) {\n";
            normPoint(k, os);
            if(k < n3)
                os << "      se[p] = e;\n";
            for(int q = 0; q < nAmp; ++q)
                os << "      sc[" << q << " * nst + p] = A[" << q << "];\n";
            for(int d = 0; d < nDeriv(k); ++d)
                os << "      sc[" << nAmp + d << " * nst + p] = dA[" << d << "];\n";
            os << "    }\n    break; }\n";
        }
        os << "  default: break;\n  }\n}\n\n";

        // reduction of the scratch columns into the integral entries, tiles of at most 36 entries
        plan.gram_tiles.clear();
        plan.gram_pairs_max = 0;
        for(int k = 0; k < NK; ++k) {
            const int ne = (int)entries(k).size();
            for(int p0 = 0; p0 < ne; p0 += 36) {
                KernelPlan::GramTile t{k, p0, std::min(ne, p0 + 36)};
                plan.gram_tiles.push_back(t);
                plan.gram_pairs_max = std::max(plan.gram_pairs_max, t.p1 - t.p0);
            }
        }
        // gf_gramr (recompute mode): the same reduction with the amplitudes and their derivatives recomputed at
        // every point instead of read from scratch columns (no per-point storage; each tile of a node evaluates
        // the node's amplitudes again)
        const int PM = plan.gram_pairs_max, NW = 256 / 32;
        for(int rv = 0; rv < (recomputeKernels ? 2 : 1); ++rv) {
        os << "extern \"C\" __global__ void __launch_bounds__(256) " << (rv ? "gf_gramr" : "gf_gram") << "(const GfArgs a) {\n";
        os << "  const int z = blockIdx.z, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;\n";
        os << "  __shared__ double red[" << NW << "][" << 2 * PM << "];\n";
        os << "  double *out = a.gram + ((i64)z * gridDim.x + blockIdx.x) * " << 2 * PM << ";\n";
        if(rv) {
            os << "  const int toy = a.gtoy;\n";
            os << "  const double *P = a.P + (i64)toy * " << np << "; (void)P;\n";
            os << "  const R *Pr = reinterpret_cast<const R *>(a.Pr) + (i64)toy * " << plan.nl.npr << "; (void)Pr;\n";
            for(int j = 0; j < T.n_params; ++j)
                os << "  const R p" << j << " = Pr[" << j << "]; (void)p" << j << ";\n";
        }
        os << "  switch(z) {\n";
        for(size_t ti = 0; ti < plan.gram_tiles.size(); ++ti) {
            const auto &tile = plan.gram_tiles[ti];
            const int k = tile.amp, nAmp = T.amp_count(k), NC = nAmp + nDeriv(k);
            const std::vector<Entry> all = entries(k);
            std::vector<Entry> es(all.begin() + tile.p0, all.begin() + tile.p1);
            std::vector<int> needV(nAmp, 0), needD(std::max(1, nDeriv(k)), 0);
            for(auto &e : es) {
                if(e.h) {
                    needD[e.i] = 1;
                    needV[e.j] = 1;
                } else
                    needV[e.i] = needV[e.j] = 1;
            }
            const int npr = (int)es.size();
            os << "  case " << ti << ": {\n";
            for(int q = 0; q < npr; ++q)
                os << "    R sr" << q << " = R(0), si" << q << " = R(0);\n";
            if(rv) {
                normPointsHead(k, os);
                os << "    for(i64 p = (i64)blockIdx.x * 256 + tid; p < npts; p += (i64)gridDim.x * 256) {\n";
                os << "      R2 A[" << nAmp << "], dA[" << std::max(1, nDeriv(k)) << "];\n";
                normPoint(k, os);
                for(int v = 0; v < nAmp; ++v)
                    if(needV[v])
                        os << "      const R2 b" << v << " = A[" << v << "];\n";
                for(int d = 0; d < nDeriv(k); ++d)
                    if(needD[d])
                        os << "      const R2 g" << d << " = dA[" << d << "];\n";
            } else {
            os << "    const R2 *sc = reinterpret_cast<const R2 *>(a.nscr[" << k << "]);\n";
            if(k < n3)
                os << "    const i64 npts = " << (int64_t)T.amp3s[k].grid.size() << "LL, nst = (npts + 3) & ~3LL;\n"
                   << "    const R *se = reinterpret_cast<const R *>(sc + " << NC << " * nst);\n";
            else
                os << "    const i64 npts = a.nnorm[" << k - n3 << "], nst = (npts + 3) & ~3LL;\n";
            os << "    for(i64 p = (i64)blockIdx.x * 256 + tid; p < npts; p += (i64)gridDim.x * 256) {\n";
            os << "      const R e = " << (k < n3 ? "se[p]" : "R(1)") << ";\n";
            for(int v = 0; v < nAmp; ++v)
                if(needV[v])
                    os << "      const R2 b" << v << " = sc[" << v << " * nst + p];\n";
            for(int d = 0; d < nDeriv(k); ++d)
                if(needD[d])
                    os << "      const R2 g" << d << " = sc[" << nAmp + d << " * nst + p];\n";
            }
            for(int q = 0; q < npr; ++q) {
                const std::string x = es[q].h ? "g" + std::to_string(es[q].i) : "b" + std::to_string(es[q].i);
                const std::string y = "b" + std::to_string(es[q].j);
                os << "      sr" << q << " += (" << x << ".x * " << y << ".x + " << x << ".y * " << y << ".y) * e;\n";
                os << "      si" << q << " += (" << x << ".y * " << y << ".x - " << x << ".x * " << y << ".y) * e;\n";
            }
            os << "    }\n";
            for(int q = 0; q < npr; ++q) {
                os << "    { const double t = gf_warp_sum((double)sr" << q << "); if(lane == 0) red[wid][" << 2 * q
                   << "] = t; }\n";
                os << "    { const double t = gf_warp_sum((double)si" << q << "); if(lane == 0) red[wid][" << 2 * q + 1
                   << "] = t; }\n";
            }
            os << "    __syncthreads();\n";
            os << "    if(tid < " << 2 * npr << ") { double t = 0.0; for(int w = 0; w < " << NW
               << "; ++w) t += red[w][tid]; out[tid] = t; }\n";
            os << "    break; }\n";
        }
        os << "  default: break;\n  }\n}\n\n";
        }
    }

    // ---------------- event pass ----------------
    // Persistent CTAs take contiguous ranges of the chunk list and stage a toy's conv tables once; each
    // thread streams 8 events per iteration with 16-byte loads.  Partial sums: FP32 per thread, then
    // compensated FP32 pairs across the warp, the CTA, the chunks of a toy; FP64 for the final value.
    // asBody: the same event pass as a device function of the one-launch kernel.  tab (one toy, an event
    // function that depends on the event only through one convolution's bin offset k): each CTA first
    // tabulates the per-event terms -log P and -dP/P over the table's k range in shared memory, and the
    // event loop gathers and adds them
    // Bin offsets of convolution ci as the event pass reads them; in tab mode the sorted copy of toy 0's offsets
    // when the engine provides one (the order of an event pass whose terms depend on the offset alone is free)
    std::string kcolExpr(int ci, bool tab) const {
        const std::string k = p0ptr("a.kcol", (int)T.convs.size(), ci, (int)T.obs.size());
        return tab && ci == 0 ? "(a.ksort ? (const void *)a.ksort : " + k + ")" : k;
    }

    // recompute (amplitude trees, gradient pass): dA/dt of the amplitude nodes is recomputed per event from the
    // FP64 event columns by the nodes' amplitude functions instead of read from stored derivative columns; the
    // amplitudes themselves are still read from their cached value columns
    void eventKernel(bool grad, bool values, bool asBody = false, bool tab = false) {
        const bool rc = recompute && grad && !values && !asBody && !tab;
        const std::string name = values ? "gf_val_n" : (grad ? (rc ? "gf_evt_gr" : "gf_evt_g") : "gf_evt_n");
        const int NGp = 1 + (grad ? T.NG : 0);
        const int NGs = 1 + T.NG;
        const int NC  = (int)T.convs.size();
        const int NO  = (int)T.obs.size();
        const int NW  = block / 32;
        const int NA  = T.n_amp_cols;
        // events per thread and iteration: 8 (16-byte loads of FP32 columns), 2 when cached amplitudes
        // (one R2 per event and resonance) are streamed as well
        const int VEC = NA > 0 ? 2 : 8;
        auto &off     = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps     = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        if(!values && !asBody)
            (grad ? plan.evt_smem_grad : plan.evt_smem_nograd) = ctabL1 ? 0 : (size_t)ctabTotal * (mixed ? 4 : 8);
        bodySmem = ctabL1 ? 0 : (size_t)ctabTotal * (mixed ? 4 : 8);

        std::vector<int> xused(NO, 0);
        std::ostringstream body;
        Ctx c{body, T, grad, true, nullptr, nullptr, nullptr, &xused};
        c.single = mixed;
        c.lohi = mixed;
        c.x    = [&](int o) {
            xused[o] = 1;
            return "ex" + std::to_string(o);
        };
        c.k   = [&](int ci) { return "ek" + std::to_string(ci); };
        c.tab = [&](int ci, int comp) -> std::string {
            int cp = cps[ci];
            if(!mixed)
                return "tp" + std::to_string(ci) + "[" + std::to_string(comp) + "]";
            if(cp == 1)
                return "tq" + std::to_string(ci);
            const char *fld[] = {".x", ".y", ".z", ".w"};
            if(cp == 2)
                return "tq" + std::to_string(ci) + fld[comp];
            return "tq" + std::to_string(ci) + "_" + std::to_string(comp / 4) + fld[comp % 4];
        };
        std::vector<int> aused(std::max(1, NA), 0);
        if(T.fit_metric != GF_FIT_UNBINNED_NLL && !values) {
            c.x(NO - 2);
            c.x(NO - 1);
        }
        c.amp = [&](int ai, int r) {
            aused[T.amp_col0(ai) + r] = 1;
            return "am" + std::to_string(T.amp_col0(ai) + r);
        };
        // derivative column -> (amplitude node, index in its dA array), and which of them the event function reads
        std::map<int, std::pair<int, int>> dcolOf;
        for(int k = 0; k < T.n_amp_nodes(); ++k) {
            int d = 0;
            for(auto &th : T.amp_theta(k))
                for(size_t j = 0; j < th.amps.size(); ++j, ++d)
                    dcolOf[th.col0 + (int)j] = {k, d};
        }
        std::vector<int> rused(std::max(1, NA), 0);
        c.ampcol = [&](int col) {
            if(rc && dcolOf.count(col)) {
                rused[col] = 1;
                return "rd" + std::to_string(col);
            }
            aused[col] = 1;
            return "am" + std::to_string(col);
        };
        Val root = emit(c, 0);
        std::vector<int> rnode(std::max(1, T.n_amp_nodes()), 0);
        for(auto &kv : dcolOf)
            if(rused[kv.first])
                rnode[kv.second.first] = 1;
        if(!values && !grad) {
            plan.obs_used_evt.clear();
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    plan.obs_used_evt.push_back(o);
        }
        const std::string rootN = T.nk[0] == NK_ONE ? "" : "N0";
        // a host-computed root normalisation is applied on the host (plan.factor_root)
        const bool factorRoot = !values && T.fit_metric == GF_FIT_UNBINNED_NLL &&
                                (T.nk[0] == NK_EXP || T.nk[0] == NK_GAUSS || T.nk[0] == NK_AMP3 || T.nk[0] == NK_AMP4);
        plan.factor_root = T.fit_metric == GF_FIT_UNBINNED_NLL &&
                           (T.nk[0] == NK_EXP || T.nk[0] == NK_GAUSS || T.nk[0] == NK_AMP3 || T.nk[0] == NK_AMP4);
        // tabulated terms per k: [-log P, -dP/P per gradient slot, (factored root) 1 if P > 0], kept in
        // blocks of 16 bytes (4 FP32 / 2 FP64 terms), each block its own array over k, the remainder in a
        // narrower array, so that an event's gather reads no padding (C2: 16 + 4 bytes)
        const int tabComps = NGp + (factorRoot ? 1 : 0);
        // mixed precision: each bin's event function and -log P as FP32 pairs (gf_df), the low part of -log P as
        // one more term after the others (an event adds it to the low part of its value sum)
        const int64_t loOff = grad ? plan.ctab_lo_off_grad : plan.ctab_lo_off_nograd;
        const bool dfTab    = tab && mixed && loOff >= 0 && dfEligible();
        const int tabAll    = tabComps + (dfTab ? 1 : 0);
        // the event function's value once more with R = gf_df: conv 0's value read as (high, low) pair
        std::ostringstream bodyDF;
        std::string pvDF;
        if(dfTab) {
            Ctx cd{bodyDF, T, false, true, nullptr, nullptr, nullptr, nullptr};
            cd.lohi = true;
            cd.single = true;
            cd.x    = [&](int) -> std::string {
                throw std::runtime_error("codegen: the tabulated event function reads an observable");
            };
            cd.k   = c.k;
            cd.tab = [&](int ci, int comp) { return "gf_df(" + c.tab(ci, comp) + ", tlo0)"; };
            const Val rd = emit(cd, 0);
            pvDF         = factorRoot ? rd.v : normMul(cd, 0, rd.v);
        }
        const int vw = mixed ? 4 : 2;
        std::vector<int> bw, boff; // per block: width (terms) and offset (elements) in ltab
        int LP = 0;
        for(int q0 = 0; q0 < tabAll; q0 += vw) {
            int w = std::min(vw, tabAll - q0);
            if(w == 3)
                w = 4;
            bw.push_back(w);
            boff.push_back(LP * (tab ? T.convs[0].nK : 0));
            LP += w;
        }
        if(tab)
            bodySmem = (size_t)T.convs[0].nK * LP * (mixed ? 4 : 8);
        auto vtype = [&](int w) -> std::string {
            return mixed ? (w == 4 ? "float4" : w == 2 ? "float2" : "float") : (w == 2 ? "double2" : "double");
        };

        // at least two CTAs per SM: the register cap (128 at 256 threads) keeps the amplitude event kernels
        // at two resident CTAs instead of one.  FP32 batch kernels with 8 events per iteration: four (58
        // registers, no spills; 1024 toys of the composite model: event kernel 0.086 -> 0.068 ms); the one-toy
        // kernel stays at two (three or four made the 2e6-event FCN 0.5 / 3 us slower)
        const int minBlocks = (VEC == 8 && mixed && batch) ? 4 : 2;
        // the one-launch kernel may have bulk-copied the CTA's events into shared memory (gf_st != null):
        // stream s at gf_st + gf_soff[s], event i at index i - gf_ib, complete once gf_mbar's phase 0 is
        kernelHead(name, std::to_string(block) + ", " + std::to_string(minBlocks), asBody,
                   ", const unsigned char *gf_st, const int *gf_soff, long long gf_ib, unsigned long long *gf_mbar");
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *stab = reinterpret_cast<R *>(smraw); (void)stab;\n";
        os << "  __shared__ int s_toy, last;\n";
        if(rc)
            os << "  __shared__ double sPd[" << std::max(1, T.n_params) << "];\n";
        if(!values)
            os << "  __shared__ ACC red[" << NW << "][" << NGp + 1 << "];\n";
        os << "  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5; (void)lane; (void)wid;\n";
        os << "  const int cb = (int)(((i64)a.n_chunks * blockIdx.x) / gridDim.x);\n";
        os << "  const int ce = (int)(((i64)a.n_chunks * (blockIdx.x + 1)) / gridDim.x);\n";
        os << "  if(tid == 0) s_toy = -1;\n";
        os << "  gf_pdl_trigger();\n";
        // event columns do not depend on the preceding kernels: pull the first chunk towards L2 meanwhile
        // (the one-launch kernel bulk-copies or bulk-prefetches every CTA's events at its start instead)
        os << "  if(" << (asBody ? "false && " : "") << "cb < ce) {\n";
        os << "    int toy; i64 b0, e0; gf_chunk(a, cb, toy, b0, e0);\n";
        os << "    {\n";
        os << "      for(i64 i0 = b0 + " << VEC << " * (i64)tid; i0 < e0; i0 += " << VEC << " * " << block << ") {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "        asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(reinterpret_cast<const R *>("
                   << p0ptr("a.col", NO, o, 0) << ") + i0));\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "        asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(reinterpret_cast<const int *>("
               << p0ptr("a.kcol", NC, ci, NO) << ") + i0));\n";
        for(int ac = 0; ac < NA; ++ac)
            if(aused[ac])
                os << "        asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(reinterpret_cast<const R2 *>("
                   << p0ptr("a.acol", NA, ac, NO + NC) << ") + i0));\n";
        os << "      }\n    }\n  }\n";
        evtStreams.clear();
        if(!values && !asBody)
            evtReadsObs[grad ? 1 : 0] = std::find(xused.begin(), xused.end(), 1) != xused.end();
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                evtStreams.push_back({p0ptr("a.col", NO, o, 0), mixed ? 4 : 8});
        for(int ci = 0; ci < NC; ++ci)
            evtStreams.push_back({kcolExpr(ci, tab), 4});
        for(int ac = 0; ac < NA; ++ac)
            if(aused[ac])
                evtStreams.push_back({p0ptr("a.acol", NA, ac, NO + NC), mixed ? 8 : 16});
        // one toy: its parameters and activity flag (written by the host, possibly read in place from
        // page-locked memory) are read once per CTA before the wait, the normalisation factors once after it
        if(!batch) {
            os << "  const int toy1 = 0;\n";
            os << "  const bool toy_on1 = !a.active || a.active[toy1];\n";
            os << "  const R *Pr1 = reinterpret_cast<const R *>(GF_PR); (void)Pr1;\n";
            for(int j = 0; j < T.n_params; ++j)
                os << "  const R p" << j << " = Pr1[" << j << "]; (void)p" << j << ";\n";
        }
        os << "  gf_pdl_wait();\n";
        os << "  __syncthreads();\n";
        if(!batch) {
            os << "  const int toy = toy1;\n  const R *Pr = Pr1; (void)Pr;\n";
            // one-launch evaluation: the status words, read before the tables (written before the grid barrier;
            // a CTA stopped later leaves its rows unwritten, which the host detects)
            if(asBody)
                os << "  int gf_q0 = 0; unsigned gf_g2 = 0;\n  if(tid == 0) { gf_q0 = a.qflag[0]; gf_g2 = a.gbar[2]; }\n";
            if(!tab)
                emitNormReads(os, T, grad, plan.nl, "  ");
            else {
                // one pass over the toy's table: every thread loads its rows once (all loads in flight), the
                // CTA sums the folded grid normalisation of the convolution's numeric node itself (from the
                // table CTAs' partials of sum_k n_k T[k], so no finishing CTA), then each row's per-event
                // terms go to shared memory
                const ConvInfo &cv = T.convs[0];
                const int cp = cps[0], per = std::min(cp, mixed ? 4 : 2), nvr = cp / per;
                const int NR = (cv.nK + block - 1) / block;
                const std::string vt = vtype(per);
                const int fq = plan.conv_fold_q[0];
                const int comps = convComps(0, grad);
                os << "  R *ltab = stab;\n";
                // rows [kr_lo, kr_hi] of the table: with the events sorted by bin, those between this CTA's first
                // and last event (read from its staged copy once that has arrived), else all of them
                os << "  int kr_lo = 0, kr_hi = " << cv.nK - 1 << ";\n";
                if(asBody) {
                    os << "  if(a.ksort) {\n    kr_hi = -1;\n";
                    os << "    const i64 le = ((i64)ce * a.chunk < a.nevt0 ? (i64)ce * a.chunk : a.nevt0) - 1;\n";
                    os << "    if(cb < ce && le >= gf_ib) {\n";
                    os << "      if(gf_st && gf_mbar_wait(gf_mbar, 0u, 1000000000ull)) {\n";
                    os << "        const int *ks = reinterpret_cast<const int *>(gf_st + gf_soff[0]);\n";
                    os << "        kr_lo = ks[0] - " << cv.kmin << "; kr_hi = ks[le - gf_ib] - " << cv.kmin << ";\n";
                    os << "      } else { kr_lo = a.ksort[gf_ib] - " << cv.kmin << "; kr_hi = a.ksort[le] - " << cv.kmin << "; }\n";
                    os << "      kr_lo = max(kr_lo, 0); kr_hi = min(kr_hi, " << cv.nK - 1 << ");\n";
                    os << "    }\n  }\n";
                }
                if(asBody)
                    os << "  int cnt_ok = 0, cnt_nrows = kr_hi - kr_lo + 1, cnt_nev = 0; (void)cnt_nev;\n";
                os << "  " << vt << " tv[" << NR << "][" << nvr << "];\n";
                os << "  {\n    const R *gt = reinterpret_cast<const R *>(a.ctab) + " << off[0] << ";\n";
                os << "#pragma unroll\n    for(int r = 0; r < " << NR << "; ++r) {\n      const int kk = kr_lo + tid + r * " << block
                   << ";\n      if(kk <= kr_hi) {\n";
                os << "#pragma unroll\n        for(int v = 0; v < " << nvr << "; ++v) tv[r][v] = *reinterpret_cast<const " << vt
                   << " *>(gt + kk * " << cp << " + " << per << " * v);\n";
                os << "      }\n    }\n  }\n";
                if(dfTab) {
                    os << "  float tlo[" << NR << "];\n";
                    os << "  {\n    const float *gl = reinterpret_cast<const float *>(a.ctab) + " << loOff << ";\n";
                    // zero, then predicated loads: nothing consumes them before the per-bin terms
                    os << "#pragma unroll\n    for(int r = 0; r < " << NR << "; ++r) {\n      const int kk = kr_lo + tid + r * "
                       << block << ";\n      tlo[r] = 0.f;\n      if(kk <= kr_hi) tlo[r] = gl[kk];\n    }\n  }\n";
                }
                // the other normalisation factors as usual
                {
                    std::ostringstream nr;
                    emitNormReads(nr, T, grad, plan.nl, "  ");
                    std::string txt = nr.str();
                    if(fq >= 0) {
                        // drop the folded node's reads from Nq: its factors come from the CTA's own sum
                        const int node = T.nums[fq].node;
                        std::istringstream in(txt);
                        std::string line, keep;
                        const std::string a1 = "const R N" + std::to_string(node) + " = Nq[";
                        const std::string a2 = "const R dN" + std::to_string(node) + "_";
                        while(std::getline(in, line))
                            if(line.find(a1) == std::string::npos && line.find(a2) == std::string::npos)
                                keep += line + "\n";
                        txt = keep;
                    }
                    os << txt;
                }
                if(fq < 0 && asBody)
                    emitCountPass(cv);
                if(fq >= 0) {
                    const NumInfo &g = T.nums[fq];
                    const int node   = g.node;
                    const double cc  = g.volume / (double)g.total;
                    os << "  __shared__ R s_fn[" << 2 + comps << "];\n";
                    os << "  __shared__ int s_fbits;\n";
                    // the table CTAs' partials of sum_k n_k T_c[k] (component c of gradient slot cs[c]), one per
                    // table CTA, summed here by every CTA in the same order
                    const int KB   = convShape(grad).KB[0];
                    const int nblk = (cv.nK + KB - 1) / KB, MGB = plan.max_grid_blocks;
                    const int NQ   = (int)T.nums.size(), NGs = 1 + T.NG;
                    os << "  {\n";
                    os << "    const ACC *gp = reinterpret_cast<const ACC *>(a.gpartial) + ((i64)toy * " << NQ << " + " << fq
                       << ") * " << NGs << " * " << MGB << ";\n";
                    if(nblk <= block) {
                        // one partial per thread and component: all loads issued before any is used
                        for(int c = 0; c < comps; ++c)
                            os << "    ACC fs" << c << " = acc_zero();\n";
                        os << "    if(tid < " << nblk << ") {\n";
                        for(int c = 0; c < comps; ++c) {
                            const int cs = c == 0 ? 0 : 1 + cv.dep[c - 1];
                            os << "      fs" << c << " = gp[" << cs * MGB << " + tid];\n";
                        }
                        os << "    }\n";
                    } else
                        for(int c = 0; c < comps; ++c) {
                            const int cs = c == 0 ? 0 : 1 + cv.dep[c - 1];
                            os << "    ACC fs" << c << " = acc_zero();\n";
                            os << "    for(int bi = tid; bi < " << nblk << "; bi += " << block << ") fs" << c << " = acc_add(fs" << c
                               << ", gp[" << cs * MGB << " + bi]);\n";
                        }
                    std::vector<std::string> vals;
                    for(int c = 0; c < comps; ++c)
                        vals.push_back("fs" + std::to_string(c));
                    if(asBody)
                        emitCountPass(cv);
                    emitCtaReduce(os, vals, "    ");
                    // GooPdf::normalize's numeric branch (src/PDFs/GooPdf.cu:366-395) on the CTA's sums
                    // lane c of warp 0 sums component c over the warps; lane 0 gathers them
                    os << "    if(tid < 32) {\n";
                    os << "      ACC tc = acc_zero();\n";
                    os << "      if(lane < " << comps << ") for(int w = 0; w < " << NW << "; ++w) tc = acc_add(tc, red[w][lane]);\n";
                    os << "      ACC tt[" << comps << "];\n";
                    os << "#pragma unroll\n      for(int c = 0; c < " << comps << "; ++c) tt[c] = acc_shfl(tc, c);\n";
                    os << "      if(lane == 0) {\n";
                    if(mixed) {
                        // N = 1 / (cc S) as an FP32 pair, from the pair S (no FP64 division on the critical path)
                        const float cch = (float)cc, ccl = (float)(cc - (double)cch);
                        char cb[96];
                        std::snprintf(cb, sizeof cb, "gf_df(%.9ef, %.9ef)", (double)cch, (double)ccl);
                        os << "      const gf_df Sd(tt[0].x, tt[0].y);\n";
                        os << "      s_fbits = isnan(Sd.h) ? 1 : !(Sd.h > 0.f) ? 2 : 0;\n";
                        os << "      const gf_df Nd = gf_df(1) / (Sd * " << cb << ");\n";
                        os << "      const R N = Nd.h;\n";
                        os << "      s_fn[0] = N;\n      s_fn[1] = Nd.l;\n";
                    } else {
                        os << "      const double S = acc_value(tt[0]);\n";
                        os << "      s_fbits = isnan(S) ? 1 : !(S > 0.0) ? 2 : 0;\n";
                        os << "      const double I = " << lit(cc) << " * S;\n";
                        os << "      const double Nd = 1.0 / I;\n";
                        os << "      const R N = (R)Nd;\n";
                        os << "      s_fn[0] = N;\n      s_fn[1] = (R)(Nd - (double)N);\n";
                    }
                    if(grad)
                        for(int j = 1; j < comps; ++j)
                            os << "      s_fn[" << 1 + j << "] = -N * N * (R)" << lit(cc) << " * (R)acc_r(tt[" << j << "]);\n";
                    os << "      }\n    }\n    __syncthreads();\n  }\n";
                    os << "  const R N" << node << " = s_fn[0], NL" << node << " = s_fn[1]; (void)NL" << node << ";\n";
                    if(grad)
                        for(auto &d : plan.nl.qdN[fq]) {
                            const auto &dep = cv.dep;
                            const int j = (int)(std::find(dep.begin(), dep.end(), d.first) - dep.begin());
                            os << "  const R dN" << node << "_" << d.first << " = s_fn[" << 2 + j << "];\n";
                        }
                }
                // per-k terms
                os << "#pragma unroll\n  for(int r = 0; r < " << NR << "; ++r) {\n    const int kk = kr_lo + tid + r * " << block
                   << ";\n    if(kk <= kr_hi) {\n";
                os << "      const int ek0 = " << cv.kmin << " + kk; (void)ek0;\n";
                if(mixed) {
                    if(cp == 1)
                        os << "      const float tq0 = tv[r][0];\n";
                    else if(cp == 2)
                        os << "      const float2 tq0 = tv[r][0];\n";
                    else
                        for(int g4 = 0; g4 < cp / 4; ++g4)
                            os << "      const float4 tq0_" << g4 << " = tv[r][" << g4 << "];\n";
                } else
                    os << "      const R *tp0 = reinterpret_cast<const R *>(tv[r]); (void)tp0;\n";
                os << "      {\n" << body.str();
                const std::string pvE = factorRoot ? root.v : normMul(c, 0, root.v);
                os << "      const R pv = " << pvE << ";\n";
                if(dfTab) {
                    os << "      gf_df pvd;\n      {\n        typedef gf_df R;\n        const float tlo0 = tlo[r];\n";
                    os << bodyDF.str();
                    os << "        pvd = " << pvDF << ";\n      }\n";
                }
                os << "      R lt[" << LP << "];\n#pragma unroll\n      for(int q = 0; q < " << LP << "; ++q) lt[q] = R(0);\n";
                os << "      if(pv > R(0)) {\n";
                if(dfTab)
                    os << "        const gf_df ld = gf_df_log(pvd);\n        lt[0] = -ld.h;\n        lt[" << tabComps
                       << "] = -ld.l;\n";
                else
                    os << "        lt[0] = -GF_LOG(pv);\n";
                if(grad && T.NG > 0) {
                    os << "        const R inv = gf_rcp(pv);\n";
                    for(int sl = 0; sl < T.NG; ++sl) {
                        std::string e;
                        auto it = root.g.find(sl);
                        if(factorRoot) {
                            if(it != root.g.end())
                                e = it->second;
                        } else {
                            if(it != root.g.end())
                                e = rootN.empty() ? it->second : it->second + " * " + rootN;
                            std::string dn = T.nk[0] == NK_ONE ? "" : dnormExpr(c, 0, sl);
                            if(!dn.empty())
                                e += (e.empty() ? "" : " + ") + root.v + " * " + dn;
                        }
                        if(!e.empty())
                            os << "        lt[" << 1 + sl << "] = -(" << e << ") * inv;\n";
                    }
                }
                if(factorRoot)
                    os << "        lt[" << tabComps - 1 << "] = R(1);\n";
                os << "      }\n";
                for(size_t b = 0; b < bw.size(); ++b)
                    for(int q = 0; q < bw[b]; ++q)
                        os << "      ltab[" << boff[b] << " + kk * " << bw[b] << " + " << q << "] = lt[" << vw * (int)b + q
                           << "];\n";
                os << "      }\n    }\n  }\n  __syncthreads();\n";
            }
        }
        const bool countMode = asBody && tab;
        if(countMode) {
            // counted events (cnt_ok, from the counting pass below the table loads): each bin's terms
            // times its events' count (the value as an exact product pair), in place of the per-event loop; the
            // CTA's sums go to its first chunk's row, its other chunks' rows get zeros
            const int NGc0 = NGp + (factorRoot ? 1 : 0);
            const char *fld[] = {".x", ".y", ".z", ".w"};
            auto compC = [&](int q) {
                const int b = q / vw;
                return "lq" + std::to_string(b) + (bw[b] == 1 ? std::string("") : std::string(fld[q % vw]));
            };
            const bool foldTab = plan.conv_fold_q[0] >= 0;
            const std::string st = std::string("(double)(gf_q0 | (gf_g2 ? 8 : 0)") + (foldTab ? " | s_fbits" : "") + ")";
            os << "  if(cnt_ok) {\n";
            os << "    ACC cs0 = acc_zero();\n";
            for(int sl = 0; sl < NGp - 1; ++sl)
                os << "    ACC cs" << 1 + sl << " = acc_zero();\n";
            if(factorRoot)
                os << "    ACC csn = acc_zero();\n";
            os << "    for(int r = tid; r < cnt_nrows; r += " << block << ") {\n";
            os << "      const int st = gf_rstart[r];\n      if(st < 0) continue;\n";
            os << "      int en = cnt_nev;\n";
            os << "      for(int q = r + 1; q < cnt_nrows; ++q) { const int sq = gf_rstart[q]; if(sq >= 0) { en = sq; break; } }\n";
            os << "      const R c = (R)(en - st);\n";
            os << "      const int lk = kr_lo + r;\n";
            for(size_t b = 0; b < bw.size(); ++b)
                os << "      const " << vtype(bw[b]) << " lq" << b << " = *reinterpret_cast<const " << vtype(bw[b])
                   << " *>(ltab + " << boff[b] << " + lk * " << bw[b] << ");\n";
            os << "      cs0 = acc_add(cs0, gf_two_prod(c, " << compC(0) << "));\n";
            if(dfTab)
                os << "      cs0 = acc_add(cs0, acc_of(c * " << compC(tabComps) << "));\n";
            for(int sl = 0; sl < NGp - 1; ++sl)
                os << "      cs" << 1 + sl << " = acc_add(cs" << 1 + sl << ", gf_two_prod(c, " << compC(1 + sl) << "));\n";
            if(factorRoot)
                os << "      csn = acc_add(csn, acc_of(c * " << compC(tabComps - 1) << "));\n";
            os << "    }\n";
            std::vector<std::string> vals{"cs0"};
            for(int sl = 0; sl < NGp - 1; ++sl)
                vals.push_back("cs" + std::to_string(1 + sl));
            if(factorRoot)
                vals.push_back("csn");
            emitCtaReduce(os, vals, "    ");
            os << "    if(tid < " << NGc0 << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
               << "; ++w) t = acc_add(t, red[w][tid]); a.hpart[(i64)cb * " << NGc0 + 1 << " + tid] = acc_value(t); }\n";
            os << "    if(tid == 0) a.hpart[(i64)cb * " << NGc0 + 1 << " + " << NGc0 << "] = " << st << ";\n";
            os << "    for(int ch = cb + 1; ch < ce; ++ch) {\n";
            os << "      if(tid < " << NGc0 << ") a.hpart[(i64)ch * " << NGc0 + 1 << " + tid] = 0.0;\n";
            os << "      if(tid == 0) a.hpart[(i64)ch * " << NGc0 + 1 << " + " << NGc0 << "] = " << st << ";\n";
            os << "    }\n";
            os << "  } else {\n";
        }
        if(asBody) {
            // staged events: every thread waits for the bulk copy (bounded); a copy that does not arrive leaves
            // this CTA's chunks unevaluated, so that their rows stay unwritten and the host reports the failure
            os << "  bool gf_ok = true;\n";
            os << "  if(gf_st && !gf_mbar_wait(gf_mbar, 0u, 1000000000ull)) {\n";
            os << "    gf_ok = false;\n    if(tid == 0 && a.gbar) atomicOr(a.gbar + 2, 2u);\n  }\n";
            os << "  for(int ch = cb; gf_ok && ch < ce; ++ch) {\n";
        } else
            os << "  for(int ch = cb; ch < ce; ++ch) {\n";
        os << "    int toy; i64 b0, e0; gf_chunk(a, ch, toy, b0, e0);\n";
        if(rc) {
            // the toy's FP64 parameters for the amplitude functions, and the FP64 event columns they read
            const int np = std::max(1, T.n_params), n3 = (int)T.amp3s.size();
            os << "    __syncthreads();\n";
            os << "    for(int q = tid; q < " << np << "; q += " << block << ") sPd[q] = a.P[(i64)toy * " << np << " + q];\n";
            os << "    __syncthreads();\n";
            for(int k = 0; k < T.n_amp_nodes(); ++k) {
                if(!rnode[k])
                    continue;
                std::vector<int> ob;
                if(k < n3)
                    ob = {T.amp3s[k].o12, T.amp3s[k].o13};
                else
                    ob.assign(T.amp4s[k - n3].obs, T.amp4s[k - n3].obs + 5);
                for(size_t v = 0; v < ob.size(); ++v)
                    os << "    const double *xd" << k << "_" << v << " = a.dcol[(i64)toy * " << NO << " + " << ob[v] << "];\n";
            }
        }
        // the activity flag is read beside the parameters (independent loads), the branch comes after them
        if(batch)
            os << "    const bool toy_on = !a.active || a.active[toy];\n";
        else
            os << "    const bool toy_on = toy_on1;\n";
        if(tab) {
            // per-k terms were tabulated before the chunk loop
        } else if(NC > 0 && ctabL1) {
            // the toy's tables are read through L1 (read-only loads): every CTA on an SM shares one copy
            os << "    const R *ttab = reinterpret_cast<const R *>(a.ctab) + (i64)toy * " << ctabTotal << ";\n";
        } else if(NC > 0) {
            // all of a thread's 16-byte loads issued before its stores (one L2 round trip, not one per load)
            const int perV = mixed ? 4 : 2;
            const int64_t nv = ctabTotal / perV;
            const int nr = (int)((nv + block - 1) / block);
            const char *vt = mixed ? "float4" : "double2";
            os << "    const R *ttab = stab;\n";
            os << "    if(toy != s_toy) {\n";
            os << "      __syncthreads();\n";
            os << "      { const " << vt << " *src = reinterpret_cast<const " << vt << " *>(reinterpret_cast<const R *>(a.ctab) + "
                  "(i64)toy * " << ctabTotal << "); " << vt << " *dst = reinterpret_cast<" << vt << " *>(stab);\n";
            if(nr <= 16) {
                os << "        " << vt << " tv[" << nr << "];\n";
                os << "#pragma unroll\n        for(int r = 0; r < " << nr << "; ++r) { const int i = tid + r * " << block
                   << "; if(i < " << nv << ") tv[r] = src[i]; }\n";
                os << "#pragma unroll\n        for(int r = 0; r < " << nr << "; ++r) { const int i = tid + r * " << block
                   << "; if(i < " << nv << ") dst[i] = tv[r]; }\n";
            } else
                os << "        for(int i = tid; i < " << nv << "; i += " << block << ") dst[i] = src[i];\n";
            os << "      }\n";
            os << "      if(tid == 0) s_toy = toy;\n";
            os << "      __syncthreads();\n";
            os << "    }\n";
        }
        if(batch) {
            emitParamsR(os, T, plan.nl, "    ");
            emitNormReads(os, T, grad, plan.nl, "    ");
        }
        if(T.fit_metric != GF_FIT_UNBINNED_NLL && !values)
            os << "    const R Tn = (R)a.toy_nevents[toy]; // c_totalEvents: the number of bins\n";
        // a staged stream's pointer is shifted by gf_ib events (integer arithmetic on the address), so that the
        // loads below index it by the global event number as they index the column in global memory
        int stream = 0;
        auto colPtr = [&](const std::string &type, int bytes, const std::string &glob) {
            std::string e = "reinterpret_cast<const " + type + " *>(" + glob + ")";
            if(asBody)
                e = "(gf_st ? reinterpret_cast<const " + type + " *>(reinterpret_cast<unsigned long long>(gf_st + gf_soff[" +
                    std::to_string(stream) + "]) - (unsigned long long)gf_ib * " + std::to_string(bytes) + "ull) : " + e + ")";
            ++stream;
            return e;
        };
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "    const R *col" << o << " = " << colPtr("R", mixed ? 4 : 8, p0ptr("a.col", NO, o, 0)) << ";\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "    const int *kc" << ci << " = " << colPtr("int", 4, kcolExpr(ci, tab)) << ";\n";
        for(int ac = 0; ac < NA; ++ac)
            if(aused[ac])
                os << "    const R2 *acp" << ac << " = " << colPtr("R2", mixed ? 8 : 16, p0ptr("a.acol", NA, ac, NO + NC))
                   << ";\n";
        os << "    if(!toy_on) continue;\n";
        // per-thread sums: each iteration's VEC events are summed plainly (av, ag), then added to a two-sum
        // compensated pair (avh + avl, agh + agl), so that a thread's many events add no rounding noise
        if(!values) {
            os << "    R avh = R(0), avl = R(0), nv = R(0); (void)nv;\n";
            for(int s = 0; s < NGp - 1; ++s)
                os << "    R agh" << s << " = R(0), agl" << s << " = R(0);\n";
        }
        // software pipelining (mixed precision, 8 events per iteration, at most 3 streamed columns): the next
        // iteration's 16-byte column loads are issued before this iteration's arithmetic
        int nStream = NC;
        for(int o = 0; o < NO; ++o)
            nStream += xused[o] ? 1 : 0;
        const bool pipe = mixed && VEC == 8 && nStream <= 3;
        if(pipe) {
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    os << "    float4 nx" << o << "a = make_float4(0.f, 0.f, 0.f, 0.f), nx" << o << "b = nx" << o << "a;\n";
            for(int ci = 0; ci < NC; ++ci)
                os << "    int4 nk" << ci << "a = make_int4(0, 0, 0, 0), nk" << ci << "b = nk" << ci << "a;\n";
            os << "    if(b0 + " << VEC << " * (i64)tid < e0) {\n";
            os << "      const i64 i1 = b0 + " << VEC << " * (i64)tid;\n";
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    os << "      nx" << o << "a = *reinterpret_cast<const float4 *>(col" << o << " + i1); nx" << o
                       << "b = *reinterpret_cast<const float4 *>(col" << o << " + i1 + 4);\n";
            for(int ci = 0; ci < NC; ++ci)
                os << "      nk" << ci << "a = *reinterpret_cast<const int4 *>(kc" << ci << " + i1); nk" << ci
                   << "b = *reinterpret_cast<const int4 *>(kc" << ci << " + i1 + 4);\n";
            os << "    }\n";
        }
        os << "    for(i64 i0 = b0 + " << VEC << " * (i64)tid; i0 < e0; i0 += " << VEC << " * " << block << ") {\n";
        if(pipe) {
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    os << "      const float4 xv" << o << "a = nx" << o << "a, xv" << o << "b = nx" << o << "b;\n";
            for(int ci = 0; ci < NC; ++ci)
                os << "      const int4 kv" << ci << "a = nk" << ci << "a, kv" << ci << "b = nk" << ci << "b;\n";
            os << "      {\n        const i64 i1 = i0 + " << VEC << " * " << block << ";\n";
            os << "        if(i1 < e0) {\n";
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    os << "          nx" << o << "a = *reinterpret_cast<const float4 *>(col" << o << " + i1); nx" << o
                       << "b = *reinterpret_cast<const float4 *>(col" << o << " + i1 + 4);\n";
            for(int ci = 0; ci < NC; ++ci)
                os << "          nk" << ci << "a = *reinterpret_cast<const int4 *>(kc" << ci << " + i1); nk" << ci
                   << "b = *reinterpret_cast<const int4 *>(kc" << ci << " + i1 + 4);\n";
            os << "        }\n      }\n";
        }
        // FP32 one-toy/batch kernels with 8 events per iteration take one log per iteration, of the product
        // of its events' probabilities (gf_log_acc); the amplitude kernels' 2-event iterations keep one per event
        const bool logProd = mixed && !values && VEC == 8 && !tab;
        if(!values) {
            os << "      R av = R(0);\n";
            for(int s = 0; s < NGp - 1; ++s)
                os << "      R ag" << s << " = R(0);\n";
            if(logProd)
                os << "      float lm = 1.0f; int le = 0;\n";
        }
        // events of this iteration inside the chunk: a 32-bit bound per event instead of a 64-bit one
        os << "      const int jn = e0 - i0 < " << VEC << " ? (int)(e0 - i0) : " << VEC << ";\n";
        for(int o = 0; o < NO && VEC == 2; ++o)
            if(xused[o]) {
                if(mixed)
                    os << "      const float2 xv" << o << " = *reinterpret_cast<const float2 *>(col" << o << " + i0);\n";
                else
                    os << "      const double2 xv" << o << " = *reinterpret_cast<const double2 *>(col" << o << " + i0);\n";
                os << "      const R xa" << o << "[2] = {xv" << o << ".x, xv" << o << ".y};\n";
            }
        for(int ci = 0; ci < NC && VEC == 2; ++ci)
            os << "      const int2 kv" << ci << " = *reinterpret_cast<const int2 *>(kc" << ci << " + i0);\n"
               << "      const int ka" << ci << "[2] = {kv" << ci << ".x, kv" << ci << ".y};\n";
        for(int ac = 0; ac < NA; ++ac) {
            if(!aused[ac])
                continue;
            if(mixed)
                os << "      const float4 av" << ac << " = *reinterpret_cast<const float4 *>(acp" << ac << " + i0);\n"
                   << "      const R2 aa" << ac << "[2] = {make_float2(av" << ac << ".x, av" << ac
                   << ".y), make_float2(av" << ac << ".z, av" << ac << ".w)};\n";
            else
                os << "      const R2 aa" << ac << "[2] = {acp" << ac << "[i0], acp" << ac << "[i0 + 1]};\n";
        }
        for(int o = 0; o < NO && VEC == 8; ++o)
            if(xused[o]) {
                if(mixed) {
                    if(!pipe)
                        os << "      const float4 xv" << o << "a = *reinterpret_cast<const float4 *>(col" << o
                           << " + i0), xv" << o << "b = *reinterpret_cast<const float4 *>(col" << o << " + i0 + 4);\n";
                    os << "      const R xa" << o << "[8] = {xv" << o << "a.x, xv" << o << "a.y, xv" << o << "a.z, xv" << o
                       << "a.w, xv" << o << "b.x, xv" << o << "b.y, xv" << o << "b.z, xv" << o << "b.w};\n";
                }
                else {
                    os << "      R xa" << o << "[8];\n";
                    os << "#pragma unroll\n      for(int h = 0; h < 4; ++h) { const double2 t = "
                          "*reinterpret_cast<const double2 *>(col"
                       << o << " + i0 + 2 * h); xa" << o << "[2 * h] = t.x; xa" << o << "[2 * h + 1] = t.y; }\n";
                }
            }
        for(int ci = 0; ci < NC && VEC == 8; ++ci) {
            if(!pipe)
                os << "      const int4 kv" << ci << "a = *reinterpret_cast<const int4 *>(kc" << ci << " + i0), kv" << ci
                   << "b = *reinterpret_cast<const int4 *>(kc" << ci << " + i0 + 4);\n";
            os << "      int ka" << ci << "[8] = {kv" << ci << "a.x, kv" << ci << "a.y, kv" << ci << "a.z, kv" << ci
               << "a.w, kv" << ci << "b.x, kv" << ci << "b.y, kv" << ci << "b.z, kv" << ci << "b.w};\n";
            // an iteration that runs past the chunk's end reads offsets beyond its events: from a staged copy,
            // shared memory past the copied bytes (any value), so they take the table's first row before any
            // gather uses them as an index (their terms are masked out)
            os << "      if(jn < 8) {\n#pragma unroll\n        for(int j = 0; j < 8; ++j) if(j >= jn) ka" << ci
               << "[j] = " << T.convs[ci].kmin << ";\n      }\n";
        }
        // tab: the iteration's events' terms are kept per component and summed pairwise after the loop
        // (exact for equal terms, as neighbouring events in bin order mostly are; three roundings otherwise)
        const int tabAcc = NGp + (factorRoot ? 1 : 0);
        if(tab) {
            // all events of the iteration in one bin (with the events sorted by bin, most iterations): one
            // gather, and each sum is 8 x the term, which is what the pairwise sum of 8 equal terms gives
            const ConvInfo &cv = T.convs[0];
            const char *fld[] = {".x", ".y", ".z", ".w"};
            auto compS = [&](int q) {
                const int b = q / vw;
                return "lq" + std::to_string(b) + (bw[b] == 1 ? std::string("") : std::string(fld[q % vw]));
            };
            os << "      const bool gsame = jn == " << VEC;
            for(int j = 1; j < VEC; ++j)
                os << " && ka0[" << j << "] == ka0[0]";
            os << ";\n      if(gsame) {\n";
            os << "        const int lk = ka0[0] - " << cv.kmin << ";\n";
            for(size_t b = 0; b < bw.size(); ++b)
                os << "        const " << vtype(bw[b]) << " lq" << b << " = *reinterpret_cast<const " << vtype(bw[b])
                   << " *>(ltab + " << boff[b] << " + lk * " << bw[b] << ");\n";
            os << "        av = R(" << VEC << ") * " << compS(0) << ";\n";
            for(int sl = 0; sl < NGp - 1; ++sl)
                os << "        ag" << sl << " = R(" << VEC << ") * " << compS(1 + sl) << ";\n";
            if(factorRoot)
                os << "        nv += R(" << VEC << ") * " << compS(tabComps - 1) << ";\n";
            if(dfTab)
                os << "        avl += R(" << VEC << ") * " << compS(tabComps) << ";\n";
            os << "      } else {\n";
            for(int q = 0; q < tabAcc; ++q)
                os << "      R tsum" << q << "[" << VEC << "];\n";
        }
        if(dfTab)
            os << "      R tsumL[" << VEC << "];\n";
        os << "#pragma unroll\n      for(int j = 0; j < " << VEC << "; ++j) {\n";
        if(tab) {
            // gather the event's tabulated terms (16-byte and narrower shared loads) and add them
            const ConvInfo &cv = T.convs[0];
            const char *fld[] = {".x", ".y", ".z", ".w"};
            os << "        const int lk = ka0[j] - " << cv.kmin << ";\n";
            for(size_t b = 0; b < bw.size(); ++b)
                os << "        const " << vtype(bw[b]) << " lq" << b << " = *reinterpret_cast<const " << vtype(bw[b])
                   << " *>(ltab + " << boff[b] << " + lk * " << bw[b] << ");\n";
            auto comp = [&](int q) {
                const int b = q / vw;
                return "lq" + std::to_string(b) + (bw[b] == 1 ? std::string("") : std::string(fld[q % vw]));
            };
            os << "        {\n        {\n";
            os << "          const bool in = j < jn;\n";
            os << "          tsum0[j] = in ? " << comp(0) << " : R(0);\n";
            for(int sl = 0; sl < NGp - 1; ++sl)
                os << "          tsum" << 1 + sl << "[j] = in ? " << comp(1 + sl) << " : R(0);\n";
            if(factorRoot)
                os << "          tsum" << NGp << "[j] = in ? " << comp(tabComps - 1) << " : R(0);\n";
            if(dfTab)
                os << "          tsumL[j] = in ? " << comp(tabComps) << " : R(0);\n";
            os << "        }\n";
        } else {
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "        const R ex" << o << " = xa" << o << "[j];\n";
        for(int ac = 0; ac < NA; ++ac)
            if(aused[ac])
                os << "        const R2 am" << ac << " = aa" << ac << "[j];\n";
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            int cp             = cps[ci];
            os << "        const int ek" << ci << " = ka" << ci << "[j];\n";
            os << "        const R *tp" << ci << " = ttab + " << off[ci] << " + (ek" << ci << " - " << cv.kmin << ") * "
               << cp << "; (void)tp" << ci << ";\n";
            if(mixed) {
                const char *ld = ctabL1 ? "__ldg(" : "*(";
                if(cp == 1)
                    os << "        const float tq" << ci << " = " << ld << "tp" << ci << ");\n";
                else if(cp == 2)
                    os << "        const float2 tq" << ci << " = " << ld << "reinterpret_cast<const float2 *>(tp" << ci
                       << "));\n";
                else
                    for(int g4 = 0; g4 < cp / 4; ++g4)
                        os << "        const float4 tq" << ci << "_" << g4 << " = " << ld
                           << "reinterpret_cast<const float4 *>(tp" << ci << " + " << 4 * g4 << "));\n";
            }
        }
        for(int k = 0; k < T.n_amp_nodes() && rc; ++k) {
            if(!rnode[k])
                continue;
            // this event's amplitudes and derivatives (a duplicate of the iteration's first event past its end)
            const int nv = k < (int)T.amp3s.size() ? 2 : 5;
            os << "        R2 rA" << k << "[" << T.amp_count(k) << "], rD" << k << "[" << std::max(1, nDeriv(k)) << "];\n";
            os << "        {\n          const i64 ij = i0 + (j < jn ? j : 0);\n          gf_ampv_" << k << "(";
            for(int v = 0; v < nv; ++v)
                os << "xd" << k << "_" << v << "[ij], ";
            os << "sPd, rA" << k << ", rD" << k << ");\n        }\n";
        }
        for(auto &kv : dcolOf)
            if(rused[kv.first])
                os << "        const R2 rd" << kv.first << " = rD" << kv.second.first << "[" << kv.second.second << "];\n";
        os << "        {\n" << body.str();
        os << "        const R pv = " << normMul(c, 0, root.v) << ";\n";
        if(values) {
            os << "        if(j < jn) {\n";
            os << "          double r;\n";
            os << "          if(a.metric == 0) r = (double)" << root.v << ";\n";
            os << "          else if(a.metric == 2) r = (double)pv;\n";
            os << "          else r = pv > R(0) ? -(double)GF_LOG(pv) : 0.0;\n";
            os << "          a.vals[i0 + j] = r;\n        }\n";
        } else {
            // d(P norm)/dp (with the normalisation's derivative) and d(P)/dp for every gradient slot
            auto dpv = [&](int s) {
                std::string e;
                auto it = root.g.find(s);
                if(it != root.g.end())
                    e = rootN.empty() ? it->second : it->second + " * " + rootN;
                std::string dn = T.nk[0] == NK_ONE ? "" : dnormExpr(c, 0, s);
                if(!dn.empty())
                    e += (e.empty() ? "" : " + ") + root.v + " * " + dn;
                return e;
            };
            const std::string nc = "ex" + std::to_string(NO - 2), vw = "ex" + std::to_string(NO - 1);
            switch(T.fit_metric) {
            case GF_FIT_BINNED_NLL: // calculateBinAvg, src/PDFs/MetricPointer.cu:23-37
                os << "        const R raw = pv * " << vw << ";\n";
                os << "        if(j < jn && raw > R(0)) {\n";
                os << "          const R mu = Tn * raw;\n";
                os << "          av += mu - " << nc << " * GF_LOG(mu);\n";
                if(grad && T.NG > 0) {
                    os << "          const R w = Tn * " << vw << " * (R(1) - " << nc << " / mu);\n";
                    for(int s = 0; s < T.NG; ++s) {
                        std::string e = dpv(s);
                        if(!e.empty())
                            os << "          ag" << s << " += (" << e << ") * w;\n";
                    }
                }
                os << "        }\n";
                break;
            case GF_FIT_BINNED_ERROR: // calculateBinWithError, MetricPointer.cu:39-52: P unnormalised
                os << "        if(j < jn) {\n";
                os << "          const R d = (" << root.v << " - " << nc << ") / " << vw << ";\n";
                os << "          av += d * d;\n";
                if(grad && T.NG > 0) {
                    os << "          const R w = R(2) * d / " << vw << ";\n";
                    for(int s = 0; s < T.NG; ++s) {
                        auto it = root.g.find(s);
                        if(it != root.g.end())
                            os << "          ag" << s << " += (" << it->second << ") * w;\n";
                    }
                }
                os << "        }\n";
                break;
            case GF_FIT_BINNED_CHISQ: // calculateChisq, MetricPointer.cu:54-60
                os << "        if(j < jn) {\n";
                os << "          const R dd = pv * " << vw << " * Tn - " << nc << ";\n";
                os << "          const R den = " << nc << " > R(1) ? " << nc << " : R(1);\n";
                os << "          av += dd * dd / den;\n";
                if(grad && T.NG > 0) {
                    os << "          const R w = R(2) * dd / den * Tn * " << vw << ";\n";
                    for(int s = 0; s < T.NG; ++s) {
                        std::string e = dpv(s);
                        if(!e.empty())
                            os << "          ag" << s << " += (" << e << ") * w;\n";
                    }
                }
                os << "        }\n";
                break;
            default: // calculateNLL, MetricPointer.cu:13-16
                if(factorRoot) {
                    // -log(P N) = -log P - log N: the event pass sums -log P and -dP/P and counts the events
                    // with P > 0; the host adds count * (-log N) and count * (-dN/N) in FP64
                    os << "        if(j < jn && " << root.v << " > R(0)) {\n";
                    if(logProd)
                        os << "          gf_log_acc(" << root.v << ", lm, le, av);\n";
                    else
                        os << "          av -= GF_LOG(" << root.v << ");\n";
                    os << "          nv += R(1);\n";
                    if(grad && T.NG > 0) {
                        if(c.ampRoot) {
                            // |T|^2 eff: d/dp over the value is 2 inner / |T|^2, the efficiency cancels
                            os << "          const R iT = R(2) / (" << c.ampTr << " * " << c.ampTr << " + " << c.ampTi
                               << " * " << c.ampTi << ");\n";
                            for(int s = 0; s < T.NG; ++s) {
                                auto it = c.ampInner.find(s);
                                if(it != c.ampInner.end())
                                    os << "          ag" << s << " -= " << it->second << " * iT;\n";
                            }
                        } else {
                            os << "          const R inv = gf_rcp(" << root.v << ");\n";
                            for(int s = 0; s < T.NG; ++s) {
                                auto it = root.g.find(s);
                                if(it != root.g.end())
                                    os << "          ag" << s << " -= (" << it->second << ") * inv;\n";
                            }
                        }
                    }
                    os << "        }\n";
                    break;
                }
                os << "        if(j < jn && pv > R(0)) {\n";
                if(logProd)
                    os << "          gf_log_acc(pv, lm, le, av);\n";
                else
                    os << "          av -= GF_LOG(pv);\n";
                if(grad && T.NG > 0) {
                    os << "          const R inv = gf_rcp(pv);\n";
                    for(int s = 0; s < T.NG; ++s) {
                        std::string e = dpv(s);
                        if(!e.empty())
                            os << "          ag" << s << " -= (" << e << ") * inv;\n";
                    }
                }
                os << "        }\n";
            }
        }
        } // not tab
        os << "        }\n      }\n";
        if(!values) {
            if(logProd) {
                os << "      av -= logf(lm) + (float)le * GF_LN2_LO;\n";
                os << "      gf_comp_add(avh, avl, (float)(-le) * GF_LN2_HI);\n";
            }
            if(tab) {
                os << "      av = gf_tree8(tsum0);\n";
                if(dfTab)
                    os << "      avl += gf_tree8(tsumL);\n";
                for(int sl = 0; sl < NGp - 1; ++sl)
                    os << "      ag" << sl << " = gf_tree8(tsum" << 1 + sl << ");\n";
                if(factorRoot)
                    os << "      nv += gf_tree8(tsum" << NGp << ");\n";
                os << "      }\n"; // the iteration's events in several bins
            }
            os << "      gf_comp_add(avh, avl, av);\n";
            // gradient sums are compensated where it is cheap (8 events per iteration) or many events per
            // thread are expected (batches of toys); the amplitude kernels' 2-event iterations add them plainly
            for(int s = 0; s < NGp - 1; ++s)
                if(VEC == 8 || batch)
                    os << "      gf_comp_add(agh" << s << ", agl" << s << ", ag" << s << ");\n";
                else
                    os << "      agh" << s << " += ag" << s << ";\n";
        }
        os << "    }\n";
        if(values) {
            os << "  }\n}\n\n";
            endBody(asBody);
            return;
        }
        // components: value, gradient slots, and (factored root normalisation) the count of events with P > 0,
        // which lands in out[2 + NG]; partials have stride 2 + NG, results 3 + NG
        const int NGc = NGp + (factorRoot ? 1 : 0);
        const int OS  = NGs + 2;
        {
            std::vector<std::string> comps{"acc_pair(avh, avl)"};
            for(int s = 0; s < NGp - 1; ++s)
                comps.push_back("acc_pair(agh" + std::to_string(s) + ", agl" + std::to_string(s) + ")");
            if(factorRoot)
                comps.push_back("acc_of(nv)");
            emitCtaReduce(os, comps, "    ");
        }
        if(asBody) {
            plan.fused_row[grad ? 1 : 0] = NGc + 1;
            // one-launch evaluation: each chunk's sums and status go straight to page-locked host memory (row
            // ch: [components..., status], each word one aligned 8-byte store); the host adds the rows in chunk
            // order as their words arrive, so no CTA waits on a completion counter and no finishing CTA runs
            const bool foldTab = tab && plan.conv_fold_q[0] >= 0;
            os << "    if(tid < " << NGc << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
               << "; ++w) t = acc_add(t, red[w][tid]); a.hpart[(i64)ch * " << NGc + 1 << " + tid] = acc_value(t); }\n";
            os << "    if(tid == 0) a.hpart[(i64)ch * " << NGc + 1 << " + " << NGc << "] = (double)(gf_q0 | (gf_g2 ? 8 : 0)"
               << (foldTab ? " | s_fbits" : "") << ");\n";
            os << "    __syncthreads();\n";
            os << "  }\n" << (countMode ? "  }\n" : "") << "}\n\n";
            endBody(asBody);
            return;
        }
        // chunk partials are component-major: part[comp][chunk], so that the finisher's loads are contiguous
        os << "    ACC *part = reinterpret_cast<ACC *>(a.partial);\n";
        os << "    if(tid < " << NGc << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
           << "; ++w) t = acc_add(t, red[w][tid]); part[(i64)tid * a.n_chunks + ch] = t; }\n";
        os << "    __threadfence();\n    __syncthreads();\n";
        os << "    if(tid == 0) { unsigned prev = atomicAdd(&a.counter[toy], 1u); last = (prev == "
              "(unsigned)((a.n_toys == 1 ? a.n_chunks : a.toy_nchunks[toy]) - 1)); }\n";
        os << "    __syncthreads();\n";
        // finishing CTA of the toy: one warp per component sums that component's chunk partials (contiguous,
        // independent loads) and reduces them across its lanes
        os << "    if(last) {\n";
        os << "      __threadfence();\n";
        os << "      const int c0 = a.n_toys == 1 ? 0 : a.toy_chunk0[toy], nc = a.n_toys == 1 ? a.n_chunks : a.toy_nchunks[toy];\n";
        os << "      double *o = a.out + (i64)toy * " << OS << ";\n";
        os << "      for(int comp = wid; comp < " << NGc << "; comp += " << NW << ") {\n";
        os << "        const ACC *pc = part + (i64)comp * a.n_chunks + c0;\n";
        os << "        ACC t = acc_zero();\n";
        os << "#pragma unroll 4\n        for(int c = lane; c < nc; c += 32) t = acc_add(t, pc[c]);\n";
        os << "        t = warp_acc2(t);\n";
        os << "        if(lane == 0) {\n";
        os << "          const double v = acc_value(t);\n";
        os << "          o[comp == 0 ? 0 : (comp == " << NGp << " && " << (factorRoot ? 1 : 0) << " ? " << 2 + T.NG
           << " : 1 + comp)] = v;\n";
        // a zero NLL is flagged here, or on the host after the factored normalisation is added
        os << "          if(comp == 0) { int st = a.qflag[toy]; " << (factorRoot ? "" : "if(v == 0.0) st |= 4; ")
           << "if(a.gbar && a.gbar[2]) st |= 8; o[1] = (double)st; a.counter[toy] = 0u; a.qflag[toy] = 0; }\n";
        os << "        }\n";
        os << "      }\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        os << "  }\n}\n\n";
        endBody(asBody);
    }

    // event columns the event pass streams (pointer expression, bytes per event), set by eventKernel
    std::vector<std::pair<std::string, int>> evtStreams;
    // dynamic shared memory of the last body eventKernel emitted
    size_t bodySmem = 0;
    // [nograd, grad]: the event function reads an observable column (set by the standalone event kernels)
    bool evtReadsObs[2] = {true, true};

    // ---------------- one launch per evaluation (one toy) ----------------
    // gf_fcn_*: a cooperative launch (every CTA resident) that runs the whole evaluation.  Each CTA first
    // copies its own event chunks into shared memory with bulk copies (or, when they do not fit, prefetches
    // them into L2), so that their HBM reads overlap the tables; then the convolution-table CTAs and the
    // numeric-grid CTAs of the separate kernels run as virtual blocks spread over the launch, a bounded grid
    // barrier follows (two when an unfolded numeric node reads a table), and the event pass runs over the same
    // CTAs, writing per-chunk sums to host memory.  Replaces three dependent launches and the finishing CTA
    // (GooPdf::calculateNLL's normalize + reduce, src/PDFs/GooPdf.cu:254-273) by one launch.
    void fusedKernel(bool grad) {
        const char *sfx = grad ? "g" : "n";
        const int NC = (int)T.convs.size(), NQ = (int)T.nums.size();
        bool hasGrid = false;
        for(int q = 0; q < NQ; ++q)
            hasGrid = hasGrid || !plan.num_folded[q];
        // the per-event terms depend on the event only through one convolution's bin offset: tabulate them
        // (at most 16 table rows per thread, held in registers)
        const bool tab = NC == 1 && T.n_amp_cols == 0 && !evtReadsObs[grad ? 1 : 0] && !tabDisabled() &&
                         (T.convs[0].nK + block - 1) / block <= 16;
        // with the tabulated terms every CTA sums the folded grid normalisation itself from the table CTAs'
        // partials: they skip the fold's completion counter and finishing CTA
        if(NC > 0)
            convKernel(grad, true, tab);
        if(hasGrid)
            gridKernel(grad, true);
        if(tab && !countDecl) {
            // the counting pass's results, shared by the fused kernel (which counts before the grid barrier) and
            // its event body (which multiplies the per-bin terms by the counts after it)
            os << "__shared__ int gf_rstart[" << kCountRows << "];\n";
            countDecl = true;
        }
        eventKernel(grad, false, true, tab);
        const size_t evtSmem = bodySmem;
        const int CB = plan.conv_blocks, MGB = plan.max_grid_blocks;
        // grid virtual blocks: only the unfolded numeric nodes' blocks, one node after another (a folded node's
        // block slots would only return, and could push a grid block onto a CTA that also builds a table)
        std::vector<std::pair<int, int>> gridNodes; // (numeric node, blocks)
        int nGridV = 0;
        for(int q = 0; q < NQ && hasGrid; ++q)
            if(!plan.num_folded[q] && plan.grid_blocks[q] > 0) {
                gridNodes.push_back({q, plan.grid_blocks[q]});
                nGridV += plan.grid_blocks[q];
            }
        const int nConvV = NC > 0 ? CB * NC : 0;
        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ", 2) gf_fcn_" << sfx
           << "(const GfArgs a) {\n";
        os << "  const int toy = 0; (void)toy;\n";
        // the toy's record (parameters, analytic factors), passed by value in the arguments (or, when too
        // large, read from page-locked host memory): one copy per CTA in shared memory, read by every phase
        const int npr = std::max(1, plan.nl.npr);
        os << "  __shared__ __align__(16) R sPr[" << npr << "];\n";
        os << "  for(int i = threadIdx.x; i < " << plan.nl.npr << "; i += blockDim.x)\n"
           << "    sPr[i] = a.rec_n ? reinterpret_cast<const R *>(a.rec)[i] : reinterpret_cast<const R *>(a.Pr)[i];\n";
        // the CTA's events (all its chunks, one contiguous range per stream): when they fit, one bulk copy per
        // stream into shared memory (the TMA unit, completion on an mbarrier) that runs while the tables are
        // built; otherwise a bulk prefetch into L2.  Chunk starts are multiples of 256 events (16-byte
        // aligned sources) and the streams are padded to 8 events, so 16-byte-rounded sizes stay in bounds.
        const int NS = (int)evtStreams.size();
        os << "  extern __shared__ __align__(16) unsigned char gf_dyn[];\n";
        os << "  __shared__ __align__(8) unsigned long long s_mbar;\n";
        os << "  __shared__ int s_soff[" << std::max(1, NS) << "];\n";
        os << "  __shared__ int s_staged;\n";
        os << "  const int cb = (int)(((i64)a.n_chunks * blockIdx.x) / gridDim.x);\n";
        os << "  const int ce = (int)(((i64)a.n_chunks * (blockIdx.x + 1)) / gridDim.x);\n";
        os << "  const i64 sb0 = (i64)cb * a.chunk;\n";
        os << "  if(threadIdx.x == 0) {\n";
        os << "    int staged = 0;\n";
        os << "    if(cb < ce) {\n";
        os << "      const i64 e0 = (i64)ce * a.chunk < a.nevt0 ? (i64)ce * a.chunk : a.nevt0;\n";
        os << "      unsigned nb[" << std::max(1, NS) << "], tot = 0;\n";
        for(int i = 0; i < NS; ++i)
            os << "      nb[" << i << "] = (unsigned)(((e0 - sb0) * " << evtStreams[i].second << " + 15) & ~15LL); s_soff["
               << i << "] = (int)tot; tot += nb[" << i << "];\n";
        os << "      if(a.stage_cap > 0u && tot <= a.stage_cap) {\n";
        os << "        const unsigned mb = (unsigned)__cvta_generic_to_shared(&s_mbar);\n";
        os << "        asm volatile(\"mbarrier.init.shared::cta.b64 [%0], 1;\" :: \"r\"(mb) : \"memory\");\n";
        os << "        asm volatile(\"fence.mbarrier_init.release.cluster;\" ::: \"memory\");\n";
        os << "        asm volatile(\"mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\" :: \"r\"(mb), \"r\"(tot) : \"memory\");\n";
        os << "        const unsigned sd = (unsigned)__cvta_generic_to_shared(gf_dyn + a.stage_off);\n";
        for(int i = 0; i < NS; ++i)
            os << "        asm volatile(\"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\" :: "
                  "\"r\"(sd + (unsigned)s_soff[" << i << "]), \"l\"(reinterpret_cast<const char *>(" << evtStreams[i].first
               << ") + sb0 * " << evtStreams[i].second << "), \"r\"(nb[" << i << "]), \"r\"(mb) : \"memory\");\n";
        os << "        staged = 1;\n";
        os << "      } else {\n";
        for(int i = 0; i < NS; ++i)
            os << "        asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], %1;\" :: \"l\"(reinterpret_cast<const char *>("
               << evtStreams[i].first << ") + sb0 * " << evtStreams[i].second << "), \"r\"(nb[" << i << "]) : \"memory\");\n";
        os << "      }\n";
        os << "    }\n";
        os << "    s_staged = staged;\n";
        os << "  }\n";
        os << "  __syncthreads();\n";
        if(tab)
            // the counting pass's run starts (written after the grid barrier, whose own barrier orders this)
            os << "  for(int r = threadIdx.x; r < " << kCountRows << "; r += blockDim.x) gf_rstart[r] = -1;\n";
        // a CTA that leaves early still waits (bounded) for its own bulk copy, so that no copy writes the shared
        // memory of a finished CTA
        auto barrier = [&]() {
            os << "  if(!gf_grid_sync(a.gbar, a.bar_target, a.bar_ns)) {\n";
            os << "    if(s_staged) gf_mbar_wait(&s_mbar, 0u, 1000000000ull);\n";
            os << "    return;\n  }\n";
        };
        auto convLoop = [&]() {
            os << "  for(unsigned vb = blockIdx.x; vb < " << nConvV << "u; vb += gridDim.x) {\n";
            os << "    gf_conv_" << sfx << "_body(a, make_uint3(vb % " << CB << "u, 0u, vb / " << CB << "u), make_uint3("
               << CB << "u, 1u, " << NC << "u), sPr);\n";
            os << "    __syncthreads();\n  }\n";
        };
        auto gridLoop = [&](bool shifted) {
            // grid virtual blocks after the table ones (same phase) or from block 0 (a phase of their own)
            os << "  for(unsigned vb = blockIdx.x; vb < " << (shifted ? nConvV : 0) + nGridV << "u; vb += gridDim.x) {\n";
            if(shifted)
                os << "    if(vb < " << nConvV << "u) gf_conv_" << sfx << "_body(a, make_uint3(vb % " << CB
                   << "u, 0u, vb / " << CB << "u), make_uint3(" << CB << "u, 1u, " << NC << "u), sPr);\n    else {\n"
                   << "      const unsigned g = vb - " << nConvV << "u;\n";
            else
                os << "    {\n      const unsigned g = vb;\n";
            os << "      unsigned gb = g, gq = " << (gridNodes.empty() ? 0 : gridNodes[0].first) << "u;\n";
            for(size_t i = 1; i < gridNodes.size(); ++i) {
                int before = 0;
                for(size_t j = 0; j < i; ++j)
                    before += gridNodes[j].second;
                os << "      if(g >= " << before << "u) { gb = g - " << before << "u; gq = " << gridNodes[i].first << "u; }\n";
            }
            os << "      gf_grid_" << sfx << "_body(a, make_uint3(gb, 0u, gq), make_uint3(" << MGB << "u, 1u, " << NQ
               << "u), sPr);\n    }\n";
            os << "    __syncthreads();\n  }\n";
        };
        if(NC > 0 && hasGrid && !plan.grid_needs_conv)
            gridLoop(true); // tables and grids in one phase
        else {
            if(NC > 0)
                convLoop();
            if(NC > 0 && hasGrid)
                barrier();
            if(hasGrid)
                gridLoop(false);
        }
        // no tables and no grids (analytic or amplitude normalisations): the event pass needs no barrier
        if(NC > 0 || hasGrid)
            barrier();
        os << "  gf_evt_" << sfx << "_body(a, blockIdx, gridDim, sPr, s_staged ? gf_dyn + a.stage_off : nullptr, s_soff, sb0, "
              "&s_mbar);\n";
        os << "}\n\n";
        plan.fused     = true;
        plan.fused_tab = plan.fused_tab || tab;
        const size_t work = std::max(grad ? plan.conv_smem_grad : plan.conv_smem_nograd, evtSmem);
        const size_t soff = (work + 127) / 128 * 128;
        // two resident CTAs per SM (228 KB of shared memory per SM, 1 KB of it reserved per CTA, a few KB of
        // static arrays): the staged events get what is left of 109 KB, at most 64 KB. 64 bytes of slack follow
        // the staging area: the event loop's last iteration reads whole 8-event (2-event) groups, up to 56 bytes
        // past a stream's last staged event, and those reads must stay inside the CTA's shared memory
        const size_t budget = 109 * 1024, slack = 64;
        const size_t cap    = soff + slack < budget ? std::min<size_t>(64 * 1024, (budget - soff - slack) / 16 * 16) : 0;
        plan.fused_stage_off[grad ? 1 : 0] = soff;
        plan.fused_stage_cap[grad ? 1 : 0] = cap;
        plan.fused_smem[grad ? 1 : 0]      = soff + cap + slack;
    }
};

} // namespace

NormLayout norm_layout(const Tree &t) { return computeNormLayout(t); }

KernelPlan generate_kernels(const Tree &t, bool mixed, int evt_block, bool batch, const Shapes &shapes) {
    KernelPlan plan;
    plan.nl                  = norm_layout(t);
    // one toy: 256 bins per CTA (C2's 10,000-bin grids: FCN 36.7 us; 1024 / 2048 / 4096 / 16384 bins per
    // CTA: 36.2 / 38.1 / 43.6 / 46.7 us, fewer CTAs leaving more of the per-bin load latency exposed)
    plan.grid_bins_per_block = shapes.grid_bpb > 0 ? shapes.grid_bpb : batch ? 1024 : 256;
    Gen g{t, mixed, evt_block, batch, plan, {}};
    g.shapes = shapes;
    g.os << "// generated likelihood kernels\n";
    if(mixed)
        g.os << "typedef float R;\ntypedef float2 R2;\n#define GF_EXP(x) expf(x)\n#define GF_LOG(x) logf(x)\n";
    else
        g.os << "typedef double R;\ntypedef double2 R2;\n#define GF_EXP(x) exp(x)\n#define GF_LOG(x) log(x)\n";
    g.os << kPrelude;
    if(t.n_amp_nodes() > 0)
        g.os << kPreludeDual;
    if(!t.amp3s.empty())
        g.os << kPreludeAmp << kPreludeAmp3T;
    if(!t.amp4s.empty()) {
        g.os << kPreludeAmp4 << kPreludeAmp4T
             << "__device__ __forceinline__ double2 gf_lineshape(bool sbw, double Mpair, double m1, double m2, double mass,\n"
                "    double width, int orbital, int FF, double radius) {\n"
                "  double re, im;\n"
                "  gf_lineshape_t<double>(sbw, Mpair, m1, m2, mass, width, orbital, FF, radius, re, im);\n"
                "  return make_double2(re, im);\n}\n";
        if(mixed)
            g.os << kPreludeAmp4F;
    }
    if(mixed)
        g.os << kPreludeF32 << dfLogTable() << kPreludeDF;
    else
        g.os << kPreludeF64;
    for(int k = 0; k < t.n_amp_nodes(); ++k)
        if(g.nDeriv(k) > 0)
            g.recomputeKernels = true;
    g.tableLayout(true);
    g.tableLayout(false);
    g.planNumerics();
    g.convKernel(true);
    g.convKernel(false);
    g.gridKernel(true);
    g.gridKernel(false);
    g.ampKernels();
    g.eventKernel(true, false);
    g.eventKernel(false, false);
    g.eventKernel(false, true);
    if(g.recomputeKernels) {
        // the recompute-mode gradient pass; the plan keeps the store-mode kernels' figures
        const KernelPlan saved = plan;
        const size_t bs        = g.bodySmem;
        const bool ro          = g.evtReadsObs[1];
        g.recompute            = true;
        g.eventKernel(true, false);
        g.recompute            = false;
        g.evtReadsObs[1]       = ro;
        const size_t smem      = plan.evt_smem_grad;
        plan                   = saved;
        plan.evt_smem_gr       = smem;
        plan.recompute_kernels = true;
        g.bodySmem             = bs;
    }
    if(!batch && t.fit_metric == GF_FIT_UNBINNED_NLL) {
        g.fusedKernel(true);
        g.fusedKernel(false);
    }
    plan.source = g.os.str();
    return plan;
}

} // namespace gf
