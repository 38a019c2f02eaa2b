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
        os << "    const R " << v << " = GF_EXP(R(-0.5) * " << d << " * " << d << " / (" << s << " * " << s
           << "));\n";
        out.v = v;
        gadd(c, out, slot(c, n.params[0]), v + " * " + d + " / (" + s + " * " + s + ")");
        gadd(c, out, slot(c, n.params[1]), v + " * " + d + " * " + d + " / (" + s + " * " + s + " * " + s + ")");
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
        for(size_t k = 0; k < ch.size(); ++k) {
            std::string ne = normExpr(c, n.children[k]);
            u.push_back(ne.empty() ? ch[k].v : "(" + ch[k].v + " * " + ne + ")");
        }
        os << "    R " << v << " = R(0);\n";
        size_t nw = ext ? ch.size() : ch.size() - 1;
        for(size_t k = 0; k < nw; ++k) {
            std::string ne = normExpr(c, n.children[k]);
            os << "    " << v << " += (" << P(n.params[k]) << " * " << ch[k].v << ")"
               << (ne.empty() ? "" : " * " + ne) << ";\n";
        }
        if(!ext) {
            std::string ne = normExpr(c, n.children.back());
            os << "    " << v << " += ((R(1) - " << tw << ") * " << ch.back().v << ")"
               << (ne.empty() ? "" : " * " + ne) << ";\n";
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
            std::string ne = normExpr(c, n.children[k]), un = c.tmp("u");
            os << "    const R " << un << " = " << ch[k].v << (ne.empty() ? "" : " * " + ne) << ";\n";
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
    int n_chunks;
    int n_toys;
    int metric;
    int pad;
};

__device__ __forceinline__ double gf_warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Programmatic dependent launch: let the next kernel of the evaluation start its independent prologue,
// and wait for the previous kernel's results (both are no-ops without a programmatic dependency).
__device__ __forceinline__ void gf_pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void gf_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

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
__device__ __forceinline__ double acc_value(ACC a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float acc_r(ACC a) { return a.x + a.y; }
#define GF_CENTRE(lo, w, b) ((float)(lo) + (float)(w) * ((float)(b) + 0.5f))
)CUDA";

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
__device__ __forceinline__ ACC acc_add(ACC a, ACC b) { return a + b; }
__device__ __forceinline__ ACC warp_acc(double v) { return gf_warp_sum(v); }
__device__ __forceinline__ ACC warp_acc2(ACC a) { return gf_warp_sum(a); }
__device__ __forceinline__ double acc_value(ACC a) { return a; }
__device__ __forceinline__ double acc_r(ACC a) { return a; }
#define GF_CENTRE(lo, w, b) gf_centre(lo, w, b)
)CUDA";

// Where every normalisation factor is kept (see NormLayout in tree.h).
NormLayout computeNormLayout(const Tree &T) {
    NormLayout nl;
    nl.npr = T.n_params;
    for(size_t i = 0; i < T.nodes.size(); ++i) {
        if(T.nk[i] != NK_EXP && T.nk[i] != NK_GAUSS)
            continue;
        NormLayout::Analytic a;
        a.node  = (int)i;
        a.kind  = T.nk[i];
        a.slotN = nl.npr++;
        for(int s : T.dep_norm[i])
            a.dN.push_back({s, nl.npr++});
        nl.analytic.push_back(a);
    }
    nl.qN.assign(T.nums.size(), -1);
    nl.qdN.assign(T.nums.size(), {});
    for(size_t q = 0; q < T.nums.size(); ++q) {
        int i    = T.nums[q].node;
        nl.qN[q] = nl.nq++;
        for(int s : T.dep_norm[i])
            nl.qdN[q].push_back({s, nl.nq++});
    }
    return nl;
}

// Parameters (type R) of the toy from its record.
void emitParamsR(std::ostream &os, const Tree &T, const NormLayout &nl, const char *ind) {
    os << ind << "const R *Pr = reinterpret_cast<const R *>(a.Pr) + (i64)toy * " << nl.npr << "; (void)Pr;\n";
    for(int j = 0; j < T.n_params; ++j)
        os << ind << "const R p" << j << " = Pr[" << j << "]; (void)p" << j << ";\n";
}

// Normalisation factors used by the event pass: analytic ones from the record, numeric ones from Nq.
void emitNormReads(std::ostream &os, const Tree &T, bool grad, const NormLayout &nl, const char *ind) {
    if(nl.nq > 0)
        os << ind << "const R *Nq = reinterpret_cast<const R *>(a.Nq) + (i64)toy * " << nl.nq << ";\n";
    for(auto &an : nl.analytic) {
        os << ind << "const R N" << an.node << " = Pr[" << an.slotN << "];\n";
        if(grad)
            for(auto &d : an.dN)
                os << ind << "const R dN" << an.node << "_" << d.first << " = Pr[" << d.second << "];\n";
    }
    for(size_t q = 0; q < T.nums.size(); ++q) {
        int i = T.nums[q].node;
        os << ind << "const R N" << i << " = Nq[" << nl.qN[q] << "];\n";
        if(grad)
            for(auto &d : nl.qdN[q])
                os << ind << "const R dN" << i << "_" << d.first << " = Nq[" << d.second << "];\n";
    }
}

int padComps(int c) { return c <= 1 ? 1 : c <= 2 ? 2 : (c + 3) / 4 * 4; }

struct Gen {
    const Tree &T;
    bool mixed;
    int block, chunk;
    KernelPlan &plan;
    std::ostringstream os;

    int convComps(int ci, bool grad) const { return 1 + (grad ? (int)T.convs[ci].dep.size() : 0); }

    // Table layout per toy: for each conv, AoS [k][cp] with cp = padded component count (16-byte rows).
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
        (grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd) = total;
    }

    // ---------------- convolution tables ----------------
    // T_c[k] = sum_m A_c[m] B_c[m + off - k] for k in [kmin, kmax].  One CTA covers KB consecutive k; a
    // thread owns KT consecutive k of one component over a contiguous slice of m (MS slices per k-tile),
    // keeping a sliding window of the resolution values in registers (KT FMAs per two shared loads).
    // The MS lane partials are combined with a compensated (two-sum) shuffle reduction.
    void convKernel(bool grad) {
        const char *sfx = grad ? "g" : "n";
        const int NC    = (int)T.convs.size();
        if(NC == 0)
            return;
        const int MS = 8, KT = 8;
        const int items = block / MS;
        auto &off       = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps       = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const int64_t total = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        size_t smem   = 0;
        int maxBlocks = 0;
        std::vector<int> KBs;
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            int comps          = convComps(ci, grad);
            if(comps > items)
                throw std::runtime_error("codegen: too many convolution derivative components");
            int ktiles = items / comps;
            int KB     = KT * ktiles;
            KBs.push_back(KB);
            int mcomp = 1 + (grad ? (int)T.dep_val[cv.model].size() : 0);
            int rcomp = 1 + (grad ? (int)T.dep_val[cv.resol].size() : 0);
            size_t sm = (size_t)(mcomp * cv.nM + rcomp * (cv.nM + KB)) * (mixed ? 4 : 8);
            smem      = std::max(smem, sm);
            maxBlocks = std::max(maxBlocks, (cv.nK + KB - 1) / KB);
        }
        (grad ? plan.conv_smem_grad : plan.conv_smem_nograd) = smem;
        plan.conv_blocks = std::max(plan.conv_blocks, maxBlocks);

        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") gf_conv_" << sfx
           << "(const GfArgs a) {\n";
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *sm = reinterpret_cast<R *>(smraw);\n";
        os << "  const int toy = blockIdx.y; const int ci = blockIdx.z; const int tid = threadIdx.x;\n";
        os << "  gf_pdl_trigger();\n";
        os << "  if(a.active && !a.active[toy]) return;\n";
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
            os << "  case " << ci << ": {\n";
            os << "    const int k0 = " << cv.kmin << " + (int)blockIdx.x * " << KB << ";\n";
            os << "    if(k0 > " << cv.kmax << ") return;\n";
            os << "    R *sM = sm; R *sR = sm + " << mcomp * cv.nM << ";\n";
            os << "    const int rbase = " << cv.offset << " - (k0 + " << KB - 1 << ");\n";
            const double wM = (cv.ic[1] - cv.ic[0]) / cv.nM, wR = (cv.ic[4] - cv.ic[3]) / cv.nR;
            for(int pass = 0; pass < 2; ++pass) {
                bool model = pass == 0;
                int sub    = model ? cv.model : cv.resol;
                const auto &dd = model ? dm : dr;
                int len        = model ? cv.nM : W1;
                if(model)
                    os << "    for(int m = tid; m < " << cv.nM << "; m += " << block << ") {\n"
                       << "      const R wx = (R)GF_CENTRE(" << lit(cv.ic[0]) << ", " << lit(wM) << ", m);\n";
                else
                    os << "    for(int w = tid; w < " << W1 << "; w += " << block << ") {\n"
                       << "      const int r = rbase + w;\n"
                       << "      if(r < 0 || r >= " << cv.nR << ") {\n"
                       << "        for(int c = 0; c < " << 1 + (grad ? (int)dr.size() : 0) << "; ++c) sR[c * " << W1
                       << " + w] = R(0);\n"
                       << "        continue;\n      }\n"
                       << "      const R wx = (R)GF_CENTRE(" << lit(cv.ic[3]) << ", " << lit(wR) << ", r);\n";
                std::ostringstream body;
                Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
                c.x   = [&](int) { return std::string("wx"); };
                c.k   = [&](int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.tab = [&](int, int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.uid = model ? 0 : 1000;
                Val v = emit(c, sub);
                std::string idx = model ? "m" : "w";
                os << "      {\n" << body.str();
                os << "      " << (model ? "sM" : "sR") << "[" << idx << "] = " << v.v << ";\n";
                if(grad)
                    for(size_t j = 0; j < dd.size(); ++j) {
                        auto it = v.g.find(dd[j]);
                        os << "      " << (model ? "sM" : "sR") << "[" << (1 + j) * len << " + " << idx << "] = "
                           << (it == v.g.end() ? std::string("R(0)") : it->second) << ";\n";
                    }
                os << "      }\n    }\n";
            }
            os << "    __syncthreads();\n";
            os << "    const int ms = tid % " << MS << ", item = tid / " << MS << ", comp = item % " << comps
               << ", kt = item / " << comps << ";\n";
            os << "    const bool live = kt < " << ktiles << ";\n";
            os << "    const int kt0 = k0 + kt * " << KT << ";\n";
            os << "    const int c0 = " << KB - 1 << " - kt * " << KT << ";\n";
            os << "    const int mlo = (" << cv.nM << " * ms) / " << MS << ", mhi = (" << cv.nM << " * (ms + 1)) / " << MS
               << ";\n";
            os << "    R acc[" << KT << "], cmp[" << KT << "];\n#pragma unroll\n    for(int j = 0; j < " << KT
               << "; ++j) { acc[j] = R(0); cmp[j] = R(0); }\n";
            os << "    if(live) {\n";
            os << "      const R *mA[2] = {nullptr, nullptr}; const R *rA[2] = {nullptr, nullptr};\n";
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
                        os << "mA[" << t << "] = sM + " << (1 + (im - dm.begin())) * cv.nM << "; rA[" << t << "] = sR; ";
                        ++t;
                    }
                    if(ir != dr.end()) {
                        os << "mA[" << t << "] = sM; rA[" << t << "] = sR + " << (1 + (ir - dr.begin())) * W1 << "; ";
                        ++t;
                    }
                    os << "break;\n";
                }
            os << "      default: break;\n      }\n";
            os << "      for(int t = 0; t < 2; ++t) {\n";
            os << "        if(!mA[t]) break;\n";
            os << "        const R *M = mA[t]; const R *Rw = rA[t] + c0;\n";
            os << "        R rv[" << KT << "];\n#pragma unroll\n        for(int j = 0; j < " << KT
               << "; ++j) rv[j] = Rw[mlo - j];\n";
            // blocks of 8 products are summed plainly, blocks are added with a two-sum correction (mixed)
            os << "        for(int mb = mlo; mb < mhi; mb += 8) {\n";
            os << "          R bs[" << KT << "];\n#pragma unroll\n          for(int j = 0; j < " << KT << "; ++j) bs[j] = R(0);\n";
            os << "          const int me = min(mb + 8, mhi);\n";
            os << "          for(int m = mb; m < me; ++m) {\n";
            os << "            const R mv = M[m];\n";
            os << "#pragma unroll\n            for(int j = 0; j < " << KT << "; ++j) bs[j] = fma(mv, rv[j], bs[j]);\n";
            os << "#pragma unroll\n            for(int j = " << KT - 1 << "; j > 0; --j) rv[j] = rv[j - 1];\n";
            os << "            rv[0] = Rw[m + 1];\n";
            os << "          }\n";
            os << "#pragma unroll\n          for(int j = 0; j < " << KT << "; ++j) gf_comp_add(acc[j], cmp[j], bs[j]);\n";
            os << "        }\n      }\n    }\n";
            os << "#pragma unroll\n    for(int j = 0; j < " << KT << "; ++j) acc[j] += cmp[j];\n";
            os << "#pragma unroll\n    for(int j = 0; j < " << KT << "; ++j) {\n";
            os << "      const R t = gf_group_sum(acc[j], " << MS << ");\n";
            os << "      const int k = kt0 + j;\n";
            os << "      if(live && ms == 0 && k <= " << cv.kmax << ") ctab[" << off[ci] << " + (k - " << cv.kmin << ") * "
               << cp << " + comp] = t;\n";
            os << "    }\n";
            os << "    break; }\n";
        }
        os << "  }\n}\n\n";
    }

    // ---------------- numeric grids ----------------
    // One CTA row per numeric node; the finishing CTA of a (toy, node) turns the grid sum into the node's
    // normalisation factor and its derivatives (GooPdf::normalize numeric branch,
    // src/PDFs/GooPdf.cu:366-395) and stores them for the event pass.
    void gridKernel(bool grad) {
        const char *sfx = grad ? "g" : "n";
        const int NQ    = (int)T.nums.size();
        if(NQ == 0)
            return;
        const int NGp = 1 + (grad ? T.NG : 0); // components reduced
        const int NGs = 1 + T.NG;              // buffer stride
        const int BPB = plan.grid_bins_per_block;
        const int NW  = block / 32;
        plan.grid_blocks.clear();
        plan.max_grid_blocks = 0;
        for(auto &g : T.nums) {
            int nb = (int)((g.total + BPB - 1) / BPB);
            plan.grid_blocks.push_back(nb);
            plan.max_grid_blocks = std::max(plan.max_grid_blocks, nb);
        }
        const int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        auto &off               = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps               = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const NormLayout &nl    = plan.nl;
        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") gf_grid_" << sfx
           << "(const GfArgs a) {\n";
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
            os << "  case " << q << ": {\n";
            os << "    nblk = " << plan.grid_blocks[q] << ";\n";
            os << "    if((int)blockIdx.x >= nblk) return;\n";
            os << "    const i64 bend = min((i64)" << g.total << "LL, (i64)(blockIdx.x + 1) * " << BPB << ");\n";
            os << "    for(i64 b = (i64)blockIdx.x * " << BPB << " + tid; b < bend; b += " << block << ") {\n";
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
        os << "  { const ACC t = warp_acc(av); if(lane == 0) red[wid][0] = t; }\n";
        for(int s = 0; s < NGp - 1; ++s)
            os << "  { const ACC t = warp_acc(ag" << s << "); if(lane == 0) red[wid][" << 1 + s << "] = t; }\n";
        os << "  __syncthreads();\n";
        os << "  ACC *gp = reinterpret_cast<ACC *>(a.gpartial) + (((i64)toy * " << NQ << " + q) * " << plan.max_grid_blocks
           << " + blockIdx.x) * " << NGs << ";\n";
        os << "  if(tid < " << NGp << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
           << "; ++w) t = acc_add(t, red[w][tid]); gp[tid] = t; }\n";
        os << "  __threadfence();\n  __syncthreads();\n";
        os << "  if(tid == 0) { unsigned prev = atomicAdd(&a.gcounter[toy * " << NQ
           << " + q], 1u); last = (prev == (unsigned)(nblk - 1)); }\n";
        os << "  __syncthreads();\n";
        os << "  if(!last) return;\n";
        os << "  __threadfence();\n";
        os << "  const ACC *g0 = reinterpret_cast<const ACC *>(a.gpartial) + ((i64)toy * " << NQ << " + q) * "
           << plan.max_grid_blocks << " * " << NGs << ";\n";
        os << "  {\n";
        os << "    ACC s[" << NGp << "];\n";
        os << "#pragma unroll\n    for(int comp = 0; comp < " << NGp << "; ++comp) s[comp] = acc_zero();\n";
        os << "    for(int bi = tid; bi < nblk; bi += " << block << ") {\n";
        os << "#pragma unroll\n      for(int comp = 0; comp < " << NGp << "; ++comp) s[comp] = acc_add(s[comp], g0[bi * " << NGs << " + comp]);\n";
        os << "    }\n";
        os << "#pragma unroll\n    for(int comp = 0; comp < " << NGp << "; ++comp) { const ACC t = warp_acc2(s[comp]); if(lane == 0) red[wid][comp] = t; }\n";
        os << "  }\n";
        os << "  __syncthreads();\n";
        os << "  if(tid < " << NGp << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW << "; ++w) t = acc_add(t, red[w][tid]); tot[tid] = t; }\n";
        os << "  __syncthreads();\n";
        os << "  if(tid == 0) {\n";
        os << "    a.gcounter[toy * " << NQ << " + q] = 0u;\n";
        os << "    R *Nq = reinterpret_cast<R *>(a.Nq) + (i64)toy * " << nl.nq << ";\n";
        os << "    const double S = acc_value(tot[0]);\n";
        os << "    a.gsum[(i64)toy * " << NQ << " + q] = S;\n";
        os << "    if(isnan(S)) atomicOr(&a.qflag[toy], 1); else if(!(S > 0.0)) atomicOr(&a.qflag[toy], 2);\n";
        os << "    switch(q) {\n";
        for(int q = 0; q < NQ; ++q) {
            const NumInfo &g = T.nums[q];
            // ((1 * volume) / bins), the reference's order of operations, evaluated on the host
            double c = 1.0;
            c *= g.volume;
            c /= (double)g.total;
            os << "    case " << q << ": {\n";
            os << "      const double I = " << lit(c) << " * S;\n";
            if(mixed)
                os << "      const R N = 1.0f / (float)I;\n";
            else
                os << "      const R N = 1.0 / I;\n";
            os << "      Nq[" << nl.qN[q] << "] = N;\n";
            if(grad)
                for(auto &d : nl.qdN[q])
                    os << "      Nq[" << d.second << "] = -N * N * (R)" << lit(c) << " * (R)acc_r(tot[" << 1 + d.first
                       << "]);\n";
            os << "      break; }\n";
        }
        os << "    }\n  }\n}\n\n";
    }

    // ---------------- event pass ----------------
    // Persistent CTAs take contiguous ranges of the chunk list and stage a toy's conv tables once; each
    // thread streams 8 events per iteration with 16-byte loads.  Partial sums: FP32 per thread, then
    // compensated FP32 pairs across the warp, the CTA, the chunks of a toy; FP64 for the final value.
    void eventKernel(bool grad, bool values) {
        const std::string name = values ? "gf_val_n" : (grad ? "gf_evt_g" : "gf_evt_n");
        const int NGp = 1 + (grad ? T.NG : 0);
        const int NGs = 1 + T.NG;
        const int NC  = (int)T.convs.size();
        const int NO  = (int)T.obs.size();
        const int NW  = block / 32;
        const int VEC = 8;
        auto &off     = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        auto &cps     = grad ? plan.ctab_cp_grad : plan.ctab_cp_nograd;
        const int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        if(!values)
            (grad ? plan.evt_smem_grad : plan.evt_smem_nograd) = (size_t)ctabTotal * (mixed ? 4 : 8);

        std::vector<int> xused(NO, 0);
        std::ostringstream body;
        Ctx c{body, T, grad, true, nullptr, nullptr, nullptr, &xused};
        c.x = [&](int o) {
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
        Val root = emit(c, 0);
        if(!values && !grad) {
            plan.obs_used_evt.clear();
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    plan.obs_used_evt.push_back(o);
        }
        const std::string rootN = T.nk[0] == NK_ONE ? "" : "N0";

        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") " << name << "(const GfArgs a) {\n";
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *stab = reinterpret_cast<R *>(smraw); (void)stab;\n";
        os << "  __shared__ int s_toy, last;\n";
        if(!values)
            os << "  __shared__ ACC red[" << NW << "][" << NGp << "];\n";
        os << "  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5; (void)lane; (void)wid;\n";
        os << "  const int cb = (int)(((i64)a.n_chunks * blockIdx.x) / gridDim.x);\n";
        os << "  const int ce = (int)(((i64)a.n_chunks * (blockIdx.x + 1)) / gridDim.x);\n";
        os << "  if(tid == 0) s_toy = -1;\n";
        os << "  gf_pdl_trigger();\n";
        // event columns do not depend on the preceding kernels: pull the first chunk towards L2 meanwhile
        os << "  if(cb < ce) {\n";
        os << "    const i64 *cd = a.chunks + 3 * (i64)cb;\n";
        os << "    const int toy = (int)cd[0]; const i64 b0 = cd[1], e0 = cd[2];\n";
        os << "    if(!a.active || a.active[toy]) {\n";
        os << "      for(i64 i0 = b0 + " << VEC << " * (i64)tid; i0 < e0; i0 += " << VEC << " * " << block << ") {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "        asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(reinterpret_cast<const R *>(a.col[(i64)toy * "
                   << NO << " + " << o << "]) + i0));\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "        asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(a.kcol[(i64)toy * " << NC << " + " << ci
               << "] + i0));\n";
        os << "      }\n    }\n  }\n";
        os << "  gf_pdl_wait();\n";
        os << "  __syncthreads();\n";
        os << "  for(int ch = cb; ch < ce; ++ch) {\n";
        os << "    const i64 *cd = a.chunks + 3 * (i64)ch;\n";
        os << "    const int toy = (int)cd[0]; const i64 b0 = cd[1], e0 = cd[2];\n";
        os << "    if(a.active && !a.active[toy]) continue;\n";
        if(NC > 0) {
            os << "    if(toy != s_toy) {\n";
            os << "      __syncthreads();\n";
            if(mixed)
                os << "      { const float4 *src = reinterpret_cast<const float4 *>(reinterpret_cast<const R *>(a.ctab) + "
                      "(i64)toy * "
                   << ctabTotal << "); float4 *dst = reinterpret_cast<float4 *>(stab);\n"
                   << "        for(int i = tid; i < " << ctabTotal / 4 << "; i += " << block << ") dst[i] = src[i]; }\n";
            else
                os << "      { const double2 *src = reinterpret_cast<const double2 *>(reinterpret_cast<const R *>(a.ctab) "
                      "+ (i64)toy * "
                   << ctabTotal << "); double2 *dst = reinterpret_cast<double2 *>(stab);\n"
                   << "        for(int i = tid; i < " << ctabTotal / 2 << "; i += " << block << ") dst[i] = src[i]; }\n";
            os << "      if(tid == 0) s_toy = toy;\n";
            os << "      __syncthreads();\n";
            os << "    }\n";
        }
        emitParamsR(os, T, plan.nl, "    ");
        emitNormReads(os, T, grad, plan.nl, "    ");
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "    const R *col" << o << " = reinterpret_cast<const R *>(a.col[(i64)toy * " << NO << " + " << o
                   << "]);\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "    const int *kc" << ci << " = a.kcol[(i64)toy * " << NC << " + " << ci << "];\n";
        if(!values) {
            os << "    R av = R(0);\n";
            for(int s = 0; s < NGp - 1; ++s)
                os << "    R ag" << s << " = R(0);\n";
        }
        os << "    for(i64 i0 = b0 + " << VEC << " * (i64)tid; i0 < e0; i0 += " << VEC << " * " << block << ") {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o]) {
                if(mixed)
                    os << "      const float4 xv" << o << "a = *reinterpret_cast<const float4 *>(col" << o
                       << " + i0), xv" << o << "b = *reinterpret_cast<const float4 *>(col" << o << " + i0 + 4);\n"
                       << "      const R xa" << o << "[8] = {xv" << o << "a.x, xv" << o << "a.y, xv" << o << "a.z, xv" << o
                       << "a.w, xv" << o << "b.x, xv" << o << "b.y, xv" << o << "b.z, xv" << o << "b.w};\n";
                else {
                    os << "      R xa" << o << "[8];\n";
                    os << "#pragma unroll\n      for(int h = 0; h < 4; ++h) { const double2 t = "
                          "*reinterpret_cast<const double2 *>(col"
                       << o << " + i0 + 2 * h); xa" << o << "[2 * h] = t.x; xa" << o << "[2 * h + 1] = t.y; }\n";
                }
            }
        for(int ci = 0; ci < NC; ++ci)
            os << "      const int4 kv" << ci << "a = *reinterpret_cast<const int4 *>(kc" << ci << " + i0), kv" << ci
               << "b = *reinterpret_cast<const int4 *>(kc" << ci << " + i0 + 4);\n"
               << "      const int ka" << ci << "[8] = {kv" << ci << "a.x, kv" << ci << "a.y, kv" << ci << "a.z, kv" << ci
               << "a.w, kv" << ci << "b.x, kv" << ci << "b.y, kv" << ci << "b.z, kv" << ci << "b.w};\n";
        os << "#pragma unroll\n      for(int j = 0; j < " << VEC << "; ++j) {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "        const R ex" << o << " = xa" << o << "[j];\n";
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            int cp             = cps[ci];
            os << "        const int ek" << ci << " = ka" << ci << "[j];\n";
            os << "        const R *tp" << ci << " = stab + " << off[ci] << " + (ek" << ci << " - " << cv.kmin << ") * "
               << cp << "; (void)tp" << ci << ";\n";
            if(mixed) {
                if(cp == 1)
                    os << "        const float tq" << ci << " = tp" << ci << "[0];\n";
                else if(cp == 2)
                    os << "        const float2 tq" << ci << " = *reinterpret_cast<const float2 *>(tp" << ci << ");\n";
                else
                    for(int g4 = 0; g4 < cp / 4; ++g4)
                        os << "        const float4 tq" << ci << "_" << g4 << " = *reinterpret_cast<const float4 *>(tp"
                           << ci << " + " << 4 * g4 << ");\n";
            }
        }
        os << "        {\n" << body.str();
        os << "        const R pv = " << root.v << (rootN.empty() ? "" : " * " + rootN) << ";\n";
        if(values) {
            os << "        if(i0 + j < e0) {\n";
            os << "          double r;\n";
            os << "          if(a.metric == 0) r = (double)" << root.v << ";\n";
            os << "          else if(a.metric == 2) r = (double)pv;\n";
            os << "          else r = pv > R(0) ? -(double)GF_LOG(pv) : 0.0;\n";
            os << "          a.vals[i0 + j] = r;\n        }\n";
        } else {
            os << "        if(i0 + j < e0 && pv > R(0)) {\n";
            os << "          av -= GF_LOG(pv);\n";
            if(grad && T.NG > 0) {
                os << "          const R inv = R(1) / pv;\n";
                for(int s = 0; s < T.NG; ++s) {
                    std::string e;
                    auto it = root.g.find(s);
                    if(it != root.g.end())
                        e = rootN.empty() ? it->second : it->second + " * " + rootN;
                    std::string dn = T.nk[0] == NK_ONE ? "" : dnormExpr(c, 0, s);
                    if(!dn.empty())
                        e += (e.empty() ? "" : " + ") + root.v + " * " + dn;
                    if(!e.empty())
                        os << "          ag" << s << " -= (" << e << ") * inv;\n";
                }
            }
            os << "        }\n";
        }
        os << "        }\n      }\n    }\n";
        if(values) {
            os << "  }\n}\n\n";
            return;
        }
        os << "    { const ACC t = warp_acc(av); if(lane == 0) red[wid][0] = t; }\n";
        for(int s = 0; s < NGp - 1; ++s)
            os << "    { const ACC t = warp_acc(ag" << s << "); if(lane == 0) red[wid][" << 1 + s << "] = t; }\n";
        os << "    __syncthreads();\n";
        os << "    ACC *part = reinterpret_cast<ACC *>(a.partial);\n";
        os << "    if(tid < " << NGp << ") { ACC t = acc_zero(); for(int w = 0; w < " << NW
           << "; ++w) t = acc_add(t, red[w][tid]); part[(i64)ch * " << NGs << " + tid] = t; }\n";
        os << "    __threadfence();\n    __syncthreads();\n";
        os << "    if(tid == 0) { unsigned prev = atomicAdd(&a.counter[toy], 1u); last = (prev == "
              "(unsigned)(a.toy_nchunks[toy] - 1)); }\n";
        os << "    __syncthreads();\n";
        // finishing CTA of the toy: every thread loads a strided share of the chunk partials (independent
        // loads), then a warp and a CTA reduction of the compensated pairs
        os << "    if(last) {\n";
        os << "      __threadfence();\n";
        os << "      const int c0 = a.toy_chunk0[toy], nc = a.toy_nchunks[toy];\n";
        os << "      ACC s[" << NGp << "];\n";
        os << "#pragma unroll\n      for(int comp = 0; comp < " << NGp << "; ++comp) s[comp] = acc_zero();\n";
        os << "#pragma unroll 4\n      for(int c = tid; c < nc; c += " << block << ") {\n";
        os << "        const ACC *pc = part + (i64)(c0 + c) * " << NGs << ";\n";
        os << "#pragma unroll\n        for(int comp = 0; comp < " << NGp << "; ++comp) s[comp] = acc_add(s[comp], pc[comp]);\n";
        os << "      }\n";
        os << "#pragma unroll\n      for(int comp = 0; comp < " << NGp << "; ++comp) { const ACC t = warp_acc2(s[comp]); if(lane == 0) red[wid][comp] = t; }\n";
        os << "      __syncthreads();\n";
        os << "      if(tid < " << NGp << ") {\n";
        os << "        ACC t = acc_zero(); for(int w = 0; w < " << NW << "; ++w) t = acc_add(t, red[w][tid]);\n";
        os << "        double *o = a.out + (i64)toy * " << NGs + 1 << ";\n";
        os << "        const double v = acc_value(t);\n";
        os << "        o[tid == 0 ? 0 : 1 + tid] = v;\n";
        os << "        if(tid == 0) { int st = a.qflag[toy]; if(v == 0.0) st |= 4; o[1] = (double)st; a.counter[toy] = 0u; }\n";
        os << "      }\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        os << "  }\n}\n\n";
    }
};

} // namespace

NormLayout norm_layout(const Tree &t) { return computeNormLayout(t); }

KernelPlan generate_kernels(const Tree &t, bool mixed, int evt_block, int chunk) {
    KernelPlan plan;
    plan.nl = norm_layout(t);
    Gen g{t, mixed, evt_block, chunk, plan, {}};
    g.os << "// generated likelihood kernels\n";
    if(mixed)
        g.os << "typedef float R;\n#define GF_EXP(x) expf(x)\n#define GF_LOG(x) logf(x)\n";
    else
        g.os << "typedef double R;\n#define GF_EXP(x) exp(x)\n#define GF_LOG(x) log(x)\n";
    g.os << kPrelude;
    if(mixed)
        g.os << kPreludeF32;
    else
        g.os << kPreludeF64;
    g.tableLayout(true);
    g.tableLayout(false);
    g.convKernel(true);
    g.convKernel(false);
    g.gridKernel(true);
    g.gridKernel(false);
    g.eventKernel(true, false);
    g.eventKernel(false, false);
    g.eventKernel(false, true);
    plan.source = g.os.str();
    return plan;
}

} // namespace gf
