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
)CUDA";

// Emits parameter loads (FP64 and R copies).
void emitParams(std::ostream &os, const Tree &T) {
    os << "    const double *Pt = a.P + (i64)toy * " << T.n_params << ";\n";
    for(int j = 0; j < T.n_params; ++j)
        os << "    const double pd" << j << " = Pt[" << j << "]; const R p" << j << " = (R)pd" << j << ";\n";
}

// Emits normalisation factors of every non-forced node for one toy, in FP64,
// and their R copies; sets `nflag` bits for NaN / non-positive sums.
void emitNorms(std::ostream &os, const Tree &T, bool grad) {
    const int NQ  = (int)T.nums.size();
    const int NGs = 1 + T.NG; // buffer stride, identical for both variants
    os << "    int nflag = 0; (void)nflag;\n";
    for(size_t i = 0; i < T.nodes.size(); ++i) {
        int kind = T.nk[i];
        if(kind == NK_ONE)
            continue;
        const TNode &n = T.nodes[i];
        std::string I = "I" + std::to_string(i), N = "Nd" + std::to_string(i);
        std::vector<std::string> dI; // per dep_norm slot, FP64 expression of dI/dslot
        if(kind == NK_EXP) {
            const gf_observable &o = T.obs[n.obs[0]];
            os << "    double " << I << ", dI" << i << ";\n";
            os << "    { const double al = pd" << n.params[0] << ", hi = " << lit(o.hi) << ", lo = " << lit(o.lo)
               << ";\n"
               << "      if(0 == al) { " << I << " = hi - lo; dI" << i << " = 0.5 * (hi * hi - lo * lo); }\n"
               << "      else { const double eh = exp(al * hi), el = exp(al * lo); " << I << " = (eh - el) / al; dI"
               << i << " = (hi * eh - lo * el) / al - " << I << " / al; } }\n";
        } else if(kind == NK_GAUSS) {
            double rootPi = std::sqrt(std::atan2(0.0, -1.0));
            double root2  = std::sqrt(2.0);
            os << "    const double " << I << " = pd" << n.params[1] << " * " << lit(root2 * rootPi) << ";\n";
            os << "    const double dI" << i << " = " << lit(root2 * rootPi) << ";\n";
        } else { // numeric
            int q = T.num_of[i];
            const NumInfo &g = T.nums[q];
            os << "    const double *gs" << i << " = a.gsum + ((i64)toy * " << NQ << " + " << q << ") * " << NGs
               << ";\n";
            os << "    double " << I << " = 1.0; " << I << " *= " << lit(g.volume) << "; " << I << " /= "
               << lit((double)g.total) << "; " << I << " *= gs" << i << "[0];\n";
            os << "    if(isnan(gs" << i << "[0])) nflag |= 1; else if(!(gs" << i << "[0] > 0.0)) nflag |= 2;\n";
        }
        os << "    const double " << N << " = 1.0 / " << I << ";\n";
        os << "    const R N" << i << " = (R)" << N << ";\n";
        if(grad)
            for(int s : T.dep_norm[i]) {
                std::string dexpr;
                if(kind == NK_NUMERIC) {
                    const NumInfo &g = T.nums[T.num_of[i]];
                    dexpr = "-" + N + " * " + N + " * (" + lit(g.volume) + " / " + lit((double)g.total) + ") * gs" +
                            std::to_string(i) + "[" + std::to_string(1 + s) + "]";
                } else {
                    dexpr = "-" + N + " * " + N + " * dI" + std::to_string(i);
                }
                os << "    const R dN" << i << "_" << s << " = (R)(" << dexpr << ");\n";
            }
    }
}

struct Gen {
    const Tree &T;
    bool mixed;
    int block, chunk;
    KernelPlan &plan;
    std::ostringstream os;

    int convComps(int ci, bool grad) const { return 1 + (grad ? (int)T.convs[ci].dep.size() : 0); }

    // ---------------- convolution tables ----------------
    void convKernel(bool grad) {
        const char *sfx = grad ? "g" : "n";
        int NC          = (int)T.convs.size();
        if(NC == 0)
            return;
        const int MS = 8; // lanes sharing one (k, component) sum
        auto &off    = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        int64_t total = 0;
        off.clear();
        size_t smem = 0;
        int maxBlocks = 0;
        std::vector<int> tks;
        for(int ci = 0; ci < NC; ++ci) {
            off.push_back(total);
            total += (int64_t)convComps(ci, grad) * T.convs[ci].nK;
            int comps = convComps(ci, grad);
            int tk    = std::max(1, block / (comps * MS));
            tks.push_back(tk);
            const ConvInfo &cv = T.convs[ci];
            int mcomp = 1 + (grad ? (int)T.dep_val[cv.model].size() : 0);
            int rcomp = 1 + (grad ? (int)T.dep_val[cv.resol].size() : 0);
            size_t sm = (size_t)(mcomp * cv.nM + rcomp * (cv.nM + tk - 1)) * (mixed ? 4 : 8);
            smem      = std::max(smem, sm);
            maxBlocks = std::max(maxBlocks, (cv.nK + tk - 1) / tk);
        }
        if(grad) {
            plan.ctab_per_toy_grad = total;
            plan.conv_smem_grad    = smem;
            plan.ctab_comps_grad.clear();
            for(int ci = 0; ci < NC; ++ci)
                plan.ctab_comps_grad.push_back(convComps(ci, true));
        } else {
            plan.ctab_per_toy_nograd = total;
            plan.conv_smem_nograd    = smem;
        }
        plan.conv_blocks = std::max(plan.conv_blocks, maxBlocks);

        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") gf_conv_" << sfx
           << "(const GfArgs a) {\n";
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *sm = reinterpret_cast<R *>(smraw);\n";
        os << "  const int toy = blockIdx.y; const int ci = blockIdx.z; const int tid = threadIdx.x;\n";
        os << "  if(a.active && !a.active[toy]) return;\n";
        emitParams(os, T);
        os << "  R *ctab = reinterpret_cast<R *>(a.ctab) + (i64)toy * " << total << ";\n";
        os << "  switch(ci) {\n";
        for(int ci = 0; ci < NC; ++ci) {
            const ConvInfo &cv = T.convs[ci];
            int comps = convComps(ci, grad), tk = tks[ci];
            const auto &dm = T.dep_val[cv.model];
            const auto &dr = T.dep_val[cv.resol];
            int mcomp = 1 + (grad ? (int)dm.size() : 0);
            int rcomp = 1 + (grad ? (int)dr.size() : 0);
            int win   = cv.nM + tk - 1;
            os << "  case " << ci << ": {\n";
            os << "    const int k0 = " << cv.kmin << " + (int)blockIdx.x * " << tk << ";\n";
            os << "    if(k0 > " << cv.kmax << ") return;\n";
            os << "    R *sM = sm; R *sR = sm + " << mcomp * cv.nM << ";\n";
            os << "    const int rbase = " << cv.offset << " - (k0 + " << tk - 1 << ");\n";
            // model workspace
            os << "    for(int m = tid; m < " << cv.nM << "; m += " << block << ") {\n";
            os << "      const R wx = (R)gf_centre(" << lit(cv.ic[0]) << ", " << lit(cv.ic[1]) << ", " << cv.nM
               << ", m);\n";
            {
                std::ostringstream body;
                Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
                c.x = [&](int) { return std::string("wx"); };
                c.k = [&](int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.tab = [&](int, int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.uid = 0;
                Val v = emit(c, cv.model);
                os << "      {\n" << body.str();
                os << "      sM[m] = " << v.v << ";\n";
                if(grad)
                    for(size_t j = 0; j < dm.size(); ++j) {
                        auto it = v.g.find(dm[j]);
                        os << "      sM[" << (1 + j) * cv.nM << " + m] = "
                           << (it == v.g.end() ? std::string("R(0)") : it->second) << ";\n";
                    }
                os << "      }\n";
            }
            os << "    }\n";
            // resolution window
            os << "    for(int w = tid; w < " << win << "; w += " << block << ") {\n";
            os << "      const int r = rbase + w;\n";
            os << "      if(r < 0 || r >= " << cv.nR << ") continue;\n";
            os << "      const R wx = (R)gf_centre(" << lit(cv.ic[3]) << ", " << lit(cv.ic[4]) << ", " << cv.nR
               << ", r);\n";
            {
                std::ostringstream body;
                Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
                c.x = [&](int) { return std::string("wx"); };
                c.k = [&](int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.tab = [&](int, int) -> std::string { throw std::runtime_error("codegen: conv in workspace"); };
                c.uid = 1000;
                Val v = emit(c, cv.resol);
                os << "      {\n" << body.str();
                os << "      sR[w] = " << v.v << ";\n";
                if(grad)
                    for(size_t j = 0; j < dr.size(); ++j) {
                        auto it = v.g.find(dr[j]);
                        os << "      sR[" << (1 + j) * win << " + w] = "
                           << (it == v.g.end() ? std::string("R(0)") : it->second) << ";\n";
                    }
                os << "      }\n";
            }
            os << "    }\n";
            os << "    __syncthreads();\n";
            // table entries: lanes (kk, comp, ms)
            os << "    const int ms = tid % " << MS << "; const int comp = (tid / " << MS << ") % " << comps
               << "; const int kk = tid / " << MS * comps << ";\n";
            os << "    const int k = k0 + kk;\n";
            os << "    const bool live = kk < " << tk << " && k <= " << cv.kmax << ";\n";
            os << "    ACC acc = 0;\n";
            os << "    if(live) {\n";
            os << "      const int rb = " << cv.offset << " - k - rbase;\n"; // window index of r for m = 0
            os << "      const R *mA; const R *rA; const R *mB = nullptr; const R *rB = nullptr;\n";
            os << "      switch(comp) {\n";
            os << "      case 0: mA = sM; rA = sR; break;\n";
            if(grad)
                for(size_t j = 0; j < cv.dep.size(); ++j) {
                    int s = cv.dep[j];
                    auto im = std::find(dm.begin(), dm.end(), s);
                    auto ir = std::find(dr.begin(), dr.end(), s);
                    os << "      case " << 1 + j << ": ";
                    bool first = true;
                    if(im != dm.end()) {
                        os << "mA = sM + " << (1 + (im - dm.begin())) * cv.nM << "; rA = sR; ";
                        first = false;
                    }
                    if(ir != dr.end()) {
                        if(first)
                            os << "mA = sM; rA = sR + " << (1 + (ir - dr.begin())) * win << "; ";
                        else
                            os << "mB = sM; rB = sR + " << (1 + (ir - dr.begin())) * win << "; ";
                    }
                    os << "break;\n";
                }
            os << "      default: mA = sM; rA = sR; break;\n";
            os << "      }\n";
            os << "      R s0 = R(0), s1 = R(0);\n";
            os << "      for(int m = ms; m < " << cv.nM << "; m += " << MS << ") { s0 = fma(mA[m], rA[m + rb], s0); }\n";
            os << "      if(mB) for(int m = ms; m < " << cv.nM << "; m += " << MS << ") { s1 = fma(mB[m], rB[m + rb], s1); }\n";
            os << "      acc = (ACC)s0 + (ACC)s1;\n";
            os << "    }\n";
            os << "#pragma unroll\n    for(int o = " << MS / 2 << "; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, " << MS << ");\n";
            os << "    if(live && ms == 0) ctab[" << off[ci] << " + comp * " << cv.nK << " + (k - " << cv.kmin
               << ")] = (R)acc;\n";
            os << "    break; }\n";
        }
        os << "  }\n}\n\n";
    }

    // ---------------- numeric grids ----------------
    void gridKernel(bool grad) {
        const char *sfx = grad ? "g" : "n";
        int NQ          = (int)T.nums.size();
        if(NQ == 0)
            return;
        int NGp = 1 + (grad ? T.NG : 0); // components reduced
        int NGs = 1 + T.NG;              // buffer stride
        int BPB = plan.grid_bins_per_block;
        plan.grid_blocks.clear();
        plan.max_grid_blocks = 0;
        for(auto &g : T.nums) {
            int nb = (int)((g.total + BPB - 1) / BPB);
            plan.grid_blocks.push_back(nb);
            plan.max_grid_blocks = std::max(plan.max_grid_blocks, nb);
        }
        int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        auto &off         = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") gf_grid_" << sfx
           << "(const GfArgs a) {\n";
        os << "  const int toy = blockIdx.y; const int q = blockIdx.z; const int tid = threadIdx.x;\n";
        os << "  if(a.active && !a.active[toy]) return;\n";
        emitParams(os, T);
        os << "  const R *ctab = reinterpret_cast<const R *>(a.ctab) + (i64)toy * " << ctabTotal << ";\n";
        os << "  (void)ctab;\n";
        os << "  R av = R(0);\n";
        for(int s = 0; s < (grad ? T.NG : 0); ++s)
            os << "  R ag" << s << " = R(0);\n";
        os << "  i64 total = 0; int nblk = 0;\n";
        os << "  switch(q) {\n";
        for(int q = 0; q < NQ; ++q) {
            const NumInfo &g = T.nums[q];
            os << "  case " << q << ": {\n";
            os << "    total = " << g.total << "LL; nblk = " << plan.grid_blocks[q] << ";\n";
            os << "    if((int)blockIdx.x >= nblk) return;\n";
            os << "    const i64 bend = min(total, (i64)(blockIdx.x + 1) * " << BPB << ");\n";
            os << "    for(i64 b = (i64)blockIdx.x * " << BPB << " + tid; b < bend; b += " << block << ") {\n";
            os << "      i64 bb = b;\n";
            for(size_t ax = 0; ax < g.obs.size(); ++ax) {
                const gf_observable &o = T.obs[g.obs[ax]];
                os << "      const int lb" << ax << " = (int)(bb % " << g.nbins[ax] << "); bb /= " << g.nbins[ax]
                   << ";\n";
                os << "      const R gx" << g.obs[ax] << " = (R)gf_centre(" << lit(o.lo) << ", " << lit(o.hi) << ", "
                   << g.nbins[ax] << ", lb" << ax << ");\n";
            }
            std::ostringstream body;
            Ctx c{body, T, grad, false, nullptr, nullptr, nullptr, nullptr};
            c.x = [&](int o) { return "gx" + std::to_string(o); };
            c.k = [&](int ci) -> std::string {
                for(size_t j = 0; j < g.convs.size(); ++j)
                    if(g.convs[j] == ci)
                        return "a.kgrid[" + std::to_string(g.kgrid_off[j]) + " + lb" +
                               std::to_string(g.conv_axis[j]) + "]";
                throw std::runtime_error("codegen: conv without grid k");
            };
            c.tab = [&](int ci, int comp) {
                const ConvInfo &cv = T.convs[ci];
                return "ctab[" + std::to_string(off[ci]) + " + " + std::to_string(comp * cv.nK) + " + (" + c.k(ci) +
                       " - " + std::to_string(cv.kmin) + ")]";
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
        // block reduction of NGp doubles
        os << "  __shared__ double red[" << block / 32 << "][" << NGp << "];\n";
        os << "  __shared__ int last;\n";
        os << "  const int lane = tid & 31, wid = tid >> 5;\n";
        os << "  { double t = gf_warp_sum((double)av); if(lane == 0) red[wid][0] = t; }\n";
        for(int s = 0; s < NGp - 1; ++s)
            os << "  { double t = gf_warp_sum((double)ag" << s << "); if(lane == 0) red[wid][" << 1 + s
               << "] = t; }\n";
        os << "  __syncthreads();\n";
        os << "  double *gp = a.gpartial + (((i64)toy * " << NQ << " + q) * " << plan.max_grid_blocks
           << " + blockIdx.x) * " << NGs << ";\n";
        os << "  if(tid < " << NGp << ") { double t = 0; for(int w = 0; w < " << block / 32
           << "; ++w) t += red[w][tid]; gp[tid] = t; }\n";
        os << "  __threadfence();\n  __syncthreads();\n";
        os << "  if(tid == 0) { unsigned prev = atomicAdd(&a.gcounter[toy * " << NQ
           << " + q], 1u); last = (prev == (unsigned)(nblk - 1)); }\n";
        os << "  __syncthreads();\n";
        os << "  if(last) {\n";
        os << "    __threadfence();\n";
        os << "    const double *g0 = a.gpartial + ((i64)toy * " << NQ << " + q) * " << plan.max_grid_blocks << " * "
           << NGs << ";\n";
        os << "    if(tid < " << NGp << ") { double t = 0; for(int bi = 0; bi < nblk; ++bi) t += g0[bi * " << NGs
           << " + tid]; a.gsum[((i64)toy * " << NQ << " + q) * " << NGs << " + tid] = t; }\n";
        os << "    if(tid == 0) a.gcounter[toy * " << NQ << " + q] = 0u;\n";
        os << "  }\n}\n\n";
    }

    // ---------------- event pass ----------------
    void eventKernel(bool grad, bool values) {
        std::string name = values ? "gf_val_n" : (grad ? "gf_evt_g" : "gf_evt_n");
        int NGp          = 1 + (grad ? T.NG : 0); // components reduced
        int NGs          = 1 + T.NG;              // buffer stride
        int NC           = (int)T.convs.size();
        int NO           = (int)T.obs.size();
        auto &off        = grad ? plan.ctab_off_grad : plan.ctab_off_nograd;
        int64_t ctabTotal = grad ? plan.ctab_per_toy_grad : plan.ctab_per_toy_nograd;
        // shared-memory staging of the toy's conv tables
        size_t smemElems = (size_t)ctabTotal;
        if(!values) {
            if(grad)
                plan.evt_smem_grad = smemElems * (mixed ? 4 : 8);
            else
                plan.evt_smem_nograd = smemElems * (mixed ? 4 : 8);
        }
        // body: tree code for one event, into a string so that used columns are known
        std::vector<int> xused(NO, 0);
        std::ostringstream body;
        Ctx c{body, T, grad, true, nullptr, nullptr, nullptr, &xused};
        c.x = [&](int o) {
            xused[o] = 1;
            return "ex" + std::to_string(o);
        };
        c.k = [&](int ci) { return "ek" + std::to_string(ci); };
        c.tab = [&](int ci, int comp) {
            const ConvInfo &cv = T.convs[ci];
            return "stab[" + std::to_string(off[ci] + (int64_t)comp * cv.nK) + " + (ek" + std::to_string(ci) + " - " +
                   std::to_string(cv.kmin) + ")]";
        };
        Val root = emit(c, 0);
        if(!values && !grad) {
            plan.obs_used_evt.clear();
            for(int o = 0; o < NO; ++o)
                if(xused[o])
                    plan.obs_used_evt.push_back(o);
        }
        std::string rootN = T.nk[0] == NK_ONE ? "" : "N0";

        os << "extern \"C\" __global__ void __launch_bounds__(" << block << ") " << name << "(const GfArgs a) {\n";
        os << "  extern __shared__ __align__(16) unsigned char smraw[];\n";
        os << "  R *stab = reinterpret_cast<R *>(smraw); (void)stab;\n";
        os << "  __shared__ double red[" << block / 32 << "][" << NGp << "];\n";
        os << "  __shared__ int last;\n";
        os << "  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;\n";
        os << "  for(int ch = blockIdx.x; ch < a.n_chunks; ch += gridDim.x) {\n";
        os << "    const i64 *cd = a.chunks + 3 * (i64)ch;\n";
        os << "    const int toy = (int)cd[0]; const i64 b0 = cd[1], e0 = cd[2];\n";
        os << "    if(a.active && !a.active[toy]) continue;\n";
        {
            std::ostringstream pr;
            emitParams(pr, T);
            emitNorms(pr, T, grad);
            os << pr.str();
        }
        if(NC > 0) {
            os << "    { const R *src = reinterpret_cast<const R *>(a.ctab) + (i64)toy * " << ctabTotal << ";\n";
            os << "      for(int i = tid; i < " << ctabTotal << "; i += " << block << ") stab[i] = src[i]; }\n";
        }
        os << "    __syncthreads();\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "    const R *col" << o << " = reinterpret_cast<const R *>(a.col[(i64)toy * " << NO << " + "
                   << o << "]);\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "    const int *kc" << ci << " = a.kcol[(i64)toy * " << NC << " + " << ci << "];\n";
        if(!values) {
            os << "    R av = R(0);\n";
            for(int s = 0; s < NGp - 1; ++s)
                os << "    R ag" << s << " = R(0);\n";
        }
        os << "    for(i64 i0 = b0 + 4 * (i64)tid; i0 < e0; i0 += 4 * " << block << ") {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o]) {
                if(mixed)
                    os << "      const float4 xv" << o << " = *reinterpret_cast<const float4 *>(col" << o
                       << " + i0);\n"
                       << "      const R xa" << o << "[4] = {xv" << o << ".x, xv" << o << ".y, xv" << o << ".z, xv"
                       << o << ".w};\n";
                else
                    os << "      const double2 xv" << o << "a = *reinterpret_cast<const double2 *>(col" << o
                       << " + i0), xv" << o << "b = *reinterpret_cast<const double2 *>(col" << o << " + i0 + 2);\n"
                       << "      const R xa" << o << "[4] = {xv" << o << "a.x, xv" << o << "a.y, xv" << o << "b.x, xv"
                       << o << "b.y};\n";
            }
        for(int ci = 0; ci < NC; ++ci)
            os << "      const int4 kv" << ci << " = *reinterpret_cast<const int4 *>(kc" << ci << " + i0);\n"
               << "      const int ka" << ci << "[4] = {kv" << ci << ".x, kv" << ci << ".y, kv" << ci << ".z, kv"
               << ci << ".w};\n";
        os << "#pragma unroll\n      for(int j = 0; j < 4; ++j) {\n";
        for(int o = 0; o < NO; ++o)
            if(xused[o])
                os << "        const R ex" << o << " = xa" << o << "[j];\n";
        for(int ci = 0; ci < NC; ++ci)
            os << "        const int ek" << ci << " = ka" << ci << "[j];\n";
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
            os << "    __syncthreads();\n  }\n}\n\n";
            return;
        }
        // block reduction
        os << "    { double t = gf_warp_sum((double)av); if(lane == 0) red[wid][0] = t; }\n";
        for(int s = 0; s < NGp - 1; ++s)
            os << "    { double t = gf_warp_sum((double)ag" << s << "); if(lane == 0) red[wid][" << 1 + s
               << "] = t; }\n";
        os << "    __syncthreads();\n";
        os << "    if(tid < " << NGp << ") { double t = 0; for(int w = 0; w < " << block / 32
           << "; ++w) t += red[w][tid]; a.partial[(i64)ch * " << NGs << " + tid] = t; }\n";
        os << "    __threadfence();\n    __syncthreads();\n";
        os << "    if(tid == 0) { unsigned prev = atomicAdd(&a.counter[toy], 1u); last = (prev == (unsigned)(a.toy_nchunks[toy] - 1)); }\n";
        os << "    __syncthreads();\n";
        os << "    if(last) {\n";
        os << "      __threadfence();\n";
        os << "      const int c0 = a.toy_chunk0[toy], nc = a.toy_nchunks[toy];\n";
        // deterministic: thread t sums chunks t, t+B, ... per component, then fixed-order tree
        os << "      for(int comp = 0; comp < " << NGp << "; ++comp) {\n";
        os << "        double t = 0; for(int c = tid; c < nc; c += " << block << ") t += a.partial[(i64)(c0 + c) * " << NGs
           << " + comp];\n";
        os << "        t = gf_warp_sum(t); if(lane == 0) red[wid][comp] = t;\n";
        os << "      }\n";
        os << "      __syncthreads();\n";
        os << "      if(tid == 0) {\n";
        os << "        double *o = a.out + (i64)toy * " << NGs + 1 << ";\n";
        os << "        double s[" << NGp << "];\n";
        os << "        for(int comp = 0; comp < " << NGp << "; ++comp) { double t = 0; for(int w = 0; w < "
           << block / 32 << "; ++w) t += red[w][comp]; s[comp] = t; }\n";
        if(T.extended_root) {
            // AddPdf::calculateNLL extended term (src/PDFs/combine/AddPdf.cu:187-204)
            os << "        { double ex = 0; ";
            for(int p : T.nodes[0].params)
                os << "ex += pd" << p << "; ";
            os << "const double ne = (double)a.toy_nevents[toy]; s[0] += (ex - ne * log(ex));\n";
            if(grad)
                for(int p : T.nodes[0].params)
                    if(T.gslot[p] >= 0)
                        os << "          s[" << 1 + T.gslot[p] << "] += 1.0 - ne / ex;\n";
            os << "        }\n";
        }
        os << "        int st = nflag;\n";
        if(rootN.empty())
            os << "        (void)0;\n";
        else
            os << "        if(!(Nd0 > 0.0)) st |= 2;\n";
        os << "        if(s[0] == 0.0) st |= 4;\n";
        os << "        o[0] = s[0]; o[1] = (double)st;\n";
        os << "        for(int comp = 1; comp < " << NGp << "; ++comp) o[1 + comp] = s[comp];\n";
        os << "        a.counter[toy] = 0u;\n";
        os << "      }\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        os << "  }\n}\n\n";
    }
};

} // namespace

KernelPlan generate_kernels(const Tree &t, bool mixed, int evt_block, int chunk) {
    KernelPlan plan;
    Gen g{t, mixed, evt_block, chunk, plan, {}};
    g.os << "// generated likelihood kernels\n";
    if(mixed)
        g.os << "typedef float R;\ntypedef double ACC;\n#define GF_EXP(x) expf(x)\n#define GF_LOG(x) logf(x)\n";
    else
        g.os << "typedef double R;\ntypedef double ACC;\n#define GF_EXP(x) exp(x)\n#define GF_LOG(x) log(x)\n";
    g.os << kPrelude;
    g.os << "__device__ __forceinline__ double gf_centre(double lo, double hi, int n, int b) { double x = hi - lo; x /= n; "
            "x *= (b + 0.5); x += lo; return x; }\n\n";
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
