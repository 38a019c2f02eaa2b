// Tree analysis: mirrors the normalisation recursion of the reference
// (GooPdf::normalize src/PDFs/GooPdf.cu:340-396, AddPdf::normalize
// src/PDFs/combine/AddPdf.cu:143-185, ProdPdf::normalize
// src/PDFs/combine/ProdPdf.cu:75-99, ConvolutionPdf::normalize
// src/PDFs/combine/ConvolutionPdf.cu:313-358) as a static plan, so that every
// FCN call runs a fixed kernel sequence.
#include "tree.h"

#include <algorithm>
#include <functional>
#include <cmath>
#include <set>
#include <sstream>

namespace gf {

namespace {

std::vector<int> merge(const std::vector<int> &a, const std::vector<int> &b) {
    std::vector<int> r;
    std::set_union(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(r));
    return r;
}

bool isExpOp(int op) {
    return op == GF_OP_EXP || op == GF_OP_EXP_OFFSET || op == GF_OP_EXP_POLY || op == GF_OP_EXP_POLY_OFFSET;
}

} // namespace

bool in_dalitz(double m12, double m13, double bigM, double dm1, double dm2, double dm3) {
    const double dm1pdm2 = dm1 + dm2, bigMmdm3 = bigM - dm3, bigMmdm1 = bigM - dm1;
    const double m23 = bigM * bigM + dm1 * dm1 + dm2 * dm2 + dm3 * dm3 - m12 - m13;
    if(m23 < 0. || m23 > bigMmdm1 * bigMmdm1)
        return false;
    const bool m12lo = !(m12 < dm1pdm2 * dm1pdm2), m12hi = !(m12 > bigMmdm3 * bigMmdm3);
    const double rt = std::sqrt(m12), dm11 = dm1 * dm1, dm22 = dm2 * dm2, dm33 = dm3 * dm3;
    const double e1 = 0.5 * (m12 - dm22 + dm11) / rt;
    const double e3 = 0.5 * (bigM * bigM - m12 - dm33) / rt;
    const double p1 = std::sqrt(e1 * e1 - dm11), p3 = std::sqrt(e3 * e3 - dm33);
    const double lo = (e1 + e3) * (e1 + e3) - (p1 + p3) * (p1 + p3);
    const double hi = (e1 + e3) * (e1 + e3) - (p1 - p3) * (p1 - p3);
    return m12lo && m12hi && !(m13 < lo) && !(m13 > hi);
}

std::vector<int> Tree::subtreeObs(int i) const {
    std::vector<int> r = nodes[i].obs;
    for(int c : nodes[i].children)
        for(int o : subtreeObs(c))
            if(std::find(r.begin(), r.end(), o) == r.end())
                r.push_back(o);
    return r;
}

bool Tree::inSubtree(int root, int i) const {
    if(root == i)
        return true;
    for(int c : nodes[root].children)
        if(inSubtree(c, i))
            return true;
    return false;
}

// ProdPdf::ProdPdf overlap detection (src/PDFs/combine/ProdPdf.cu:28-68): each
// component is compared with the previous one; separateNorm cancels it.
bool Tree::prodOverlaps(int i) const {
    bool over = false;
    std::vector<int> check;
    for(int c : nodes[i].children) {
        if(over)
            continue;
        std::vector<int> cur = subtreeObs(c);
        for(int o : cur)
            if(std::find(check.begin(), check.end(), o) != check.end()) {
                over = true;
                break;
            }
        check = cur;
    }
    if(over)
        for(int c : nodes[i].children)
            if(nodes[c].flags & GF_FLAG_SEPARATE_NORM)
                over = false;
    return over;
}

std::string Tree::build(const gf_node *in, int n_nodes, const gf_observable *ob, int n_obs, int np,
                        const int32_t *grad_mask) {
    std::ostringstream err;
    if(n_nodes <= 0 || !in)
        return "empty tree";
    if(n_obs <= 0 || n_obs > 16 || !ob)
        return "observable count must be 1..16";
    if(np < 0)
        return "negative parameter count";
    nodes.assign(n_nodes, TNode());
    obs.assign(ob, ob + n_obs);
    n_params = np;
    for(int o = 0; o < n_obs; ++o)
        if(!(obs[o].hi > obs[o].lo) || obs[o].nbins <= 0)
            return "observable " + std::to_string(o) + " needs lo < hi and nbins > 0";
    for(int i = 0; i < n_nodes; ++i) {
        const gf_node &g = in[i];
        TNode &n         = nodes[i];
        if(g.n_params < 0 || g.n_consts < 0 || g.n_obs < 0 || g.n_children < 0)
            return "node " + std::to_string(i) + ": negative count";
        n.op    = g.op;
        n.flags = g.flags;
        n.params.assign(g.params, g.params + g.n_params);
        n.consts.assign(g.consts, g.consts + g.n_consts);
        n.obs.assign(g.obs, g.obs + g.n_obs);
        n.children.assign(g.children, g.children + g.n_children);
        n.ibins = g.integration_bins;
        for(int p : n.params)
            if(p < 0 || p >= np)
                return "node " + std::to_string(i) + ": parameter index out of range";
        for(int o : n.obs)
            if(o < 0 || o >= n_obs)
                return "node " + std::to_string(i) + ": observable index out of range";
        for(int c : n.children)
            if(c <= i || c >= n_nodes)
                return "node " + std::to_string(i) + ": children must follow their parent";
    }
    // per-op arity
    for(int i = 0; i < n_nodes; ++i) {
        const TNode &n = nodes[i];
        size_t P = n.params.size(), C = n.children.size();
        bool ok  = true;
        switch(n.op) {
        case GF_OP_EXP: ok = P == 1 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_EXP_OFFSET: ok = P == 2 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_EXP_POLY: ok = P >= 1 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_EXP_POLY_OFFSET: ok = P >= 2 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_GAUSSIAN: ok = P == 2 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_POLYNOMIAL:
        case GF_OP_POLYNOMIAL_OFFSET: ok = P >= 1 && n.consts.size() >= 1 && n.obs.size() == 1 && C == 0; break;
        case GF_OP_ADD: ok = C >= 2 && P + 1 == C; break;
        case GF_OP_ADD_EXT: ok = C >= 1 && P == C; break;
        case GF_OP_PROD: ok = C >= 1; break;
        case GF_OP_CONVOLUTION: ok = C == 2 && n.consts.size() >= 3 && n.obs.size() >= 1 && n.consts[2] > 0; break;
        case GF_OP_MULTIPOLYNOMIAL: {
            ok = n.obs.size() >= 1 && n.obs.size() <= 8 && n.consts.size() >= 1 && n.consts[0] >= 0 &&
                 n.consts[0] <= 16 && C == 0;
            if(ok) {
                // monomials of total degree <= maxDegree (device_MultiPolynomial's coefficient count)
                const int deg = (int)n.consts[0] + 1;
                int64_t boxes = 1, count = 0;
                for(size_t k = 0; k < n.obs.size(); ++k)
                    boxes *= deg;
                ok = boxes <= (1 << 20);
                for(int64_t b = 0; ok && b < boxes; ++b) {
                    int64_t ci = b, sum = 0;
                    for(size_t k = 0; k < n.obs.size(); ++k) {
                        sum += ci % deg;
                        ci /= deg;
                    }
                    count += sum < deg;
                }
                ok = ok && (int64_t)P >= (int64_t)n.obs.size() + count;
            }
            break;
        }
        case GF_OP_RES_RBW: ok = P == 2 && n.consts.size() >= 3 && C == 0 && n.consts[0] >= 0 && n.consts[0] <= 2 &&
                                 n.consts[1] >= 0 && n.consts[1] <= 2; break;
        case GF_OP_RES_NONRES: ok = P == 0 && C == 0; break;
        case GF_OP_AMP4BODY:
            ok = n.consts.size() >= 5 && n.obs.size() >= 5 && C >= 2 && P == 2 * (C - 1);
            break;
        case GF_OP_AMPLITUDE:
            ok = n.consts.size() >= 3 && n.consts[0] >= 1 && n.consts[1] >= 0 && n.consts[2] >= 0 && P == 0 &&
                 (int)C == (int)n.consts[1] + (int)n.consts[2] && ((int)n.consts[1] % (int)n.consts[0]) == 0 &&
                 ((int)n.consts[2] % (int)n.consts[0]) == 0;
            break;
        case GF_OP_LS_RBW:
        case GF_OP_LS_SBW:
            ok = P == 2 && C == 0 && n.consts.size() >= 4 && n.consts[0] >= 0 && n.consts[0] <= 17 && n.consts[1] >= 0 &&
                 n.consts[1] <= 2 && n.consts[2] >= 0 && n.consts[2] <= 3;
            break;
        case GF_OP_SPINFACTOR:
            ok = P == 0 && C == 0 && n.consts.size() >= 6 && n.consts[0] >= 0 && n.consts[0] <= 15;
            for(int k = 2; ok && k < 6; ++k)
                ok = n.consts[k] >= 0 && n.consts[k] <= 3;
            break;
        case GF_OP_AMP3BODY:
            ok = n.consts.size() >= 8 && n.obs.size() >= 2 && C >= 2 && P == 2 * (C - 1) && (int)n.consts[0] == (int)C - 1;
            break;
        default: return "node " + std::to_string(i) + ": operator " + std::to_string(n.op) + " not supported";
        }
        if(!ok)
            return "node " + std::to_string(i) + ": wrong arity for operator " + std::to_string(n.op);
        if(n.flags & GF_FLAG_COMMON_NORM)
            return "node " + std::to_string(i) + ": setCommonNorm is not supported by the engine";
    }
    // every node reachable exactly once from the root
    {
        std::vector<int> seen(n_nodes, 0);
        std::vector<int> stack{0};
        while(!stack.empty()) {
            int i = stack.back();
            stack.pop_back();
            if(seen[i]++)
                return "node " + std::to_string(i) + " is shared; each PdfBase object may appear once";
            for(int c : nodes[i].children)
                stack.push_back(c);
        }
        for(int i = 0; i < n_nodes; ++i)
            if(!seen[i])
                return "node " + std::to_string(i) + " is not reachable from the root";
    }
    extended_root = nodes[0].op == GF_OP_ADD_EXT;

    // gradient slots
    gslot.assign(np, -1);
    gparam.clear();
    for(int p = 0; p < np; ++p)
        if(grad_mask && grad_mask[p]) {
            gslot[p] = (int)gparam.size();
            gparam.push_back(p);
        }
    NG = (int)gparam.size();

    // normalisation plan
    nk.assign(n_nodes, NK_ONE);
    std::vector<std::pair<int, bool>> st{{0, false}};
    while(!st.empty()) {
        auto [i, forced] = st.back();
        st.pop_back();
        const TNode &n = nodes[i];
        bool childForced = forced;
        if(forced) {
            nk[i] = NK_ONE;
        } else if(n.op == GF_OP_ADD || n.op == GF_OP_ADD_EXT) {
            nk[i] = NK_ONE;
        } else if(n.op == GF_OP_PROD) {
            if(prodOverlaps(i)) {
                nk[i]       = NK_NUMERIC;
                childForced = true;
            } else
                nk[i] = NK_ONE;
        } else if(n.op == GF_OP_CONVOLUTION) {
            nk[i]       = NK_NUMERIC;
            childForced = true;
        } else if(n.op == GF_OP_AMP3BODY) {
            nk[i]       = NK_AMP3;
            childForced = true;
        } else if(n.op == GF_OP_AMP4BODY) {
            nk[i]       = NK_AMP4;
            childForced = true;
        } else if(n.op == GF_OP_RES_RBW || n.op == GF_OP_RES_NONRES || n.op == GF_OP_AMPLITUDE ||
                  n.op == GF_OP_LS_RBW || n.op == GF_OP_LS_SBW || n.op == GF_OP_SPINFACTOR) {
            nk[i] = NK_ONE;
        } else if(isExpOp(n.op) && n.params.size() == 1) {
            nk[i] = NK_EXP;
        } else if(n.op == GF_OP_GAUSSIAN) {
            nk[i] = NK_GAUSS;
        } else {
            nk[i] = NK_NUMERIC;
        }
        for(int c : n.children)
            st.push_back({c, childForced});
    }

    // gradient dependencies (children have larger indices: iterate backwards)
    dep_val.assign(n_nodes, {});
    dep_norm.assign(n_nodes, {});
    for(int i = n_nodes - 1; i >= 0; --i) {
        const TNode &n = nodes[i];
        std::vector<int> own;
        for(int p : n.params)
            if(gslot[p] >= 0)
                own.push_back(gslot[p]);
        std::sort(own.begin(), own.end());
        own.erase(std::unique(own.begin(), own.end()), own.end());
        std::vector<int> v = own;
        for(int c : n.children)
            v = merge(v, merge(dep_val[c], dep_norm[c]));
        if(n.op == GF_OP_POLYNOMIAL_OFFSET) {
            // device_OffsetPolynomial reads parameters 2..nP-1 only
            std::vector<int> used;
            for(size_t k = 2; k < n.params.size(); ++k)
                if(gslot[n.params[k]] >= 0)
                    used.push_back(gslot[n.params[k]]);
            std::sort(used.begin(), used.end());
            used.erase(std::unique(used.begin(), used.end()), used.end());
            v = used;
        }
        if(n.op == GF_OP_AMP3BODY || n.op == GF_OP_AMP4BODY) {
            // value gradient: the coefficients and, through derivative columns of the cached amplitudes, the
            // resonance / line-shape parameters; the efficiency's parameters have no analytic derivative
            v = own;
            for(size_t r = 0; r + 1 < n.children.size(); ++r)
                v = merge(v, dep_val[n.children[r]]);
            if(!dep_val[n.children.back()].empty())
                return std::string(n.op == GF_OP_AMP3BODY ? "Amp3Body" : "Amp4Body") +
                       ": analytic gradients with respect to efficiency parameters are not provided";
        }
        dep_val[i] = v;
        if(nk[i] == NK_AMP3 || nk[i] == NK_AMP4) {
            dep_norm[i] = v;
        } else if(nk[i] == NK_EXP) {
            int s = gslot[n.params[0]];
            if(s >= 0)
                dep_norm[i] = {s};
        } else if(nk[i] == NK_GAUSS) {
            int s = gslot[n.params[1]];
            if(s >= 0)
                dep_norm[i] = {s};
        } else if(nk[i] == NK_NUMERIC) {
            dep_norm[i] = v;
        }
    }

    // convolutions
    conv_of.assign(n_nodes, -1);
    convs.clear();
    for(int i = 0; i < n_nodes; ++i) {
        const TNode &n = nodes[i];
        if(n.op != GF_OP_CONVOLUTION)
            continue;
        ConvInfo c;
        c.node  = i;
        c.model = n.children[0];
        c.resol = n.children[1];
        c.obs   = n.obs[0];
        c.lo    = n.consts[0];
        c.hi    = n.consts[1];
        c.step  = n.consts[2];
        const gf_observable &dep = obs[c.obs];
        c.nM    = (int)std::floor((c.hi - c.lo) / c.step + 0.5);
        c.ic[0] = c.lo;
        c.ic[1] = c.hi;
        c.ic[2] = c.nM;
        c.ic[3] = c.lo - dep.hi;
        c.ic[4] = c.hi - dep.lo;
        c.nR    = (int)std::floor((c.ic[4] - c.ic[3]) / c.step + 0.5);
        c.ic[5] = c.nR;
        c.offset = (int)(dep.hi / c.step);
        c.kmin   = conv_offset_in_bins(dep.lo, c.lo, c.step);
        c.kmax   = conv_offset_in_bins(dep.hi, c.lo, c.step);
        c.nK     = c.kmax - c.kmin + 1;
        if(c.nM <= 0 || c.nR <= 0 || c.nK <= 0)
            return "convolution node " + std::to_string(i) + ": empty workspace";
        if(c.offset - c.kmax < 0 || c.nM - 1 + c.offset - c.kmin >= c.nR)
            return "convolution node " + std::to_string(i) + ": resolution workspace index leaves its range";
        for(int sub : {c.model, c.resol}) {
            std::vector<int> so = subtreeObs(sub);
            if(so.size() != 1)
                return "convolution node " + std::to_string(i) + ": model and resolution must use one observable";
            for(int j = sub; j < n_nodes; ++j)
                if(inSubtree(sub, j) && nodes[j].op == GF_OP_CONVOLUTION)
                    return "nested ConvolutionPdf is not supported";
        }
        c.dep = merge(dep_val[c.model], dep_val[c.resol]);
        conv_of[i] = (int)convs.size();
        convs.push_back(c);
    }
    if(convs.size() > 8)
        return "at most 8 ConvolutionPdf nodes per tree";

    // Amp3Body nodes
    amp3_of.assign(n_nodes, -1);
    amp3s.clear();
    n_amp_cols = 0;
    for(int i = 0; i < n_nodes; ++i) {
        const TNode &n = nodes[i];
        if(n.op != GF_OP_AMP3BODY)
            continue;
        Amp3Info a;
        a.node = i;
        a.nRes = (int)n.consts[0];
        for(int r = 0; r < a.nRes; ++r) {
            int rn = n.children[r];
            if(nodes[rn].op != GF_OP_RES_RBW && nodes[rn].op != GF_OP_RES_NONRES)
                return "Amp3Body node " + std::to_string(i) + ": resonance " + std::to_string(r) +
                       " must be RBW or NonRes";
            a.res.push_back(rn);
        }
        a.eff = n.children[a.nRes];
        a.o12 = n.obs[0];
        a.o13 = n.obs[1];
        a.M = n.consts[2], a.m1 = n.consts[3], a.m2 = n.consts[4], a.m3 = n.consts[5];
        a.r = n.consts[6], a.rm = n.consts[7];
        a.nb12  = obs[a.o12].nbins;
        a.nb13  = obs[a.o13].nbins;
        a.nb13q = a.nb12;
        double b12 = (obs[a.o12].hi - obs[a.o12].lo) / a.nb12, b13 = (obs[a.o13].hi - obs[a.o13].lo) / a.nb13;
        a.area = 1;
        a.area *= b12;
        a.area *= b13;
        for(int j = i + 1; j < n_nodes; ++j)
            if(inSubtree(i, j)) {
                if(nodes[j].op == GF_OP_CONVOLUTION || nodes[j].op == GF_OP_AMP3BODY)
                    return "Amp3Body node " + std::to_string(i) + ": convolutions or Dalitz PDFs below it are not supported";
                for(int p : nodes[j].params)
                    a.cache_params.push_back(p);
            }
        if(nodes[a.eff].op == GF_OP_RES_RBW || nodes[a.eff].op == GF_OP_RES_NONRES)
            return "Amp3Body node " + std::to_string(i) + ": the last child must be the efficiency";
        for(int o : subtreeObs(a.eff))
            if(o != a.o12 && o != a.o13 && o != 0)
                return "Amp3Body node " + std::to_string(i) +
                       ": the efficiency may depend on the two Dalitz variables only";
        if(a.nb12 > 65535 || a.nb13 > 65535)
            return "Amp3Body node " + std::to_string(i) + ": at most 65535 bins per Dalitz axis";
        {
            // normalisation bins inside the kinematic boundary; bin centres as
            // src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:61-78 computes them
            const gf_observable &g12 = obs[a.o12], &g13 = obs[a.o13];
            a.grid.clear();
            for(int b13 = 0; b13 < a.nb13; ++b13) {
                double c13 = g13.hi - g13.lo;
                c13 /= a.nb13q;
                c13 *= (b13 + 0.5);
                c13 += g13.lo;
                for(int b12 = 0; b12 < a.nb12; ++b12) {
                    double c12 = g12.hi - g12.lo;
                    c12 /= a.nb12;
                    c12 *= (b12 + 0.5);
                    c12 += g12.lo;
                    if(in_dalitz(c12, c13, a.M, a.m1, a.m2, a.m3))
                        a.grid.push_back((uint32_t)b12 | ((uint32_t)b13 << 16));
                }
            }
        }
        std::sort(a.cache_params.begin(), a.cache_params.end());
        a.cache_params.erase(std::unique(a.cache_params.begin(), a.cache_params.end()), a.cache_params.end());
        a.col0 = n_amp_cols;
        n_amp_cols += a.nRes;
        amp3_of[i] = (int)amp3s.size();
        amp3s.push_back(a);
    }
    if(amp3s.size() > 4)
        return "at most 4 Amp3Body nodes per tree";

    // Amp4Body nodes: distinct line shapes and spin factors (by operator, parameters and constants)
    amp4_of.assign(n_nodes, -1);
    amp4s.clear();
    for(int i = 0; i < n_nodes; ++i) {
        const TNode &n = nodes[i];
        if(n.op != GF_OP_AMP4BODY)
            continue;
        Amp4Info a;
        a.node = i;
        a.nAmp = (int)n.children.size() - 1;
        a.eff  = n.children.back();
        for(int k = 0; k < 5; ++k)
            a.obs[k] = n.obs[k];
        a.M = n.consts[0];
        for(int k = 0; k < 4; ++k)
            a.m[k] = n.consts[1 + k];
        auto same = [&](int x, int y) {
            return nodes[x].op == nodes[y].op && nodes[x].params == nodes[y].params && nodes[x].consts == nodes[y].consts;
        };
        for(int k = 0; k < a.nAmp; ++k) {
            const int an = n.children[k];
            if(nodes[an].op != GF_OP_AMPLITUDE)
                return "Amp4Body node " + std::to_string(i) + ": child " + std::to_string(k) + " must be an Amplitude";
            const TNode &A = nodes[an];
            Amp4Info::Amp am;
            am.node  = an;
            am.nPerm = (int)A.consts[0];
            const int nLS = (int)A.consts[1];
            for(size_t c = 0; c < A.children.size(); ++c) {
                const int cn = A.children[c];
                const bool isLS = (int)c < nLS;
                const int want  = isLS ? 1 : 2;
                const int op    = nodes[cn].op;
                if((want == 1) != (op == GF_OP_LS_RBW || op == GF_OP_LS_SBW) || (want == 2) != (op == GF_OP_SPINFACTOR))
                    return "Amplitude node " + std::to_string(an) + ": line shapes first, then spin factors";
                std::vector<int> &uniq = isLS ? a.ls : a.sf;
                int found = -1;
                for(size_t u = 0; u < uniq.size(); ++u)
                    if(same(uniq[u], cn))
                        found = (int)u;
                if(found < 0) {
                    found = (int)uniq.size();
                    uniq.push_back(cn);
                }
                (isLS ? am.ls : am.sf).push_back(found);
            }
            a.amps.push_back(am);
        }
        if(nodes[a.eff].op == GF_OP_AMPLITUDE)
            return "Amp4Body node " + std::to_string(i) + ": the last child must be the efficiency";
        for(int j = i + 1; j < n_nodes; ++j)
            if(inSubtree(i, j)) {
                if(nodes[j].op == GF_OP_CONVOLUTION || nodes[j].op == GF_OP_AMP3BODY || nodes[j].op == GF_OP_AMP4BODY)
                    return "Amp4Body node " + std::to_string(i) + ": convolutions or amplitude PDFs below it are not supported";
                if(inSubtree(a.eff, j))
                    continue;
                for(int p : nodes[j].params)
                    a.cache_params.push_back(p);
            }
        std::sort(a.cache_params.begin(), a.cache_params.end());
        a.cache_params.erase(std::unique(a.cache_params.begin(), a.cache_params.end()), a.cache_params.end());
        a.col0 = n_amp_cols;
        n_amp_cols += a.nAmp;
        amp4_of[i] = (int)amp4s.size();
        amp4s.push_back(a);
    }
    // derivative columns for the floated resonance / line-shape parameters
    auto thetas = [&](int node, int nAmp, std::function<bool(int, int)> depends) {
        std::vector<AmpTheta> out;
        std::vector<int> own;
        for(int p : nodes[node].params)
            if(gslot[p] >= 0)
                own.push_back(gslot[p]);
        for(int sl : dep_val[node]) {
            if(std::find(own.begin(), own.end(), sl) != own.end())
                continue;
            AmpTheta t;
            t.slot  = sl;
            t.param = gparam[sl];
            for(int a = 0; a < nAmp; ++a)
                if(depends(a, t.param))
                    t.amps.push_back(a);
            if(!t.amps.empty())
                out.push_back(t);
        }
        return out;
    };
    auto hasParam = [&](int node, int p) {
        return std::find(nodes[node].params.begin(), nodes[node].params.end(), p) != nodes[node].params.end();
    };
    for(auto &A : amp3s)
        A.theta = thetas(A.node, A.nRes, [&](int r, int p) { return hasParam(A.res[r], p); });
    for(auto &A : amp4s)
        A.theta = thetas(A.node, A.nAmp, [&](int a, int p) {
            for(int u : A.amps[a].ls)
                if(hasParam(A.ls[u], p))
                    return true;
            return false;
        });
    for(auto &A : amp3s)
        for(auto &t : A.theta) {
            t.col0 = n_amp_cols;
            n_amp_cols += (int)t.amps.size();
        }
    for(auto &A : amp4s)
        for(auto &t : A.theta) {
            t.col0 = n_amp_cols;
            n_amp_cols += (int)t.amps.size();
        }
    if(n_amp_cols > 128)
        return "at most 128 amplitude and derivative columns per tree";

    // numeric grids
    num_of.assign(n_nodes, -1);
    nums.clear();
    kgrid.clear();
    for(int i = 0; i < n_nodes; ++i) {
        if(nk[i] != NK_NUMERIC)
            continue;
        for(int j = i + 1; j < n_nodes; ++j)
            if(inSubtree(i, j) && (nodes[j].op == GF_OP_AMP3BODY || nodes[j].op == GF_OP_AMP4BODY))
                return "a numerically normalised node cannot contain an Amp3Body or Amp4Body";
        NumInfo g;
        g.node = i;
        g.obs  = nodes[i].obs;
        if(g.obs.empty())
            return "numerically normalised node " + std::to_string(i) + " has no observables";
        for(int o : g.obs) {
            int nb = nodes[i].ibins > 0 ? nodes[i].ibins : obs[o].nbins;
            g.nbins.push_back(nb);
            g.total *= nb;
            g.volume *= obs[o].hi - obs[o].lo;
        }
        if(g.total > (int64_t)1 << 31)
            return "numeric grid too large";
        for(size_t c = 0; c < convs.size(); ++c) {
            if(!inSubtree(i, convs[c].node))
                continue;
            int axis = -1;
            for(size_t a = 0; a < g.obs.size(); ++a)
                if(g.obs[a] == convs[c].obs)
                    axis = (int)a;
            if(axis < 0)
                return "convolution observable missing from the grid of node " + std::to_string(i);
            g.convs.push_back((int)c);
            g.conv_axis.push_back(axis);
            g.kgrid_off.push_back((int64_t)kgrid.size());
            const gf_observable &o = obs[g.obs[axis]];
            for(int b = 0; b < g.nbins[axis]; ++b) {
                double x = bin_centre(o.lo, o.hi, g.nbins[axis], b);
                kgrid.push_back(conv_offset_in_bins(x, convs[c].lo, convs[c].step));
            }
        }
        num_of[i] = (int)nums.size();
        nums.push_back(g);
    }
    return "";
}

} // namespace gf
