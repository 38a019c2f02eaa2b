// FP64 CPU oracle for the GooFit fit path.  TEST INFRASTRUCTURE ONLY: the
// engine never links, loads or calls this file; tests/, bench.py's CPU
// baseline leg and __graft_entry__.smoke() use it as the checker.
//
// It restates the reference's per-event device functions, normalisation
// recursion and NLL metric in plain FP64 C++ (OpenMP over events), walking the
// same node list the engine receives (include/gfengine.h).  Each function
// cites the reference file:line it follows.  Parity is pinned against the
// reference's own known-answer tests (tests/simple/NormalizeTest.cpp,
// tests/simple/AddNormTest.cpp, python/tests/test_min_conv.py) in
// tests/test_oracle_golden.py.
//
// Deliberate deviation: for multi-dimensional numeric grids the reference's
// binned MetricTaker writes every bin centre into the slot of the node's first
// observable (src/PDFs/MetricTaker.cu:74-88) and leaves the other slots
// uninitialised; the oracle evaluates the proper N-D grid.  1-D grids (all
// configs) are identical.
#include "../include/gfengine.h"
#include "amp4.h"

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Node {
    int op, flags;
    std::vector<int> params;
    std::vector<double> consts;
    std::vector<int> obs;
    std::vector<int> children;
    int integration_bins;
};

struct ConvWork {
    // host_iConsts of ConvolutionPdf::setIntegrationConstants (src/PDFs/combine/ConvolutionPdf.cu:228-282)
    double ic[6];
    int model_offset;
    std::vector<double> model, resol;
    // memo of sum_i M[i] R[i+off-k] keyed by k (same summation order as the per-event loop)
    std::vector<double> table;
    int kmin = 0, kmax = -1;
};

typedef std::complex<double> cplx;

// inDalitz (src/PDFs/physics/DalitzPlotHelpers.cu:14-59)
bool inDalitz(double m12, double m13, double bigM, double dm1, double dm2, double dm3) {
    double dm1pdm2  = dm1 + dm2;
    double bigMmdm3 = bigM - dm3;
    double bigMmdm1 = bigM - dm1;
    double m23      = bigM * bigM + dm1 * dm1 + dm2 * dm2 + dm3 * dm3 - m12 - m13;
    if(m23 < 0. || m23 > bigMmdm1 * bigMmdm1)
        return false;
    bool m12less   = (m12 < dm1pdm2 * dm1pdm2) ? false : true;
    bool m12grea   = (m12 > bigMmdm3 * bigMmdm3) ? false : true;
    double sqrtM12 = std::sqrt(m12);
    double dm11 = dm1 * dm1, dm22 = dm2 * dm2, dm33 = dm3 * dm3;
    double e1star    = 0.5 * (m12 - dm22 + dm11) / sqrtM12;
    double e3star    = 0.5 * (bigM * bigM - m12 - dm33) / sqrtM12;
    double rte1mdm11 = std::sqrt(e1star * e1star - dm11);
    double rte3mdm33 = std::sqrt(e3star * e3star - dm33);
    double minimum   = (e1star + e3star) * (e1star + e3star) - (rte1mdm11 + rte3mdm33) * (rte1mdm11 + rte3mdm33);
    bool m13less     = (m13 < minimum) ? false : true;
    double maximum   = (e1star + e3star) * (e1star + e3star) - (rte1mdm11 - rte3mdm33) * (rte1mdm11 - rte3mdm33);
    bool m13grea     = (m13 > maximum) ? false : true;
    return m12less && m12grea && m13less && m13grea;
}

// Resonance helpers (src/PDFs/physics/resonances/Resonance.cu:48-155)
double twoBodyCMmom(double rMassSq, double d1m, double d2m) {
    double kin1 = 1 - (d1m + d2m) * (d1m + d2m) / rMassSq;
    kin1        = kin1 >= 0 ? std::sqrt(kin1) : 1;
    double kin2 = 1 - (d1m - d2m) * (d1m - d2m) / rMassSq;
    kin2        = kin2 >= 0 ? std::sqrt(kin2) : 1;
    return 0.5 * std::sqrt(rMassSq) * kin1 * kin2;
}
double twoBodyCMMothermom(double rMassSq, double dm, double d3m) {
    double kin1 = 1 - (dm + d3m) * (dm + d3m) / rMassSq;
    kin1        = kin1 >= 0 ? std::sqrt(kin1) : 1;
    double kin2 = 1 - (dm - d3m) * (dm - d3m) / rMassSq;
    kin2        = kin2 >= 0 ? std::sqrt(kin2) : 1;
    return 0.5 * rMassSq * kin1 * kin2 / dm;
}
double dampingFactorSquare(double cmmom, int spin, double mRadius) {
    double square  = mRadius * mRadius * cmmom * cmmom;
    double dfsq    = 2 * square;
    double dfsqres = 13 * square / std::pow(square - 3, 2) + 9 * square * square;
    return (spin == 2) ? dfsqres : dfsq;
}
double dampingFactorSquareNorm(double cmmom, int spin, double mRadius) {
    double square  = mRadius * mRadius * cmmom * cmmom;
    double dfsq    = 1 + square;
    double dfsqres = dfsq + 8 + 2 * square + square * square;
    return (spin == 2) ? dfsqres : dfsq;
}
double spinFactor(unsigned spin, double motherMass, double daug1Mass, double daug2Mass, double daug3Mass, double m12,
                  double m13, double m23, unsigned cyclic_index) {
    if(0 == spin)
        return 1;
    double _mA  = (0 == cyclic_index ? daug1Mass : (1 == cyclic_index ? daug3Mass : daug2Mass));
    double _mB  = (0 == cyclic_index ? daug2Mass : (1 == cyclic_index ? daug1Mass : daug3Mass));
    double _mC  = (0 == cyclic_index ? daug3Mass : (1 == cyclic_index ? daug2Mass : daug1Mass));
    double _mAC = (0 == cyclic_index ? m13 : (1 == cyclic_index ? m23 : m12));
    double _mBC = (0 == cyclic_index ? m23 : (1 == cyclic_index ? m12 : m13));
    double _mAB = (0 == cyclic_index ? m12 : (1 == cyclic_index ? m13 : m23));
    double massFactor = 1.0 / (_mAB);
    double sFactor    = -1;
    sFactor *= ((_mBC - _mAC) + (massFactor * (motherMass * motherMass - _mC * _mC) * (_mA * _mA - _mB * _mB)));
    if(2 == spin) {
        sFactor *= sFactor;
        double extraterm = ((_mAB - (2 * motherMass * motherMass) - (2 * _mC * _mC))
                            + massFactor * (motherMass * motherMass - _mC * _mC) * (motherMass * motherMass - _mC * _mC));
        extraterm *= ((_mAB - (2 * _mA * _mA) - (2 * _mB * _mB)) + massFactor * (_mA * _mA - _mB * _mB) * (_mA * _mA - _mB * _mB));
        extraterm /= 3;
        sFactor -= extraterm;
    }
    return sFactor;
}

struct Decay3 {
    double M, m1, m2, m3, r, rm;
};

// plainBW<I> (src/PDFs/physics/resonances/RBW.cu:9-86)
cplx plainBW(int I, double resmass, double reswidth, unsigned spin, unsigned cyclic_index, bool norm, double m12,
             double m13, double m23, const Decay3 &d) {
    cplx result(0.0, 0.0);
    double resmass2 = resmass * resmass;
    for(int i = 0; i < I; i++) {
        double rMassSq      = (0 == cyclic_index ? m12 : (1 == cyclic_index ? m13 : m23));
        double mass_daug1   = 2 == cyclic_index ? d.m2 : d.m1;
        double mass_daug2   = 0 == cyclic_index ? d.m2 : d.m3;
        double bachelorMass = (0 == cyclic_index ? d.m3 : (1 == cyclic_index ? d.m2 : d.m1));
        double frFactor = 1, frFactorMother = 1;
        double measureDaughterMoms = twoBodyCMmom(rMassSq, mass_daug1, mass_daug2);
        double nominalDaughterMoms = twoBodyCMmom(resmass2, mass_daug1, mass_daug2);
        double measureDaughterMomsMother, nominalDaughterMomsMother = 0;
        if(norm) {
            measureDaughterMomsMother = twoBodyCMMothermom(rMassSq, d.M, bachelorMass);
            nominalDaughterMomsMother = twoBodyCMMothermom(resmass2, d.M, bachelorMass);
        } else {
            measureDaughterMomsMother = twoBodyCMmom(d.M * d.M, std::sqrt(rMassSq), bachelorMass);
        }
        if(0 != spin) {
            if(norm) {
                frFactor = dampingFactorSquareNorm(nominalDaughterMoms, spin, d.r)
                           / dampingFactorSquareNorm(measureDaughterMoms, spin, d.r);
                frFactorMother = dampingFactorSquareNorm(nominalDaughterMomsMother, spin, d.rm)
                                 / dampingFactorSquareNorm(measureDaughterMomsMother, spin, d.rm);
            } else {
                frFactor       = dampingFactorSquare(measureDaughterMoms, spin, d.r);
                frFactorMother = dampingFactorSquare(measureDaughterMomsMother, spin, d.rm);
            }
        }
        double A = (resmass2 - rMassSq);
        double B = resmass2 * reswidth * std::pow(measureDaughterMoms / nominalDaughterMoms, 2.0 * spin + 1) * frFactor
                   / std::sqrt(rMassSq);
        double C = 1.0 / (A * A + B * B);
        cplx ret(A * C, B * C);
        ret *= std::sqrt(frFactor);
        ret *= std::sqrt(frFactorMother);
        ret *= spinFactor(spin, d.M, d.m1, d.m2, d.m3, m12, m13, m23, cyclic_index);
        result += ret;
        if(I > 1)
            cyclic_index = (cyclic_index + 1) % 3;
    }
    return result;
}

// Flat phase-space normalisation events of Amp4Body trees, SoA [m12, m34, cos12, cos34, phi] x n
// (set by oracle_set_amp4_norm_events; the reference generates them with MCBooster in the Amp4Body
// constructor, src/PDFs/physics/Amp4Body.cu:243-290).
std::vector<double> g_norm_events;
int64_t g_n_norm = 0;

struct Oracle {
    std::vector<Node> nodes;
    std::vector<gf_observable> obs;
    std::vector<double> P;
    std::vector<double> norm;     // host_normalizations[normalIdx + 1]
    std::vector<double> integral; // value returned by normalize()
    std::map<int, ConvWork> conv;
    std::map<int, std::vector<cplx>> amp3I; // Amp3Body node -> n x n integrals I_ij
    std::map<int, std::vector<cplx>> amp4G; // Amp4Body node -> n x n sums of A_a conj(A_b) over norm events
    bool brute_force = false;
    std::string err;

    const Node &N(int i) const { return nodes.at(i); }
    double par(int node, int i) const { return P.at(nodes[node].params.at(i)); }

    // PdfBase::recursiveSetNormalization (src/goofit/PdfBase.cpp:29-38)
    void recursiveSetNormalization(int i, double v) {
        norm[i] = v;
        for(int c : nodes[i].children)
            recursiveSetNormalization(c, v);
    }

    // Observables of a subtree in first-appearance order (PdfBase::getObservables, src/goofit/PdfBase.cpp:90-101)
    std::vector<int> subtreeObs(int i) const {
        std::vector<int> r = nodes[i].obs;
        for(int c : nodes[i].children)
            for(int o : subtreeObs(c)) {
                bool f = false;
                for(int q : r)
                    f |= (q == o);
                if(!f)
                    r.push_back(o);
            }
        return r;
    }

    // ProdPdf::ProdPdf overlap detection (src/PDFs/combine/ProdPdf.cu:28-68): each component is
    // compared with the previous one only; a component with separateNorm cancels it.
    bool prodOverlaps(int i) const {
        const Node &n = nodes[i];
        bool over = false;
        std::vector<int> check;
        for(int c : n.children) {
            if(over)
                continue;
            std::vector<int> cur = subtreeObs(c);
            for(int o : cur) {
                bool f = false;
                for(int q : check)
                    f |= (q == o);
                if(f) {
                    over = true;
                    break;
                }
            }
            check = cur;
        }
        if(over)
            for(int c : n.children)
                if(nodes[c].flags & GF_FLAG_SEPARATE_NORM)
                    over = false;
        return over;
    }

    bool hasAnalyticIntegral(int i) const {
        const Node &n = nodes[i];
        switch(n.op) {
        case GF_OP_EXP:
        case GF_OP_EXP_OFFSET:
        case GF_OP_EXP_POLY:
        case GF_OP_EXP_POLY_OFFSET:
            // ExpPdf::hasAnalyticIntegral: 1 == nParams (include/goofit/PDFs/basic/ExpPdf.h:35)
            return n.params.size() == 1;
        case GF_OP_GAUSSIAN:
            return true; // include/goofit/PDFs/basic/GaussianPdf.h:24
        default:
            return false;
        }
    }

    // ExpPdf::integrate (src/PDFs/basic/ExpPdf.cu:121-132), GaussianPdf::integrate (src/PDFs/basic/GaussianPdf.cu:28-35)
    double integrate(int i, double lo, double hi) const {
        const Node &n = nodes[i];
        if(n.op == GF_OP_GAUSSIAN) {
            static const double rootPi = std::sqrt(std::atan2(0.0, -1.0));
            double sigma               = par(i, 1);
            sigma *= std::sqrt(2.0) * rootPi;
            return sigma;
        }
        double alpha = par(i, 0); // host_parameters[parametersIdx + 1]
        if(0 == alpha)
            return hi - lo;
        double ret = std::exp(alpha * hi) - std::exp(alpha * lo);
        ret /= alpha;
        return ret;
    }

    // GooPdf::normalize (src/PDFs/GooPdf.cu:340-396) with the per-class overrides
    double normalize(int i) {
        const Node &n = nodes[i];
        if(n.op == GF_OP_ADD || n.op == GF_OP_ADD_EXT) {
            // AddPdf::normalize (src/PDFs/combine/AddPdf.cu:143-185)
            bool extended = n.op == GF_OP_ADD_EXT;
            double ret = 0, totalWeight = 0;
            size_t nc = n.children.size();
            for(size_t c = 0; c + 1 < nc; ++c) {
                double weight = par(i, (int)c);
                totalWeight += weight;
                double curr = normalize(n.children[c]);
                ret += curr * weight;
            }
            double last = normalize(n.children[nc - 1]);
            if(extended) {
                double lastWeight = par(i, (int)nc - 1);
                totalWeight += lastWeight;
                ret += last * lastWeight;
                ret /= totalWeight;
            } else {
                ret += (1 - totalWeight) * last;
            }
            norm[i]     = 1.0;
            integral[i] = ret;
            if(n.flags & GF_FLAG_COMMON_NORM)
                for(int c : n.children)
                    norm[c] = 1.0 / ret;
            return ret;
        }
        if(n.op == GF_OP_PROD) {
            // ProdPdf::normalize (src/PDFs/combine/ProdPdf.cu:75-99)
            if(prodOverlaps(i)) {
                recursiveSetNormalization(i, 1.0);
                return numericNormalize(i);
            }
            for(int c : n.children)
                normalize(c);
            norm[i]     = 1.0;
            integral[i] = 1.0;
            return 1.0;
        }
        if(n.op == GF_OP_AMP3BODY)
            return normalizeAmp3(i);
        if(n.op == GF_OP_AMP4BODY)
            return normalizeAmp4(i);
        if(n.op == GF_OP_CONVOLUTION) {
            // ConvolutionPdf::normalize (src/PDFs/combine/ConvolutionPdf.cu:313-358)
            recursiveSetNormalization(i, 1.0);
            fillWorkspaces(i);
            return numericNormalize(i);
        }
        if(hasAnalyticIntegral(i)) {
            double ret = 1;
            for(int o : n.obs)
                ret *= integrate(i, obs[o].lo, obs[o].hi);
            norm[i]     = 1.0 / ret;
            integral[i] = ret;
            return ret;
        }
        return numericNormalize(i);
    }

    int gridBins(int i, int o) const {
        return nodes[i].integration_bins > 0 ? nodes[i].integration_bins : obs[o].nbins;
    }

    // Numeric branch of GooPdf::normalize + GooPdf::reduce_with_bins + binned MetricTaker
    // (src/PDFs/GooPdf.cu:83-108,366-395; src/PDFs/MetricTaker.cu:48-96; src/PDFs/GooPdf.cpp:32-50)
    double numericNormalize(int i) {
        const Node &n = nodes[i];
        size_t totalBins = 1;
        for(int o : n.obs)
            totalBins *= (size_t)gridBins(i, o);
        double ret = 1;
        double vol = 1.0;
        for(int o : n.obs)
            vol *= obs[o].hi - obs[o].lo;
        ret *= vol;
        ret /= totalBins;
        double sum = 0;
#pragma omp parallel for reduction(+ : sum) schedule(static)
        for(int64_t b = 0; b < (int64_t)totalBins; ++b) {
            std::vector<double> evt(obs.size(), 0.0);
            int64_t bin = b;
            for(int o : n.obs) {
                int nb       = gridBins(i, o);
                int localBin = (int)(bin % nb);
                double x     = obs[o].hi - obs[o].lo;
                x /= nb;
                x *= (localBin + 0.5);
                x += obs[o].lo;
                evt[o] = x;
                bin /= nb;
            }
            sum += eval(i, evt.data());
        }
        if(std::isnan(sum))
            throw std::runtime_error("NaN in normalization");
        if(0 >= sum)
            throw std::runtime_error("Non-positive normalization");
        ret *= sum;
        if(0 == ret)
            throw std::runtime_error("Zero integral");
        norm[i]     = 1.0 / ret;
        integral[i] = ret;
        return ret;
    }

    // ConvolutionPdf::setIntegrationConstants (src/PDFs/combine/ConvolutionPdf.cu:228-282) and the
    // workspace fills of ConvolutionPdf::normalize (src/PDFs/combine/ConvolutionPdf.cu:325-353)
    void fillWorkspaces(int i) {
        const Node &n = nodes[i];
        ConvWork &w   = conv[i];
        double lo = n.consts.at(0), hi = n.consts.at(1), step = n.consts.at(2);
        const gf_observable &dep = obs.at(n.obs.at(0));
        int nM  = (int)std::floor((hi - lo) / step + 0.5);
        w.ic[0] = lo;
        w.ic[1] = hi;
        w.ic[2] = nM;
        w.ic[3] = lo - dep.hi;
        w.ic[4] = hi - dep.lo;
        int nR  = (int)std::floor((w.ic[4] - w.ic[3]) / step + 0.5);
        w.ic[5] = nR;
        w.model_offset = (int)(dep.hi / step);
        int model = n.children.at(0), resol = n.children.at(1);
        w.model.assign(nM, 0.0);
        w.resol.assign(nR, 0.0);
        binnedEval(model, w.ic + 0, w.model);
        binnedEval(resol, w.ic + 3, w.resol);
        w.table.clear();
        w.kmax = w.kmin - 1;
    }

    // binned MetricTaker over one range triple (lo, hi, nbins) with the Eval metric
    void binnedEval(int node, const double *range, std::vector<double> &out) {
        int id      = nodes[node].obs.at(0);
        int numBins = (int)std::floor(range[2] + 0.5);
        for(int b = 0; b < (int)out.size(); ++b) {
            std::vector<double> evt(obs.size(), 0.0);
            int localBin = b % numBins;
            double x     = range[1] - range[0];
            x /= numBins;
            x *= (localBin + 0.5);
            x += range[0];
            evt[id] = x;
            out[b]  = eval(node, evt.data());
        }
    }

    static int offsetInBins(double x0, double loBound, double step) {
        double lowerBoundOffset = loBound / step;
        lowerBoundOffset -= std::floor(lowerBoundOffset);
        return (int)std::floor(x0 / step - lowerBoundOffset);
    }

    double convSum(int i, int k) const {
        const Node &n     = nodes[i];
        const ConvWork &w = conv.at(i);
        double loBound = n.consts[0], hiBound = n.consts[1], step = n.consts[2];
        int numbins = (int)std::floor((hiBound - loBound) / step + 0.5);
        double ret  = 0;
        for(int m = 0; m < numbins; ++m) {
            int r = m + w.model_offset - k;
            if(r < 0 || r >= (int)w.resol.size())
                throw std::runtime_error("convolution resolution index out of range");
            ret += w.model[m] * w.resol[r];
        }
        return ret;
    }

    // Fills the per-k memo over [kmin, kmax]; identical values to convSum(i, k).
    void buildConvTable(int i, int kmin, int kmax) {
        ConvWork &w = conv.at(i);
        w.kmin      = kmin;
        w.kmax      = kmax;
        w.table.assign(kmax - kmin + 1, 0.0);
#pragma omp parallel for schedule(static)
        for(int k = kmin; k <= kmax; ++k)
            w.table[k - kmin] = convSum(i, k);
    }

    // Per-event device functions (src/PDFs/basic/*.cu, src/PDFs/combine/*.cu)
    double eval(int i, const double *evt) const {
        const Node &n = nodes[i];
        switch(n.op) {
        case GF_OP_EXP: { // src/PDFs/basic/ExpPdf.cu:7-17
            double x = evt[n.obs[0]];
            return std::exp(par(i, 0) * x);
        }
        case GF_OP_EXP_OFFSET: { // src/PDFs/basic/ExpPdf.cu:19-30
            double x = evt[n.obs[0]];
            x -= par(i, 0);
            return std::exp(par(i, 1) * x);
        }
        case GF_OP_EXP_POLY: { // src/PDFs/basic/ExpPdf.cu:32-46
            double x = evt[n.obs[0]], exparg = 0;
            for(size_t k = 0; k < n.params.size(); ++k)
                exparg += std::pow(x, (double)k) * par(i, (int)k);
            return std::exp(exparg);
        }
        case GF_OP_EXP_POLY_OFFSET: { // src/PDFs/basic/ExpPdf.cu:48-63
            double x = evt[n.obs[0]];
            x -= par(i, 0);
            double exparg = 0;
            for(size_t k = 1; k < n.params.size(); ++k)
                exparg += std::pow(x, (double)k) * par(i, (int)k);
            return std::exp(exparg);
        }
        case GF_OP_GAUSSIAN: { // src/PDFs/basic/GaussianPdf.cu:7-17
            double x = evt[n.obs[0]], mean = par(i, 0), sigma = par(i, 1);
            return std::exp(-0.5 * (x - mean) * (x - mean) / (sigma * sigma));
        }
        case GF_OP_POLYNOMIAL: { // src/PDFs/basic/PolynomialPdf.cu:8-26
            int lowestDegree = (int)n.consts.at(0);
            double x = evt[n.obs[0]], ret = 0;
            for(size_t k = 0; k < n.params.size(); ++k)
                ret += par(i, (int)k) * std::pow(x, (double)(lowestDegree + (int)k));
            return ret;
        }
        case GF_OP_POLYNOMIAL_OFFSET: { // src/PDFs/basic/PolynomialPdf.cu:28-44
            int lowestDegree = (int)n.consts.at(0);
            double x = evt[n.obs[0]], ret = 0;
            for(size_t k = 2; k < n.params.size(); ++k)
                ret += par(i, (int)k) * std::pow(x, (double)(lowestDegree + (int)k - 2));
            return ret;
        }
        case GF_OP_ADD: { // src/PDFs/combine/AddPdf.cu:16-51
            double ret = 0, totalWeight = 0;
            size_t np = n.params.size();
            for(size_t k = 0; k < np; ++k) {
                double weight = par(i, (int)k);
                totalWeight += weight;
                int c       = n.children[k];
                double curr = eval(c, evt);
                ret += weight * curr * norm[c];
            }
            int c       = n.children[np];
            double last = eval(c, evt);
            ret += (1 - totalWeight) * last * norm[c];
            return ret;
        }
        case GF_OP_ADD_EXT: { // src/PDFs/combine/AddPdf.cu:53-80
            double ret = 0, totalWeight = 0;
            for(size_t k = 0; k < n.params.size(); ++k) {
                double weight = par(i, (int)k);
                int c         = n.children[k];
                double curr   = eval(c, evt);
                ret += weight * curr * norm[c];
                totalWeight += weight;
            }
            ret /= totalWeight;
            return ret;
        }
        case GF_OP_PROD: { // src/PDFs/combine/ProdPdf.cu:9-26
            double ret = 1;
            for(int c : n.children) {
                double curr = eval(c, evt);
                curr *= norm[c];
                ret *= curr;
            }
            return ret;
        }
        case GF_OP_CONVOLUTION: { // src/PDFs/combine/ConvolutionPdf.cu:27-75
            double x0 = evt[n.obs[0]];
            int k     = offsetInBins(x0, n.consts[0], n.consts[2]);
            const ConvWork &w = conv.at(i);
            double ret;
            if(!brute_force && k >= w.kmin && k <= w.kmax)
                ret = w.table[k - w.kmin];
            else
                ret = convSum(i, k);
            ret *= norm[n.children[0]];
            ret *= norm[n.children[1]];
            return ret;
        }
        case GF_OP_MULTIPOLYNOMIAL: { // src/PDFs/basic/PolynomialPdf.cu:46-107
            int num_observables = (int)n.obs.size();
            int maxDegree       = (int)n.consts.at(0) + 1;
            int numBoxes        = 1;
            for(int k = 0; k < num_observables; ++k)
                numBoxes *= maxDegree;
            int coeffNumber = num_observables;
            double ret      = par(i, coeffNumber);
            coeffNumber++;
            for(int b = 1; b < numBoxes; ++b) {
                double currTerm  = 1;
                int currIndex    = b;
                int sumOfIndices = 0;
                for(int j = 0; j < num_observables; ++j) {
                    double x = evt[n.obs[j]];
                    x -= par(i, j);
                    int currPower = currIndex % maxDegree;
                    currIndex /= maxDegree;
                    currTerm *= std::pow(x, (double)currPower);
                    sumOfIndices += currPower;
                }
                if(sumOfIndices >= maxDegree)
                    continue;
                currTerm *= par(i, coeffNumber);
                coeffNumber++;
                ret += currTerm;
            }
            return ret;
        }
        case GF_OP_AMP3BODY: { // device_DalitzPlot, src/PDFs/physics/Amp3Body.cu:60-122
            const Decay3 d = decay3(i);
            double m12 = evt[n.obs[0]], m13 = evt[n.obs[1]];
            if(!inDalitz(m12, m13, d.M, d.m1, d.m2, d.m3))
                return 0;
            double m23 = d.M * d.M + d.m1 * d.m1 + d.m2 * d.m2 + d.m3 * d.m3 - m12 - m13;
            int nRes   = (int)n.consts.at(0);
            cplx totalAmp(0, 0);
            for(int r = 0; r < nRes; ++r) {
                cplx amp(par(i, 2 * r), par(i, 2 * r + 1));
                totalAmp += amp * resonance(n.children[r], m12, m13, m23, d);
            }
            double ret = std::norm(totalAmp);
            ret *= eval(n.children[nRes], evt);
            return ret;
        }
        case GF_OP_AMP4BODY: { // device_DP, src/PDFs/physics/Amp4Body.cu:53-90
            const double v[5] = {evt[n.obs[0]], evt[n.obs[1]], evt[n.obs[2]], evt[n.obs[3]], evt[n.obs[4]]};
            const int nAmp    = (int)n.children.size() - 1;
            std::vector<cplx> A(nAmp);
            amp4Amplitudes(i, v, A.data());
            cplx totalAmp(0, 0);
            for(int a = 0; a < nAmp; ++a)
                totalAmp += A[a] * cplx(par(i, 2 * a), par(i, 2 * a + 1));
            double ret = std::norm(totalAmp);
            ret *= eval(n.children[nAmp], evt);
            return ret;
        }
        default:
            throw std::runtime_error("oracle: unsupported op " + std::to_string(n.op));
        }
    }

    // Amplitudes A_a of Amp4Body node i at one point of the 5 variables: AmpCalc
    // (src/PDFs/physics/detail/AmpCalc.cu:14-59) over the line shapes (LSCalculator,
    // src/PDFs/physics/detail/LSCalculator.cu:11-68) and spin factors (SFCalculator, SFCalculator.cu:11-55).
    void amp4Amplitudes(int i, const double *v, cplx *A) const {
        const Node &n = nodes[i];
        const double M = n.consts.at(0), m1 = n.consts.at(1), m2 = n.consts.at(2), m3 = n.consts.at(3),
                     m4 = n.consts.at(4);
        double V[16];
        amp4::get4Vecs(V, v[0], v[1], v[2], v[3], v[4], M, m1, m2, m3, m4);
        const int nAmp = (int)n.children.size() - 1;
        for(int a = 0; a < nAmp; ++a) {
            const Node &an = nodes[n.children[a]];
            const int nPerm = (int)an.consts.at(0), nLS = (int)an.consts.at(1), nSF = (int)an.consts.at(2);
            const int LS_step = nLS / nPerm, SF_step = nSF / nPerm;
            cplx ret2(0, 0);
            for(int p = 0; p < nPerm; ++p) {
                cplx ret(1, 0);
                for(int j = p * LS_step; j < (p + 1) * LS_step; ++j) {
                    const Node &ls = nodes[an.children[j]];
                    const unsigned pair = (unsigned)ls.consts.at(0);
                    double d1, d2, mres;
                    if(pair < 2) {
                        mres = pair == 0 ? v[0] : v[1];
                        d1   = pair == 0 ? m1 : m3;
                        d2   = pair == 0 ? m2 : m4;
                    } else
                        mres = amp4::getmass(pair, d1, d2, V, m1, m2, m3, m4);
                    ret *= amp4::lineshape(ls.op == GF_OP_LS_SBW, mres, d1, d2, P.at(ls.params.at(0)),
                                           P.at(ls.params.at(1)), (unsigned)ls.consts.at(1), (unsigned)ls.consts.at(2),
                                           ls.consts.at(3));
                }
                for(int j = p * SF_step; j < (p + 1) * SF_step; ++j) {
                    const Node &sf = nodes[an.children[nLS + j]];
                    const int pp[4] = {(int)sf.consts.at(2), (int)sf.consts.at(3), (int)sf.consts.at(4),
                                       (int)sf.consts.at(5)};
                    ret *= amp4::spinFactor((int)sf.consts.at(0), sf.consts.at(1), pp, V);
                }
                ret2 += ret;
            }
            ret2 *= (1 / std::sqrt((double)nPerm));
            A[a] = ret2;
        }
    }

    // Amp4Body::normalize (src/PDFs/physics/Amp4Body.cu:398-558) with NormIntegrator
    // (src/PDFs/physics/detail/NormIntegrator.cu:15-68): mean of |sum_a c_a A_a|^2 over the flat
    // phase-space events; the efficiency does not enter.
    double normalizeAmp4(int i) {
        const Node &n = nodes[i];
        recursiveSetNormalization(i, 1.0);
        if(g_n_norm <= 0)
            throw std::runtime_error("oracle: Amp4Body without normalisation events");
        const int nAmp = (int)n.children.size() - 1;
        std::vector<cplx> c(nAmp);
        for(int a = 0; a < nAmp; ++a)
            c[a] = cplx(par(i, 2 * a), par(i, 2 * a + 1));
        int nthreads = 1;
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#endif
        std::vector<double> part(nthreads, 0.0);
        std::vector<cplx> gram(nAmp * nAmp, cplx(0, 0));
        std::vector<std::vector<cplx>> gpart(nthreads, std::vector<cplx>(nAmp * nAmp, cplx(0, 0)));
#pragma omp parallel
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            std::vector<cplx> A(nAmp);
#pragma omp for schedule(static)
            for(int64_t e = 0; e < g_n_norm; ++e) {
                const double v[5] = {g_norm_events[e], g_norm_events[g_n_norm + e], g_norm_events[2 * g_n_norm + e],
                                     g_norm_events[3 * g_n_norm + e], g_norm_events[4 * g_n_norm + e]};
                amp4Amplitudes(i, v, A.data());
                cplx t(0, 0);
                for(int a = 0; a < nAmp; ++a)
                    t += A[a] * c[a];
                part[tid] += std::norm(t);
                for(int a = 0; a < nAmp; ++a)
                    for(int b = 0; b < nAmp; ++b)
                        gpart[tid][a * nAmp + b] += A[a] * std::conj(A[b]);
            }
        }
        double sumIntegral = 0;
        for(double p : part)
            sumIntegral += p;
        for(auto &g : gpart)
            for(int k = 0; k < nAmp * nAmp; ++k)
                gram[k] += g[k];
        amp4G[i] = gram;
        sumIntegral /= (double)g_n_norm;
        norm[i]     = 1.0 / sumIntegral;
        integral[i] = sumIntegral;
        return sumIntegral;
    }

    Decay3 decay3(int i) const {
        const Node &n = nodes[i];
        return Decay3{n.consts.at(2), n.consts.at(3), n.consts.at(4), n.consts.at(5), n.consts.at(6), n.consts.at(7)};
    }

    cplx resonance(int r, double m12, double m13, double m23, const Decay3 &d) const {
        const Node &rn = nodes[r];
        if(rn.op == GF_OP_RES_NONRES) // nonres, src/PDFs/physics/resonances/NonRes.cu:8-11
            return cplx(1.0, 0.0);
        if(rn.op != GF_OP_RES_RBW)
            throw std::runtime_error("oracle: unsupported resonance op");
        int I = (rn.consts.size() > 3 && rn.consts[3] != 0) ? 2 : 1;
        return plainBW(I, par(r, 0), par(r, 1), (unsigned)rn.consts.at(0), (unsigned)rn.consts.at(1), rn.consts.at(2) != 0,
                       m12, m13, m23, d);
    }

    // Amp3Body::normalize (src/PDFs/physics/Amp3Body.cu:238-359) with the integrals of
    // SpecialResonanceIntegrator (src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:7-121); the m13
    // bin count is read from the m12 slot as the reference does (line 72).
    double normalizeAmp3(int i) {
        const Node &n = nodes[i];
        recursiveSetNormalization(i, 1.0);
        const Decay3 d = decay3(i);
        int nRes       = (int)n.consts.at(0);
        int eff        = n.children[nRes];
        const gf_observable &o12 = obs[n.obs[0]], &o13 = obs[n.obs[1]];
        int nb12 = o12.nbins, nb13 = o13.nbins;
        int nb13q = (int)std::floor((double)nb12 + 0.5);
        int64_t totalBins = (int64_t)nb12 * nb13;
        int nthreads      = 1;
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#endif
        std::vector<std::vector<cplx>> part(nthreads, std::vector<cplx>(nRes * nRes, cplx(0, 0)));
#pragma omp parallel
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            std::vector<cplx> B(nRes);
            std::vector<double> evt(obs.size(), 0.0);
#pragma omp for schedule(static)
            for(int64_t b = 0; b < totalBins; ++b) {
                int binNumberM12 = (int)(b % nb12);
                double c12       = o12.hi - o12.lo;
                c12 /= nb12;
                c12 *= (binNumberM12 + 0.5);
                c12 += o12.lo;
                int64_t g   = b / nb12;
                double c13  = o13.hi - o13.lo;
                c13 /= nb13q;
                c13 *= (g + 0.5);
                c13 += o13.lo;
                if(!inDalitz(c12, c13, d.M, d.m1, d.m2, d.m3))
                    continue;
                double m23 = d.M * d.M + d.m1 * d.m1 + d.m2 * d.m2 + d.m3 * d.m3 - c12 - c13;
                for(int r = 0; r < nRes; ++r)
                    B[r] = resonance(n.children[r], c12, c13, m23, d);
                if(!evt.empty())
                    evt[0] = 2;
                evt[n.obs[0]] = c12;
                evt[n.obs[1]] = c13;
                double e      = eval(eff, evt.data());
                for(int r = 0; r < nRes; ++r)
                    for(int q = 0; q < nRes; ++q)
                        part[tid][r * nRes + q] += B[r] * std::conj(B[q]) * e;
            }
        }
        std::vector<cplx> I(nRes * nRes, cplx(0, 0));
        for(auto &p : part)
            for(int k = 0; k < nRes * nRes; ++k)
                I[k] += p[k];
        amp3I[i] = I;
        cplx sumIntegral(0, 0);
        for(int r = 0; r < nRes; ++r) {
            cplx ai(par(i, 2 * r), par(i, 2 * r + 1));
            for(int q = 0; q < nRes; ++q) {
                cplx aj(par(i, 2 * q), -par(i, 2 * q + 1));
                sumIntegral += ai * aj * I[r * nRes + q];
            }
        }
        double ret           = sumIntegral.real();
        double binSizeFactor = 1;
        binSizeFactor *= (o12.hi - o12.lo) / o12.nbins;
        binSizeFactor *= (o13.hi - o13.lo) / o13.nbins;
        ret *= binSizeFactor;
        norm[i]     = 1.0 / ret;
        integral[i] = ret;
        return ret;
    }

    // Pre-builds conv memo tables over the k range of the given events (no effect on values).
    void prepareConvTables(const double *soa, int64_t n_events) {
        if(brute_force)
            return;
        for(auto &kv : conv) {
            int i         = kv.first;
            const Node &n = nodes[i];
            int o         = n.obs[0];
            int kmin = offsetInBins(obs[o].lo, n.consts[0], n.consts[2]);
            int kmax = offsetInBins(obs[o].hi, n.consts[0], n.consts[2]);
            for(int64_t e = 0; e < n_events; ++e) {
                int k = offsetInBins(soa[o * n_events + e], n.consts[0], n.consts[2]);
                kmin  = k < kmin ? k : kmin;
                kmax  = k > kmax ? k : kmax;
            }
            buildConvTable(i, kmin, kmax);
        }
    }
};

bool load(Oracle &O,
          const gf_node *nodes,
          int n_nodes,
          const gf_observable *obs,
          int n_obs,
          const double *params,
          int n_params,
          int brute_force) {
    O.nodes.clear();
    for(int i = 0; i < n_nodes; ++i) {
        const gf_node &g = nodes[i];
        Node n;
        n.op    = g.op;
        n.flags = g.flags;
        n.params.assign(g.params, g.params + g.n_params);
        n.consts.assign(g.consts, g.consts + g.n_consts);
        n.obs.assign(g.obs, g.obs + g.n_obs);
        n.children.assign(g.children, g.children + g.n_children);
        n.integration_bins = g.integration_bins;
        O.nodes.push_back(n);
    }
    O.obs.assign(obs, obs + n_obs);
    O.P.assign(params, params + n_params);
    O.norm.assign(n_nodes, 1.0);
    O.integral.assign(n_nodes, 1.0);
    O.brute_force = brute_force != 0;
    return true;
}

thread_local std::string g_err;

} // namespace

extern "C" {

const char *oracle_last_error() { return g_err.c_str(); }

// Normalises the tree rooted at `root` and evaluates `metric` for every event
// (GooPdf::evaluate_with_metric, src/PDFs/GooPdf.cu:112-173).  integrals/norms
// (may be NULL) receive every node's normalize() value and factor.
int oracle_evaluate(const gf_node *nodes,
                    int n_nodes,
                    const gf_observable *obs,
                    int n_obs,
                    const double *params,
                    int n_params,
                    const double *soa,
                    int64_t n_events,
                    int root,
                    int metric,
                    int brute_force,
                    double *out,
                    double *integrals,
                    double *norms) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, brute_force);
        O.normalize(root);
        O.prepareConvTables(soa, n_events);
        double rootNorm = O.norm[root];
        std::vector<double> tmp;
#pragma omp parallel for schedule(static) private(tmp)
        for(int64_t e = 0; e < n_events; ++e) {
            tmp.resize(n_obs);
            for(int o = 0; o < n_obs; ++o)
                tmp[o] = soa[o * n_events + e];
            double raw = O.eval(root, tmp.data());
            double v;
            if(metric == GF_METRIC_EVAL)
                v = raw; // calculateEval, src/PDFs/MetricPointer.cu:8-11
            else if(metric == GF_METRIC_PROB)
                v = raw * rootNorm; // calculateProb, src/PDFs/MetricPointer.cu:18-21
            else {
                raw *= rootNorm; // calculateNLL, src/PDFs/MetricPointer.cu:13-16
                v = raw > 0.0 ? -std::log(raw) : 0.0;
            }
            out[e] = v;
        }
        if(integrals)
            for(int i = 0; i < n_nodes; ++i)
                integrals[i] = O.integral[i];
        if(norms)
            for(int i = 0; i < n_nodes; ++i)
                norms[i] = O.norm[i];
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// GooPdf::calculateNLL (src/PDFs/GooPdf.cu:254-273) + AddPdf::calculateNLL extended term
// (src/PDFs/combine/AddPdf.cu:187-204).  Root is node 0.
int oracle_nll(const gf_node *nodes,
               int n_nodes,
               const gf_observable *obs,
               int n_obs,
               const double *params,
               int n_params,
               const double *soa,
               int64_t n_events,
               int brute_force,
               double *nll) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, brute_force);
        O.normalize(0);
        if(O.norm[0] <= 0)
            throw std::runtime_error("non-positive normalization");
        O.prepareConvTables(soa, n_events);
        double rootNorm = O.norm[0];
        double ret      = 0;
#pragma omp parallel for reduction(+ : ret) schedule(static)
        for(int64_t e = 0; e < n_events; ++e) {
            double evt[16];
            for(int o = 0; o < n_obs; ++o)
                evt[o] = soa[o * n_events + e];
            double raw = O.eval(0, evt) * rootNorm;
            ret += raw > 0.0 ? -std::log(raw) : 0.0;
        }
        if(0.0 == ret)
            throw std::runtime_error("zero NLL");
        if(O.nodes[0].op == GF_OP_ADD_EXT) {
            double expEvents = 0;
            for(size_t k = 0; k < O.nodes[0].params.size(); ++k)
                expEvents += O.par(0, (int)k);
            ret += (expEvents - (double)n_events * std::log(expEvents));
        }
        *nll = ret;
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// A binned fit's objective (MetricPointer.cu:23-60 over PdfBase::setData's binned layout,
// src/PDFs/PdfBase.cu:439-527): soa holds n_obs - 2 centre columns, the bin contents and the bin volumes
// (metric 2: the bin errors); c_totalEvents is the number of bins.
int oracle_binned(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, const double *params,
                  int n_params, const double *soa, int64_t n_bins, int metric, double *out) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, 0);
        O.normalize(0);
        O.prepareConvTables(soa, n_bins);
        const double rootNorm = O.norm[0];
        const double T        = (double)n_bins;
        const double *cont = soa + (int64_t)(n_obs - 2) * n_bins, *vw = soa + (int64_t)(n_obs - 1) * n_bins;
        double ret = 0, total = 0;
#pragma omp parallel for reduction(+ : ret, total) schedule(static)
        for(int64_t e = 0; e < n_bins; ++e) {
            double evt[16];
            for(int o = 0; o < n_obs; ++o)
                evt[o] = soa[o * n_bins + e];
            const double rawPdf = O.eval(0, evt);
            total += cont[e];
            if(metric == 1) {
                double r = rawPdf * rootNorm;
                r *= vw[e];
                if(r > 0) {
                    const double expEvents = T * r;
                    ret += (expEvents - cont[e] * std::log(expEvents));
                }
            } else if(metric == 2) {
                double r = rawPdf;
                r -= cont[e];
                r /= vw[e];
                r *= r;
                ret += r;
            } else {
                double r = rawPdf * rootNorm;
                r *= vw[e];
                const double d = r * T - cont[e];
                ret += d * d / (cont[e] > 1 ? cont[e] : 1);
            }
        }
        if(O.nodes[0].op == GF_OP_ADD_EXT) {
            double expEvents = 0;
            for(size_t k = 0; k < O.nodes[0].params.size(); ++k)
                expEvents += O.par(0, (int)k);
            ret += (expEvents - total * std::log(expEvents));
        }
        *out = ret;
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// The Amp3Body integrals I_ij (n x n complex, interleaved re/im) of node `node` at the given parameters.
int oracle_amp3_integrals(const gf_node *nodes,
                          int n_nodes,
                          const gf_observable *obs,
                          int n_obs,
                          const double *params,
                          int n_params,
                          int node,
                          double *out) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, 0);
        O.normalize(node);
        const auto &I = O.amp3I.at(node);
        for(size_t k = 0; k < I.size(); ++k) {
            out[2 * k]     = I[k].real();
            out[2 * k + 1] = I[k].imag();
        }
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// Amplitude of resonance node `res` (child of Amp3Body `node`) at (m12, m13), interleaved re/im.
int oracle_amp3_resonance(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, const double *params,
                          int n_params, int node, int res, const double *m12, const double *m13, int64_t n,
                          double *out) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, 0);
        const Decay3 d = O.decay3(node);
        for(int64_t e = 0; e < n; ++e) {
            cplx v(0, 0);
            if(inDalitz(m12[e], m13[e], d.M, d.m1, d.m2, d.m3)) {
                double m23 = d.M * d.M + d.m1 * d.m1 + d.m2 * d.m2 + d.m3 * d.m3 - m12[e] - m13[e];
                v          = O.resonance(res, m12[e], m13[e], m23, d);
            }
            out[2 * e]     = v.real();
            out[2 * e + 1] = v.imag();
        }
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

void oracle_set_amp4_norm_events(const double *soa5, int64_t n) {
    g_norm_events.assign(soa5, soa5 + 5 * std::max<int64_t>(n, 0));
    g_n_norm = n;
}

// The Amp4Body sums G_ab = sum over norm events of A_a conj(A_b) (n x n complex, interleaved).
int oracle_amp4_gram(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, const double *params,
                     int n_params, int node, double *out) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, 0);
        O.normalize(node);
        const auto &G = O.amp4G.at(node);
        for(size_t k = 0; k < G.size(); ++k) {
            out[2 * k]     = G[k].real();
            out[2 * k + 1] = G[k].imag();
        }
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// Amplitudes A_a of Amp4Body `node` at n points (SoA 5 x n), interleaved complex [point][amplitude].
int oracle_amp4_amplitudes(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs,
                           const double *params, int n_params, int node, const double *soa5, int64_t n, double *out) {
    try {
        Oracle O;
        load(O, nodes, n_nodes, obs, n_obs, params, n_params, 0);
        const int nAmp = (int)O.nodes.at(node).children.size() - 1;
        std::vector<cplx> A(nAmp);
        for(int64_t e = 0; e < n; ++e) {
            const double v[5] = {soa5[e], soa5[n + e], soa5[2 * n + e], soa5[3 * n + e], soa5[4 * n + e]};
            O.amp4Amplitudes(node, v, A.data());
            for(int a = 0; a < nAmp; ++a) {
                out[2 * (e * nAmp + a)]     = A[a].real();
                out[2 * (e * nAmp + a) + 1] = A[a].imag();
            }
        }
        return 0;
    } catch(std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// get4Vecs at one point (16 values, (x, y, z, E) per daughter).
void oracle_get4vecs(const double *v5, const double *masses5, double *out16) {
    amp4::get4Vecs(out16, v5[0], v5[1], v5[2], v5[3], v5[4], masses5[0], masses5[1], masses5[2], masses5[3],
                   masses5[4]);
}

int oracle_in_dalitz(double m12, double m13, double M, double d1, double d2, double d3) {
    return inDalitz(m12, m13, M, d1, d2, d3) ? 1 : 0;
}

// std::mt19937(seed) + std::exponential_distribution<>(lambda), the generator of the
// reference's tests (tests/simple/NormalizeTest.cpp:16-30, tests/convert/GaussianTest.cpp).
void oracle_mt19937_exponential(uint32_t seed, double lambda, int64_t n, double *out) {
    std::mt19937 gen(seed);
    std::exponential_distribution<> d(lambda);
    for(int64_t i = 0; i < n; ++i)
        out[i] = d(gen);
}

int oracle_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
