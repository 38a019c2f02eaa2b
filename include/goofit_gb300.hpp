// GooFit-compatible C++ host API over the likelihood engine's C ABI (gfengine.h).
//
// Header-only, C++17.  The class names, constructor argument orders and the methods a fit uses follow the
// reference's C++ API (include/goofit/Variable.h, UnbinnedDataSet.h, PDFs/basic/*.h, PDFs/combine/*.h,
// PDFs/physics/Amp3Body.h, FitManager.h), so that user code of the form
//
//     Observable x{"x", 0, 10};
//     Variable alpha{"alpha", -2, 0.1, -10, 10};
//     UnbinnedDataSet data{x};
//     ... x.setValue(v); data.addEvent(); ...
//     ExpPdf pdf{"exppdf", x, alpha};
//     pdf.setData(&data);
//     FitManager fitter{&pdf};
//     fitter.fit();
//
// builds against this header and libgfengine.so.  Each PDF object becomes one gf_node (op, parameter slots,
// constants, observable columns, children) in the depth-first order of PdfBase::populateArrays
// (src/PDFs/PdfBase.cu:268-311); FitManager hands the flattened tree and the data to the engine and runs the
// engine's MIGRAD with the analytic gradient (numerical when a free parameter has none).
//
// Variable and Observable copies alias one shared state, as the reference's do (include/goofit/Variable.h:27-37).
#pragma once

#include "gfengine.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace GooFit {

using fptype = double;

class GeneralError : public std::runtime_error {
  public:
    explicit GeneralError(const std::string &what) : std::runtime_error(what) {}
};

namespace detail {
struct VarState {
    std::string name;
    double value = 0, error = 0, lo = 0, hi = 0, blind = 0;
    bool fixed = false, event_number = false;
    int numbins = 100, fitter_index = -1;
};
inline void check(int rc, const gf_engine *e) {
    if(rc != GF_OK)
        throw GeneralError(std::string("gfengine: ") + gf_last_error(e));
}
} // namespace detail

// ---------------------------------------------------------------- variables
class Indexable {
  protected:
    std::shared_ptr<detail::VarState> s_;
    Indexable(const std::string &n, double v, double lo, double hi) : s_(std::make_shared<detail::VarState>()) {
        s_->name  = n;
        s_->value = v;
        s_->lo    = lo;
        s_->hi    = hi;
    }

  public:
    const std::string &getName() const { return s_->name; }
    double getValue() const { return s_->value; }
    void setValue(double v) { s_->value = v; }
    double getLowerLimit() const { return s_->lo; }
    double getUpperLimit() const { return s_->hi; }
    void setLowerLimit(double v) { s_->lo = v; }
    void setUpperLimit(double v) { s_->hi = v; }
    operator double() const { return s_->value; }
    Indexable &operator=(double v) {
        s_->value = v;
        return *this;
    }
    const detail::VarState *state() const { return s_.get(); }
    bool sameAs(const Indexable &o) const { return s_ == o.s_; }
};

class Observable : public Indexable {
  public:
    Observable(const std::string &n, double lo, double hi) : Indexable(n, 0.0, lo, hi) {}
    void setNumBins(int n) { s_->numbins = n; }
    int getNumBins() const { return s_->numbins; }
    double getBinSize() const { return (s_->hi - s_->lo) / s_->numbins; }
    bool isEventNumber() const { return s_->event_number; }
    Observable &operator=(double v) {
        s_->value = v;
        return *this;
    }
};

class EventNumber : public Observable {
  public:
    explicit EventNumber(const std::string &n, double lo = 0, double hi = double(1LL << 53)) : Observable(n, lo, hi) {
        s_->event_number = true;
    }
};

// Variable(n, v): constant; (n, v, err): fixed, no limits; (n, v, lo, hi): free, error 0.1 (hi - lo);
// (n, v, err, lo, hi[, fixed]) as in include/goofit/Variable.h:143-190.
class Variable : public Indexable {
  public:
    Variable(const std::string &n, double v) : Indexable(n, v, v + 0.01, v - 0.01) {
        s_->error = 0.002;
        s_->fixed = true;
    }
    Variable(const std::string &n, double v, double err) : Indexable(n, v, 0, 0) {
        s_->error = err;
        s_->fixed = true;
    }
    Variable(const std::string &n, double v, double lo, double hi) : Indexable(n, v, lo, hi) {
        s_->error = 0.1 * (hi - lo);
    }
    Variable(const std::string &n, double v, double err, double lo, double hi, bool fixed = false)
        : Indexable(n, v, lo, hi) {
        s_->error = err;
        s_->fixed = fixed;
    }
    double getError() const { return s_->error; }
    void setError(double e) { s_->error = e; }
    bool IsFixed() const { return s_->fixed; }
    void setFixed(bool f) { s_->fixed = f; }
    void setBlind(double b) { s_->blind = b; }
    int getFitterIndex() const { return s_->fitter_index; }
    Variable &operator=(double v) {
        s_->value = v;
        return *this;
    }
};

// ---------------------------------------------------------------- data
class DataSet {
  protected:
    std::vector<Observable> obs_;

  public:
    explicit DataSet(const std::vector<Observable> &obs) : obs_(obs) {}
    virtual ~DataSet() = default;
    const std::vector<Observable> &getObservables() const { return obs_; }
    virtual size_t getNumEvents() const = 0;
    virtual void addEvent() = 0;
};

class UnbinnedDataSet : public DataSet {
    std::vector<std::vector<double>> cols_;

  public:
    UnbinnedDataSet(const Observable &x) : UnbinnedDataSet(std::vector<Observable>{x}) {}
    UnbinnedDataSet(std::initializer_list<Observable> obs) : UnbinnedDataSet(std::vector<Observable>(obs)) {}
    explicit UnbinnedDataSet(const std::vector<Observable> &obs) : DataSet(obs), cols_(obs.size()) {}
    size_t getNumEvents() const override { return cols_.empty() ? 0 : cols_[0].size(); }
    // the current values of the observables as one event (DataSet::addEvent, src/goofit/DataSet.cpp:57-80)
    void addEvent() override {
        for(auto &o : obs_)
            if(o.getValue() < o.getLowerLimit() || o.getValue() > o.getUpperLimit())
                throw GeneralError("Observable " + o.getName() + " out of range");
        for(size_t k = 0; k < obs_.size(); ++k)
            cols_[k].push_back(obs_[k].getValue());
    }
    double getValue(const Observable &o, size_t i) const {
        for(size_t k = 0; k < obs_.size(); ++k)
            if(obs_[k].sameAs(o))
                return cols_[k].at(i);
        throw GeneralError("Invalid variable access into dataset!");
    }
    const std::vector<double> &column(const Observable &o) const {
        for(size_t k = 0; k < obs_.size(); ++k)
            if(obs_[k].sameAs(o))
                return cols_[k];
        throw GeneralError("observable " + o.getName() + " is not in the data set");
    }
};

// ---------------------------------------------------------------- PDFs
class PdfBase {
  protected:
    std::string name_;
    int op_    = 0;
    int flags_ = 0;
    int ibins_ = 0;
    std::vector<Variable> params_;
    std::vector<double> consts_;
    std::vector<Observable> obs_;
    std::vector<PdfBase *> components_;
    DataSet *data_ = nullptr;

    PdfBase(int op, const std::string &n) : name_(n), op_(op) {}
    void registerParameter(const Variable &v) { params_.push_back(v); }
    void registerConstant(double c) { consts_.push_back(c); }
    void registerObservable(const Observable &o) {
        for(auto &q : obs_)
            if(q.sameAs(o))
                return;
        obs_.push_back(o);
    }

  public:
    virtual ~PdfBase() = default;
    const std::string &getName() const { return name_; }
    void setData(DataSet *d) { data_ = d; }
    DataSet *getData() const { return data_; }
    void setIntegrationFineness(int i) { ibins_ = i; }
    void setSeparateNorm() { flags_ |= GF_FLAG_SEPARATE_NORM; }
    const std::vector<PdfBase *> &getComponents() const { return components_; }

    // PdfBase::getParameters / getObservables: own first, then the components', each once
    std::vector<Variable> getParameters() const {
        std::vector<Variable> out;
        collectParams(out);
        return out;
    }
    std::vector<Observable> getObservables() const {
        std::vector<Observable> out;
        collectObs(out);
        return out;
    }
    void collectParams(std::vector<Variable> &out) const {
        for(auto &p : params_)
            if(std::none_of(out.begin(), out.end(), [&](const Variable &q) { return q.sameAs(p); }))
                out.push_back(p);
        for(auto *c : components_)
            c->collectParams(out);
    }
    void collectObs(std::vector<Observable> &out) const {
        for(auto &o : obs_)
            if(std::none_of(out.begin(), out.end(), [&](const Observable &q) { return q.sameAs(o); }))
                out.push_back(o);
        for(auto *c : components_)
            c->collectObs(out);
    }
    // parameters without an analytic derivative in the engine (an amplitude PDF's efficiency)
    virtual void collectNondiff(std::vector<Variable> &out) const {
        for(auto *c : components_)
            c->collectNondiff(out);
    }

    // ---- flattening into gf_node records (storage owned by Flat) ----
    struct Flat {
        std::vector<gf_node> nodes;
        std::vector<std::vector<int32_t>> p, o, ch;
        std::vector<std::vector<double>> c;
        std::vector<Variable> params;
        std::vector<Observable> obs;
    };
    Flat flatten() const {
        Flat f;
        f.params = getParameters();
        f.obs    = getObservables();
        std::vector<const PdfBase *> order;
        visit(order);
        const size_t n = order.size();
        f.nodes.resize(n);
        f.p.resize(n);
        f.o.resize(n);
        f.ch.resize(n);
        f.c.resize(n);
        for(size_t i = 0; i < n; ++i) {
            const PdfBase *q = order[i];
            for(auto &v : q->params_)
                f.p[i].push_back(indexOf(f.params, v));
            for(auto &ob : q->obs_)
                f.o[i].push_back(indexOf(f.obs, ob));
            for(auto *cc : q->components_)
                f.ch[i].push_back((int32_t)(std::find(order.begin(), order.end(), cc) - order.begin()));
            f.c[i] = q->consts_;
        }
        for(size_t i = 0; i < n; ++i) {
            gf_node &g     = f.nodes[i];
            g              = gf_node{};
            g.op           = order[i]->op_;
            g.flags        = order[i]->flags_;
            g.n_params     = (int)f.p[i].size();
            g.n_consts     = (int)f.c[i].size();
            g.n_obs        = (int)f.o[i].size();
            g.n_children   = (int)f.ch[i].size();
            g.params       = f.p[i].data();
            g.consts       = f.c[i].data();
            g.obs          = f.o[i].data();
            g.children     = f.ch[i].data();
            g.integration_bins = order[i]->ibins_;
        }
        return f;
    }

  private:
    void visit(std::vector<const PdfBase *> &order) const {
        order.push_back(this);
        for(auto *c : components_)
            c->visit(order);
    }
    template <class T>
    static int32_t indexOf(const std::vector<T> &v, const T &x) {
        for(size_t i = 0; i < v.size(); ++i)
            if(v[i].sameAs(x))
                return (int32_t)i;
        throw GeneralError("internal: object not found while flattening");
    }
};

class GooPdf : public PdfBase {
  protected:
    using PdfBase::PdfBase;
};
class CombinePdf : public GooPdf {
  protected:
    using GooPdf::GooPdf;
};

// ExpPdf (include/goofit/PDFs/basic/ExpPdf.h): exp(alpha x), with an offset, or exp of a polynomial
class ExpPdf : public GooPdf {
  public:
    ExpPdf(const std::string &n, const Observable &x, const Variable &alpha) : GooPdf(GF_OP_EXP, n) {
        registerObservable(x);
        registerParameter(alpha);
    }
    ExpPdf(const std::string &n, const Observable &x, const Variable &alpha, const Variable &offset)
        : GooPdf(GF_OP_EXP_OFFSET, n) {
        registerObservable(x);
        registerParameter(offset);
        registerParameter(alpha);
    }
    ExpPdf(const std::string &n, const Observable &x, const std::vector<Variable> &weights)
        : GooPdf(GF_OP_EXP_POLY, n) {
        if(weights.empty())
            throw GeneralError("Weights are empty!");
        registerObservable(x);
        for(auto &w : weights)
            registerParameter(w);
    }
    ExpPdf(const std::string &n, const Observable &x, const std::vector<Variable> &weights, const Variable &offset)
        : GooPdf(GF_OP_EXP_POLY_OFFSET, n) {
        if(weights.empty())
            throw GeneralError("Weights are empty!");
        registerObservable(x);
        registerParameter(offset);
        for(auto &w : weights)
            registerParameter(w);
    }
};

class GaussianPdf : public GooPdf {
  public:
    GaussianPdf(const std::string &n, const Observable &x, const Variable &mean, const Variable &sigma)
        : GooPdf(GF_OP_GAUSSIAN, n) {
        registerObservable(x);
        registerParameter(mean);
        registerParameter(sigma);
    }
};

// PolynomialPdf: one observable (optionally with an offset), or the multivariate form
class PolynomialPdf : public GooPdf {
  public:
    PolynomialPdf(const std::string &n, const Observable &x, const std::vector<Variable> &weights,
                  unsigned int lowestDegree = 0)
        : GooPdf(GF_OP_POLYNOMIAL, n) {
        registerObservable(x);
        registerConstant(lowestDegree);
        for(auto &w : weights)
            registerParameter(w);
    }
    PolynomialPdf(const std::string &n, const Observable &x, const std::vector<Variable> &weights, const Variable &x0,
                  unsigned int lowestDegree = 0)
        : GooPdf(GF_OP_POLYNOMIAL_OFFSET, n) {
        registerObservable(x);
        registerConstant(lowestDegree);
        for(auto &w : weights)
            registerParameter(w);
        registerParameter(x0);
    }
    PolynomialPdf(const std::string &n, const std::vector<Observable> &obses, std::vector<Variable> coeffs,
                  std::vector<Variable> offsets, unsigned int maxDegree = 1)
        : GooPdf(GF_OP_MULTIPOLYNOMIAL, n) {
        unsigned int numParameters = 1;
        registerConstant(maxDegree);
        for(size_t i = 0; i < obses.size(); ++i) {
            registerObservable(obses[i]);
            numParameters *= maxDegree + 1 + (unsigned)i;
            registerConstant(maxDegree + 1 + i);
        }
        for(size_t i = obs_.size(); i > 1; --i)
            numParameters /= (unsigned)i;
        while(numParameters > coeffs.size())
            coeffs.emplace_back(n + "_extra_coeff_" + std::to_string(coeffs.size()), 0.0);
        while(offsets.size() < obses.size())
            offsets.emplace_back(n + "_extra_offset_" + std::to_string(offsets.size()), 0.0);
        for(auto &o : offsets)
            registerParameter(o);
        for(auto &c : coeffs)
            registerParameter(c);
    }
};

class AddPdf : public CombinePdf {
  public:
    AddPdf(const std::string &n, const Variable &frac, PdfBase *func1, PdfBase *func2) : CombinePdf(GF_OP_ADD, n) {
        components_ = {func1, func2};
        registerParameter(frac);
        for(auto &o : getObservables())
            registerObservable(o);
    }
    AddPdf(const std::string &n, const std::vector<Variable> &weights, const std::vector<PdfBase *> &comps)
        : CombinePdf(weights.size() == comps.size() ? GF_OP_ADD_EXT : GF_OP_ADD, n) {
        if(weights.size() != comps.size() && weights.size() + 1 != comps.size())
            throw GeneralError("Size of weights (+1) != comps");
        components_ = comps;
        for(auto &w : weights)
            registerParameter(w);
        for(auto &o : getObservables())
            registerObservable(o);
    }
};

class ProdPdf : public CombinePdf {
  public:
    ProdPdf(const std::string &n, const std::vector<PdfBase *> &comps) : CombinePdf(GF_OP_PROD, n) {
        components_ = comps;
        for(auto &o : getObservables())
            registerObservable(o);
        registerConstant(comps.size());
    }
};

class ConvolutionPdf : public CombinePdf {
  public:
    ConvolutionPdf(const std::string &n, const Observable &x, GooPdf *model, GooPdf *resolution)
        : CombinePdf(GF_OP_CONVOLUTION, n) {
        registerObservable(x);
        components_ = {model, resolution};
        for(auto &o : getObservables())
            registerObservable(o);
        consts_ = {-10.0, 10.0, 0.01, 0.0};
    }
    void setIntegrationConstants(fptype lo, fptype hi, fptype step) {
        consts_[0] = lo;
        consts_[1] = hi;
        consts_[2] = step;
    }
};

// ---- Dalitz plots ----
enum DaughterPair { PAIR_12 = 0, PAIR_13, PAIR_23 };

class ResonancePdf : public GooPdf {
  public:
    Variable amp_real, amp_imag;

  protected:
    ResonancePdf(int op, const std::string &n, const Variable &ar, const Variable &ai)
        : GooPdf(op, n), amp_real(ar), amp_imag(ai) {}
};

namespace Resonances {
class RBW : public ResonancePdf {
  public:
    RBW(const std::string &n, const Variable &ar, const Variable &ai, const Variable &mass, const Variable &width,
        unsigned int sp, unsigned int cyc, bool norm = true, bool sym = false)
        : ResonancePdf(GF_OP_RES_RBW, n, ar, ai) {
        registerParameter(mass);
        registerParameter(width);
        registerConstant(sp);
        registerConstant(cyc);
        registerConstant(norm ? 1 : 0);
        registerConstant(sym ? 1 : 0);
    }
};
class NonRes : public ResonancePdf {
  public:
    NonRes(const std::string &n, const Variable &ar, const Variable &ai) : ResonancePdf(GF_OP_RES_NONRES, n, ar, ai) {}
};
} // namespace Resonances

struct DecayInfo3 {
    fptype motherMass = 0, daug1Mass = 0, daug2Mass = 0, daug3Mass = 0, meson_radius = 0, mother_meson_radius = 0;
    std::vector<ResonancePdf *> resonances;
};

// Amp3Body (include/goofit/PDFs/physics/Amp3Body.h): |sum_r c_r B_r|^2 * eff over (m12, m13)
class Amp3Body : public GooPdf {
    GooPdf *eff_;

  public:
    Amp3Body(const std::string &n, const Observable &m12, const Observable &m13, const EventNumber &eventNumber,
             const DecayInfo3 &decay, GooPdf *eff)
        : GooPdf(GF_OP_AMP3BODY, n), eff_(eff) {
        if(!eff)
            throw GeneralError("Amp3Body needs an efficiency function");
        registerObservable(m12);
        registerObservable(m13);
        registerObservable(eventNumber);
        registerConstant(decay.resonances.size());
        static int cacheCount = 0;
        registerConstant(cacheCount++);
        for(double c : {decay.motherMass, decay.daug1Mass, decay.daug2Mass, decay.daug3Mass, decay.meson_radius,
                        decay.mother_meson_radius})
            registerConstant(c);
        for(auto *r : decay.resonances) {
            registerParameter(r->amp_real);
            registerParameter(r->amp_imag);
            components_.push_back(r);
        }
        components_.push_back(eff);
        setSeparateNorm();
    }
    void collectNondiff(std::vector<Variable> &out) const override { eff_->collectParams(out); }
};

// ---------------------------------------------------------------- fitting
// FitManagerMinuit2 surface (include/goofit/fitting/FitManagerMinuit2.h) on the engine's MIGRAD.
class FitManager {
    PdfBase *pdf_;
    int precision_ = GF_MIXED;
    int verbosity_ = 3, strategy_ = 1, maxfcn_ = 0;
    double tolerance_ = 0.1;
    bool valid_       = false;
    gf_fit_result last_{};

  public:
    explicit FitManager(PdfBase *pdf) : pdf_(pdf) {}
    void setMaxCalls(int n = 0) { maxfcn_ = n; }
    void setVerbosity(int v) { verbosity_ = v; }
    void setStrategy(int s) { strategy_ = s; }
    void setTolerance(double t) { tolerance_ = t; }
    // GF_MIXED (FP32 events, FP64 reductions; the default) or GF_FP64
    void setPrecision(int p) { precision_ = p; }
    operator bool() const { return valid_; }
    operator int() const { return valid_ ? 0 : 51; }
    const gf_fit_result &result() const { return last_; }

    gf_fit_result fit() {
        auto *data = dynamic_cast<UnbinnedDataSet *>(pdf_->getData());
        if(!data)
            throw GeneralError("FitManager: the PDF needs an UnbinnedDataSet (setData)");
        PdfBase::Flat f = pdf_->flatten();
        const int np    = (int)f.params.size();
        std::vector<Variable> nondiff;
        pdf_->collectNondiff(nondiff);
        auto isNondiff = [&](const Variable &v) {
            return std::any_of(nondiff.begin(), nondiff.end(), [&](const Variable &q) { return q.sameAs(v); });
        };
        std::vector<int32_t> mask(np), fixed(np), limited(np);
        std::vector<double> x0(np), err(np), lo(np), hi(np), x(np), e(np);
        bool analytic = true;
        for(int i = 0; i < np; ++i) {
            const Variable &v = f.params[i];
            fixed[i]          = v.IsFixed() ? 1 : 0;
            mask[i]           = (!v.IsFixed() && !isNondiff(v)) ? 1 : 0;
            if(!v.IsFixed() && isNondiff(v))
                analytic = false;
            limited[i] = (!v.IsFixed() && v.getLowerLimit() != v.getUpperLimit()) ? 1 : 0;
            x0[i]      = v.getValue() - v.state()->blind;
            err[i]     = v.getError();
            lo[i]      = v.getLowerLimit() - v.state()->blind;
            hi[i]      = v.getUpperLimit() - v.state()->blind;
        }
        std::vector<gf_observable> ob(f.obs.size());
        for(size_t k = 0; k < f.obs.size(); ++k)
            ob[k] = gf_observable{f.obs[k].getLowerLimit(), f.obs[k].getUpperLimit(), f.obs[k].getNumBins(),
                                  f.obs[k].isEventNumber() ? 1 : 0};
        std::vector<double> soa;
        const int64_t n = (int64_t)data->getNumEvents();
        for(auto &o : f.obs) {
            const auto &c = data->column(o);
            soa.insert(soa.end(), c.begin(), c.end());
        }
        gf_engine *eng = nullptr;
        detail::check(gf_engine_create(&eng, 0, precision_), nullptr);
        std::unique_ptr<gf_engine, int (*)(gf_engine *)> guard(eng, gf_engine_destroy);
        detail::check(gf_set_tree(eng, f.nodes.data(), (int)f.nodes.size(), ob.data(), (int)ob.size(), np, mask.data()),
                      eng);
        detail::check(gf_upload_events(eng, 0, soa.data(), n), eng);
        gf_fit_options o{};
        o.err        = err.data();
        o.lo         = lo.data();
        o.hi         = hi.data();
        o.limited    = limited.data();
        o.fixed      = fixed.data();
        o.up         = 0.5;
        o.tolerance  = tolerance_;
        o.strategy   = strategy_;
        o.maxfcn     = maxfcn_;
        o.use_grad   = analytic ? 1 : 0;
        o.fnoise_rel = precision_ == GF_MIXED ? std::min(2e-8, std::max(1e-9, 1.5e-6 / std::sqrt(std::max<double>(1, n))))
                                              : 0.0;
        detail::check(gf_fit(eng, 0, &o, x0.data(), x.data(), e.data(), &last_), eng);
        for(int i = 0; i < np; ++i) {
            Variable v = f.params[i];
            v.setValue(x[i] + v.state()->blind);
            v.setError(e[i]);
        }
        valid_ = last_.valid != 0;
        if(verbosity_ > 0) {
            std::printf("MIGRAD %s: fmin=%.10g edm=%.3g nfcn=%d\n", valid_ ? "valid" : "INVALID", last_.fmin, last_.edm,
                        last_.nfcn);
            for(auto &v : f.params)
                if(!v.IsFixed())
                    std::printf("   %s: %.8g +/- %.3g\n", v.getName().c_str(), v.getValue(), v.getError());
        }
        return last_;
    }
};
using FitManagerMinuit2 = FitManager;

} // namespace GooFit
