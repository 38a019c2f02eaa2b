// GooFit-compatible C++ host API over the likelihood engine's C ABI (gfengine.h).
//
// Header-only, C++17.  The class names, constructor argument orders and the methods a fit uses follow the
// reference's C++ API (include/goofit/Variable.h, UnbinnedDataSet.h, BinnedDataSet.h, FitControl.h,
// PDFs/basic/*.h, PDFs/combine/*.h, PDFs/physics/Amp3Body.h, Amp4Body.h, Amplitude.h, SpinFactors.h,
// lineshapes/RBW.h and SBW.h, fitting/FitManagerMinuit2.h), so that user code of the form
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
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
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
    void setFitterIndex(int i) { s_->fitter_index = i; }
    Variable &operator=(double v) {
        s_->value = v;
        return *this;
    }
};

// ---------------------------------------------------------------- data
class DataSet {
  protected:
    std::vector<Observable> obs_;
    std::string name_;

    // DataSet::checkAllVars (src/goofit/DataSet.cpp:72-77): every observable inside its limits
    void checkAllVars() const {
        for(auto &o : obs_)
            if(o.getValue() < o.getLowerLimit() || o.getValue() > o.getUpperLimit())
                throw GeneralError("Observable " + o.getName() + " out of range");
    }

  public:
    explicit DataSet(const std::vector<Observable> &obs, const std::string &n = "") : obs_(obs), name_(n) {}
    virtual ~DataSet() = default;
    const std::vector<Observable> &getObservables() const { return obs_; }
    const std::string &getName() const { return name_; }
    size_t numVariables() const { return obs_.size(); }
    size_t indexOfVariable(const Observable &o) const {
        for(size_t k = 0; k < obs_.size(); ++k)
            if(obs_[k].sameAs(o))
                return k;
        throw GeneralError("observable " + o.getName() + " is not in the data set");
    }
    virtual size_t getNumEvents() const = 0;
    virtual void addEvent() = 0;
    virtual void addWeightedEvent(double weight) = 0;
};

class UnbinnedDataSet : public DataSet {
    std::vector<std::vector<double>> cols_;

  public:
    UnbinnedDataSet(const Observable &x) : UnbinnedDataSet(std::vector<Observable>{x}) {}
    UnbinnedDataSet(std::initializer_list<Observable> obs) : UnbinnedDataSet(std::vector<Observable>(obs)) {}
    explicit UnbinnedDataSet(const std::vector<Observable> &obs, const std::string &n = "")
        : DataSet(obs, n), cols_(obs.size()) {}
    size_t getNumEvents() const override { return cols_.empty() ? 0 : cols_[0].size(); }
    // the current values of the observables as one event (DataSet::addEvent, src/goofit/DataSet.cpp:57-80)
    void addEvent() override {
        checkAllVars();
        for(size_t k = 0; k < obs_.size(); ++k)
            cols_[k].push_back(obs_[k].getValue());
    }
    // UnbinnedDataSet::addWeightedEvent (src/goofit/UnbinnedDataSet.cpp): not supported
    void addWeightedEvent(double) override {
        throw GeneralError("Weighted events are not supported for the UnbinnedDataSet");
    }
    // one event from explicit values, in the data set's observable order
    void addEvent(const std::vector<double> &values) {
        if(values.size() != obs_.size())
            throw GeneralError("addEvent: wrong number of values");
        for(size_t k = 0; k < obs_.size(); ++k)
            obs_[k].setValue(values[k]);
        addEvent();
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

// BinnedDataSet (include/goofit/BinnedDataSet.h, src/goofit/BinnedDataSet.cpp): counts on the observables' bin
// grid, global bin = sum_i local_i * prod_{j<i} nbins_j.
class BinnedDataSet : public DataSet {
    std::vector<size_t> binsizes_;
    std::vector<double> binvalues_, binerrors_;
    size_t numEventsAdded_ = 0;

    void collectBins() {
        binsizes_.clear();
        for(auto &o : obs_)
            binsizes_.push_back((size_t)o.getNumBins());
        binvalues_.assign(getNumBins(), 0.0);
    }

  public:
    BinnedDataSet(const Observable &x, const std::string &n = "") : BinnedDataSet(std::vector<Observable>{x}, n) {}
    BinnedDataSet(std::initializer_list<Observable> obs, const std::string &n = "")
        : BinnedDataSet(std::vector<Observable>(obs), n) {}
    explicit BinnedDataSet(const std::vector<Observable> &obs, const std::string &n = "") : DataSet(obs, n) {
        collectBins();
    }
    size_t getNumEvents() const override { return numEventsAdded_; }
    size_t getNumBins() const {
        size_t r = 1;
        for(size_t b : binsizes_)
            r *= b;
        return r;
    }
    std::vector<size_t> getDiminsions() const { return binsizes_; }
    double getBinSize(size_t ivar) const {
        return (obs_.at(ivar).getUpperLimit() - obs_[ivar].getLowerLimit()) / (double)binsizes_[ivar];
    }
    // values clamped into the limits, then floor((v - lo) / bin size) (BinnedDataSet::convertValuesToBins)
    std::vector<size_t> convertValuesToBins(const std::vector<double> &vals) const {
        if(vals.size() != obs_.size())
            throw GeneralError("Incorrect number of values for the data set's variables");
        std::vector<size_t> out;
        for(size_t i = 0; i < obs_.size(); ++i) {
            const double v = std::min(std::max(vals[i], obs_[i].getLowerLimit()), obs_[i].getUpperLimit());
            out.push_back((size_t)std::floor((v - obs_[i].getLowerLimit()) / getBinSize(i)));
        }
        return out;
    }
    size_t localToGlobal(const std::vector<size_t> &locals) const {
        size_t prior = 1, ret = 0;
        for(size_t i = 0; i < obs_.size(); ++i) {
            ret += locals[i] * prior;
            prior *= binsizes_[i];
        }
        return ret;
    }
    std::vector<size_t> globalToLocal(size_t global) const {
        std::vector<size_t> locals;
        for(size_t i = 0; i < obs_.size(); ++i) {
            locals.push_back(global % binsizes_[i]);
            global /= binsizes_[i];
        }
        return locals;
    }
    size_t getBinNumber() const {
        std::vector<double> vals;
        for(auto &o : obs_)
            vals.push_back(o.getValue());
        return localToGlobal(convertValuesToBins(vals));
    }
    void addEvent() override { addWeightedEvent(1.0); }
    void addWeightedEvent(double weight) override {
        checkAllVars();
        const size_t b = getBinNumber();
        if(b >= binvalues_.size())
            throw GeneralError("BinnedDataSet: an observable at its upper limit falls outside the last bin");
        binvalues_[b] += weight;
        ++numEventsAdded_;
    }
    double getBinContent(size_t bin) const { return binvalues_.at(bin); }
    void setBinContent(size_t bin, double value) { binvalues_.at(bin) = value; }
    double getBinCenter(size_t ivar, size_t bin) const {
        return getBinSize(ivar) * ((double)globalToLocal(bin).at(ivar) + 0.5) + obs_[ivar].getLowerLimit();
    }
    double getBinCenter(const Observable &o, size_t bin) const { return getBinCenter(indexOfVariable(o), bin); }
    double getBinVolume(size_t) const {
        double r = 1;
        for(size_t i = 0; i < obs_.size(); ++i)
            r *= getBinSize(i);
        return r;
    }
    // sqrt(content) until the first setBinError, which switches every bin to explicit errors (zero where unset)
    double getBinError(size_t bin) const {
        return binerrors_.empty() ? std::sqrt(binvalues_.at(bin)) : binerrors_.at(bin);
    }
    void setBinError(size_t bin, double value) {
        if(binerrors_.empty())
            binerrors_.assign(binvalues_.size(), 0.0);
        binerrors_.at(bin) = value;
    }
    // the sum of the bin contents (summed in double; the reference accumulates into an int)
    double getNumWeightedEvents() const {
        double s = 0;
        for(double v : binvalues_)
            s += v;
        return s;
    }
    // the engine's binned event layout (PdfBase::setData, src/PDFs/PdfBase.cu:439-495): per bin the centres of
    // `obs` in that order, then the content, then the volume (or, with errors = true, the bin error); SoA
    std::vector<double> engineColumns(const std::vector<Observable> &obs, bool errors) const {
        const size_t n = getNumBins();
        std::vector<double> soa;
        soa.reserve((obs.size() + 2) * n);
        for(auto &o : obs) {
            const size_t iv = indexOfVariable(o);
            for(size_t b = 0; b < n; ++b)
                soa.push_back(getBinCenter(iv, b));
        }
        for(size_t b = 0; b < n; ++b)
            soa.push_back(binvalues_[b]);
        for(size_t b = 0; b < n; ++b)
            soa.push_back(errors ? getBinError(b) : getBinVolume(b));
        return soa;
    }
};

// ---------------------------------------------------------------- fit controls
// include/goofit/FitControl.h:40-76: what the fit minimises (enum gf_fit_metric)
class FitControl {
  protected:
    int metric_;
    bool binned_, errors_;
    FitControl(int metric, bool binned, bool errors) : metric_(metric), binned_(binned), errors_(errors) {}

  public:
    virtual ~FitControl() = default;
    int metric() const { return metric_; }
    bool binnedFit() const { return binned_; }
    bool binErrors() const { return errors_; }
};
class UnbinnedNllFit : public FitControl {
  public:
    UnbinnedNllFit() : FitControl(GF_FIT_UNBINNED_NLL, false, false) {}
};
class BinnedNllFit : public FitControl {
  public:
    BinnedNllFit() : FitControl(GF_FIT_BINNED_NLL, true, false) {}
};
class BinnedErrorFit : public FitControl {
  public:
    BinnedErrorFit() : FitControl(GF_FIT_BINNED_ERROR, true, true) {}
};
class BinnedChisqFit : public FitControl {
  public:
    BinnedChisqFit() : FitControl(GF_FIT_BINNED_CHISQ, true, false) {}
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
    std::shared_ptr<FitControl> fitControl_ = std::make_shared<UnbinnedNllFit>();

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
    // PdfBase::setData: a BinnedDataSet switches an unbinned fit control to BinnedNllFit
    // (src/PDFs/PdfBase.cu:444-445)
    void setData(DataSet *d) {
        data_ = d;
        if(dynamic_cast<BinnedDataSet *>(d) && !fitControl_->binnedFit())
            fitControl_ = std::make_shared<BinnedNllFit>();
    }
    DataSet *getData() const { return data_; }
    void setFitControl(std::shared_ptr<FitControl> fc) { fitControl_ = std::move(fc); }
    const std::shared_ptr<FitControl> &getFitControl() const { return fitControl_; }
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
        std::vector<const PdfBase *> order; // the PDF object behind each node
    };
    // per-node engine state beyond the tree (Amp4Body: its normalisation events)
    virtual void engineSetup(gf_engine *, int) const {}
    Flat flatten() const {
        Flat f;
        f.params = getParameters();
        f.obs    = getObservables();
        std::vector<const PdfBase *> order;
        visit(order);
        f.order        = order;
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

// ---------------------------------------------------------------- 4-body amplitudes
// include/goofit/PDFs/physics/SpinFactors.h:18-35
enum class SF_4Body : int {
    DtoPP1_PtoSP2_StoP3P4 = 0,
    DtoPP1_PtoVP2_VtoP3P4,
    DtoV1V2_V1toP1P2_V2toP3P4_S,
    DtoV1V2_V1toP1P2_V2toP3P4_P,
    DtoV1V2_V1toP1P2_V2toP3P4_D,
    DtoAP1_AtoVP2_VtoP3P4,
    DtoAP1_AtoVP2Dwave_VtoP3P4,
    DtoVS_VtoP1P2_StoP3P4,
    DtoV1P1_V1toV2P2_V2toP3P4,
    DtoAP1_AtoSP2_StoP3P4,
    DtoTP1_TtoVP2_VtoP3P4,
    FF_12_34_L1,
    FF_12_34_L2,
    FF_123_4_L1,
    FF_123_4_L2,
    ONE
};
// form factor of a line shape (include/goofit/PDFs/physics/lineshapes/Lineshape.h:18)
enum class FF : unsigned int { One = 0, BL, BL_Prime, BL2 };
// daughter combination of a line shape (include/goofit/PDFs/physics/DalitzPlotHelpers.h:58-77)
enum DP4Pair {
    M_12 = 0,
    M_34,
    M_13,
    M_14,
    M_23,
    M_24,
    M_12_3,
    M_13_2,
    M_23_1,
    M_12_4,
    M_14_2,
    M_24_1,
    M_13_4,
    M_14_3,
    M_34_1,
    M_23_4,
    M_24_3,
    M_34_2
};

class AmpComponent : public GooPdf {
  protected:
    using GooPdf::GooPdf;
};

// SpinFactor (src/PDFs/physics/SpinFactors.cu:586-664): consts [kind, mD0, P0, P1, P2, P3]
class SpinFactor : public AmpComponent {
  public:
    SpinFactor(const std::string &n, SF_4Body SF, fptype mD0, unsigned int P0, unsigned int P1, unsigned int P2,
               unsigned int P3)
        : AmpComponent(GF_OP_SPINFACTOR, n) {
        for(double c : {(double)(int)SF, mD0, (double)P0, (double)P1, (double)P2, (double)P3})
            registerConstant(c);
    }
    SpinFactor(const std::string &n, SF_4Body SF, unsigned int P0, unsigned int P1, unsigned int P2, unsigned int P3)
        : SpinFactor(n, SF, 1.86484, P0, P1, P2, P3) {}
};

// Lineshape (include/goofit/PDFs/physics/lineshapes/Lineshape.h): params [mass, width],
// consts [Mpair, L, form factor, radius]
class Lineshape : public AmpComponent {
  protected:
    Lineshape(int op, const std::string &n, const Variable &mass, const Variable &width, unsigned int L,
              unsigned int Mpair, FF FormFac, fptype radius)
        : AmpComponent(op, n) {
        registerParameter(mass);
        registerParameter(width);
        for(double c : {(double)Mpair, (double)L, (double)(unsigned)FormFac, radius})
            registerConstant(c);
    }
};

namespace Lineshapes {
// relativistic Breit-Wigner with a mass-dependent width (src/PDFs/physics/lineshapes/BW.cu:14-68)
class RBW : public Lineshape {
  public:
    RBW(const std::string &n, const Variable &mass, const Variable &width, unsigned int L, unsigned int Mpair,
        FF FormFac = FF::BL_Prime, fptype radius = 1.5)
        : Lineshape(GF_OP_LS_RBW, n, mass, width, L, Mpair, FormFac, radius) {}
};
// Breit-Wigner with a constant width (src/PDFs/physics/lineshapes/BW.cu:70-110)
class SBW : public Lineshape {
  public:
    SBW(const std::string &n, const Variable &mass, const Variable &width, unsigned int L, unsigned int Mpair,
        FF FormFac = FF::BL_Prime, fptype radius = 1.5)
        : Lineshape(GF_OP_LS_SBW, n, mass, width, L, Mpair, FormFac, radius) {}
};
} // namespace Lineshapes

// Amplitude (src/PDFs/physics/Amplitude.cu:11-31): the sum over nPerm permutations of the products of its line
// shapes and spin factors, divided by sqrt(nPerm).  consts [nPerm, nLS, nSF], children [LS..., SF...]; the
// complex coefficient (ar, ai) is a parameter of the Amp4Body that holds the amplitude.
class Amplitude : public AmpComponent {
    Variable ar_, ai_;
    std::vector<Lineshape *> ls_;
    std::vector<SpinFactor *> sf_;

  public:
    Amplitude(const std::string &uniqueDecayStr, const Variable &ar, const Variable &ai,
              const std::vector<Lineshape *> &LS, const std::vector<SpinFactor *> &SF, unsigned int nPerm = 1)
        : AmpComponent(GF_OP_AMPLITUDE, uniqueDecayStr), ar_(ar), ai_(ai), ls_(LS), sf_(SF) {
        if(nPerm == 0 || LS.size() % nPerm || SF.size() % nPerm)
            throw GeneralError("Amplitude " + uniqueDecayStr +
                               ": line shape and spin factor counts must be multiples of nPerm");
        for(auto *l : LS)
            components_.push_back(l);
        for(auto *s : SF)
            components_.push_back(s);
        for(double c : {(double)nPerm, (double)LS.size(), (double)SF.size()})
            registerConstant(c);
    }
    const Variable &getAmpReal() const { return ar_; }
    const Variable &getAmpImag() const { return ai_; }
    std::vector<Lineshape *> getLineShapes() const { return ls_; }
    std::vector<SpinFactor *> getSpinFactors() const { return sf_; }
};

// include/goofit/PDFs/physics/DalitzPlotHelpers.h:114-120; particle_masses = {M, m1, m2, m3, m4}
struct DecayInfo4 {
    std::vector<fptype> particle_masses;
    fptype meson_radius = 1.5;
    std::vector<Amplitude *> amplitudes;
    std::vector<Amplitude *> amplitudes_B;
};

namespace detail {
struct P4 {
    double x, y, z, e;
};
inline P4 operator+(const P4 &a, const P4 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.e + b.e}; }
inline double mdot(const P4 &a, const P4 &b) { return a.e * b.e - (a.x * b.x + a.y * b.y + a.z * b.z); }
inline double dot3(const P4 &a, const P4 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double d3mag(const P4 &a) { return std::sqrt(dot3(a, a)); }
inline P4 cross3(const P4 &a, const P4 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0};
}
inline P4 scale3(const P4 &a, double s) { return {a.x * s, a.y * s, a.z * s, 0.0}; }
inline P4 div3(const P4 &a, double s) { return {a.x / s, a.y / s, a.z / s, 0.0}; }

// cosine of the helicity angle of d in the rest frame of q, against the direction of p (MCBooster's
// EvtGen-style decayAngle, as Dim5 uses it: include/goofit/PDFs/physics/detail/Dim5.h:19-111)
inline double cosHelicity(const P4 &p, const P4 &q, const P4 &d) {
    const double pd = mdot(p, d), pq = mdot(p, q), qd = mdot(q, d);
    const double mp2 = mdot(p, p), mq2 = mdot(q, q), md2 = mdot(d, d);
    return (pd * mq2 - pq * qd) / std::sqrt((pq * pq - mq2 * mp2) * (qd * qd - mq2 * md2));
}
// the angle between the decay planes (d1, d2) and (h1, h2), signed by the direction of h1 + h2
inline double planeAngle(const P4 &d1, const P4 &d2, const P4 &h1, const P4 &h2) {
    const P4 d1n = div3(d1, d3mag(d1)), d2n = div3(d2, d3mag(d2));
    const P4 h1n = div3(h1, d3mag(h1)), h2n = div3(h2, d3mag(h2));
    const P4 h12  = h1 + h2;
    const P4 h12n = scale3(h12, 1.0 / d3mag(h12));
    P4 n1         = cross3(d1n, d2n);
    P4 n2         = cross3(h1n, h2n);
    n1            = scale3(n1, 1.0 / d3mag(n1));
    n2            = scale3(n2, 1.0 / d3mag(n2));
    const P4 n3   = cross3(n1, n2);
    const double phi = std::acos(dot3(n1, n2));
    return dot3(n3, h12n) < 0 ? -phi : phi;
}
// four daughter 4-vectors -> (m12, m34, cos12, cos34, phi), the Amp4Body observables
inline void dim5(const P4 *p, double out[5]) {
    const P4 pm  = p[0] + p[1] + p[2] + p[3];
    const P4 p01 = p[0] + p[1], p23 = p[2] + p[3];
    out[0]       = std::sqrt(mdot(p01, p01));
    out[1]       = std::sqrt(mdot(p23, p23));
    out[2]       = cosHelicity(pm, p01, p[0]);
    out[3]       = cosHelicity(pm, p23, p[2]);
    out[4]       = planeAngle(p[0], p[1], p[2], p[3]);
}

inline double breakupMomentum(double a, double b, double c) {
    const double x = (a - b - c) * (a + b + c) * (a - b + c) * (a + b - c);
    return std::sqrt(std::max(x, 0.0)) / (2.0 * a);
}
inline P4 boost(const P4 &p, double bx, double by, double bz) {
    const double b2 = bx * bx + by * by + bz * bz;
    const double g  = 1.0 / std::sqrt(1.0 - b2);
    const double bp = bx * p.x + by * p.y + bz * p.z;
    const double g2 = b2 > 0 ? (g - 1.0) / b2 : 0.0;
    const double c  = g2 * bp + g * p.e;
    return {p.x + c * bx, p.y + c * by, p.z + c * bz, g * (p.e + bp)};
}

// Flat phase space of M -> masses (parent at rest; the generator Amp4Body uses for its normalisation events in
// place of MCBooster's PhaseSpace::Generate + Unweight, src/PDFs/physics/Amp4Body.cu:243-290).  The invariant
// masses of the nested subsystems (1 2), (1 2 3), ... are drawn uniformly between their limits, the event weight
// is the product of the two-body break-up momenta, and an event is kept with probability weight / (largest weight
// of its batch); momenta follow from isotropic two-body decays in each subsystem's rest frame, boosted back to
// the parent frame.  Calls sink(const P4 *daughters) for each of the n kept events.
template <class Sink>
void phaseSpace(double M, const std::vector<double> &masses, size_t n, std::mt19937_64 &rng, Sink sink) {
    const size_t k = masses.size();
    double msum    = 0;
    for(double m : masses)
        msum += m;
    if(k < 2 || M <= msum)
        throw GeneralError("phase space is empty");
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const double tecm = M - msum;
    std::vector<double> cum(k);
    cum[0] = masses[0];
    for(size_t j = 1; j < k; ++j)
        cum[j] = cum[j - 1] + masses[j];
    const double twopi = 6.283185307179586476925286766559;
    auto isotropic     = [&](double mag) {
        const double cost = -1.0 + 2.0 * U(rng), phi = twopi * U(rng);
        const double sint = std::sqrt(1.0 - cost * cost);
        return P4{mag * sint * std::cos(phi), mag * sint * std::sin(phi), mag * cost, 0.0};
    };
    size_t have = 0;
    std::vector<double> inv, pd, w, r(k);
    std::vector<P4> p(k);
    while(have < n) {
        const size_t m = std::min<size_t>(1000000, std::max<size_t>(10000, 4 * (n - have)));
        inv.resize(m * k);
        pd.resize(m * (k - 1));
        w.resize(m);
        double wmax = 0;
        for(size_t e = 0; e < m; ++e) {
            double *iv = &inv[e * k];
            for(size_t j = 0; j + 2 < k; ++j)
                r[j] = U(rng);
            std::sort(r.begin(), r.begin() + (k - 2));
            iv[0] = masses[0];
            for(size_t j = 1; j + 1 < k; ++j)
                iv[j] = cum[j] + r[j - 1] * tecm;
            iv[k - 1] = M;
            double we = 1;
            for(size_t j = 1; j < k; ++j) {
                pd[e * (k - 1) + j - 1] = breakupMomentum(iv[j], iv[j - 1], masses[j]);
                we *= pd[e * (k - 1) + j - 1];
            }
            w[e] = we;
            wmax = std::max(wmax, we);
        }
        for(size_t e = 0; e < m && have < n; ++e) {
            if(!(U(rng) * wmax < w[e]))
                continue;
            const double *iv = &inv[e * k];
            const double *q  = &pd[e * (k - 1)];
            const P4 d       = isotropic(q[0]);
            const double d2  = dot3(d, d);
            p[0]             = {d.x, d.y, d.z, std::sqrt(masses[0] * masses[0] + d2)};
            p[1]             = {-d.x, -d.y, -d.z, std::sqrt(masses[1] * masses[1] + d2)};
            for(size_t j = 2; j < k; ++j) {
                // subsystem (0 .. j-1) recoils against particle j in the rest frame of subsystem (0 .. j)
                const P4 u        = isotropic(q[j - 1]);
                const double u2   = dot3(u, u);
                const double esub = std::sqrt(iv[j - 1] * iv[j - 1] + u2);
                for(size_t i = 0; i < j; ++i)
                    p[i] = boost(p[i], u.x / esub, u.y / esub, u.z / esub);
                p[j] = {-u.x, -u.y, -u.z, std::sqrt(masses[j] * masses[j] + u2)};
            }
            sink(p.data());
            ++have;
        }
    }
}

// n flat phase-space events of the 4-body decay as the Amp4Body variables, SoA [m12 | m34 | cos12 | cos34 | phi]
inline std::vector<double> normEvents4(const std::vector<double> &particle_masses, size_t n, uint64_t seed) {
    if(particle_masses.size() != 5)
        throw GeneralError("DecayInfo4::particle_masses must hold the parent and four daughter masses");
    std::mt19937_64 rng(seed);
    std::vector<double> soa(5 * n);
    size_t i = 0;
    phaseSpace(particle_masses[0], std::vector<double>(particle_masses.begin() + 1, particle_masses.end()), n, rng,
               [&](const P4 *d) {
                   double v[5];
                   dim5(d, v);
                   for(int c = 0; c < 5; ++c)
                       soa[c * n + i] = v[c];
                   ++i;
               });
    return soa;
}
} // namespace detail

// Amp4Body (include/goofit/PDFs/physics/Amp4Body.h, src/PDFs/physics/Amp4Body.cu:94-292):
// |sum_a c_a A_a|^2 * efficiency over (m12, m34, cos12, cos34, phi[, eventNumber]), normalised by the mean of
// |sum_a c_a A_a|^2 over MCeventsNorm flat phase-space events.  The events are generated on first use (seeded by
// normSeed), or given with setNormEvents.  Without an efficiency a constant one is used.
class Amp4Body : public GooPdf {
    GooPdf *eff_;
    std::unique_ptr<GooPdf> ownEff_;
    std::vector<fptype> masses_;
    size_t nNorm_;
    uint64_t seed_;
    mutable std::vector<double> norm_;

  public:
    Amp4Body(const std::string &n, const std::vector<Observable> &observables, const DecayInfo4 &decay, GooPdf *eff,
             unsigned int MCeventsNorm = 5000000, uint64_t normSeed = 4242)
        : GooPdf(GF_OP_AMP4BODY, n), eff_(eff), masses_(decay.particle_masses), nNorm_(MCeventsNorm),
          seed_(normSeed) {
        if(observables.size() < 5)
            throw GeneralError("Amp4Body needs the observables m12, m34, cos12, cos34, phi (and eventNumber)");
        if(masses_.size() != 5)
            throw GeneralError("DecayInfo4::particle_masses must hold the parent and four daughter masses");
        if(decay.amplitudes.empty())
            throw GeneralError("Amp4Body needs at least one amplitude");
        for(auto &o : observables)
            registerObservable(o);
        for(double m : masses_)
            registerConstant(m);
        static int cacheCount = 0;
        registerConstant(cacheCount++);
        for(auto *a : decay.amplitudes) {
            registerParameter(a->getAmpReal());
            registerParameter(a->getAmpImag());
            components_.push_back(a);
        }
        if(!eff_) {
            ownEff_.reset(new PolynomialPdf(n + "_constantEff", {observables[0], observables[1]},
                                            {Variable(n + "_constantOne", 1)},
                                            {Variable(n + "_zero0", 0), Variable(n + "_zero1", 0)}, 0));
            eff_ = ownEff_.get();
        }
        components_.push_back(eff_);
        setSeparateNorm();
    }
    // explicit normalisation events, SoA [m12 | m34 | cos12 | cos34 | phi] (5 n values)
    void setNormEvents(const std::vector<double> &soa5) {
        if(soa5.empty() || soa5.size() % 5)
            throw GeneralError("setNormEvents: expected 5 n values");
        norm_  = soa5;
        nNorm_ = soa5.size() / 5;
    }
    const std::vector<double> &getNormEvents() const {
        if(norm_.empty())
            norm_ = detail::normEvents4(masses_, nNorm_, seed_);
        return norm_;
    }
    void engineSetup(gf_engine *eng, int node) const override {
        const auto &ev = getNormEvents();
        detail::check(gf_set_norm_events(eng, node, ev.data(), (int64_t)(ev.size() / 5)), eng);
    }
    void collectNondiff(std::vector<Variable> &out) const override { eff_->collectParams(out); }
    GooPdf *getEfficiency() const { return eff_; }
};

// ---------------------------------------------------------------- fitting
// FitManagerMinuit2 surface (include/goofit/fitting/FitManagerMinuit2.h) on the engine's MIGRAD.
class FitManager {
    PdfBase *pdf_;
    int precision_ = GF_MIXED;
    int verbosity_ = 3, strategy_ = 1, maxfcn_ = 0;
    double tolerance_ = 0.1;
    bool valid_ = false, minos_ = false;
    gf_fit_result last_{};
    std::vector<std::pair<double, double>> minos_errors_;
    std::vector<double> cov_;

  public:
    explicit FitManager(PdfBase *pdf) : pdf_(pdf) {}
    void setMaxCalls(int n = 0) { maxfcn_ = n; }
    void setVerbosity(int v) { verbosity_ = v; }
    int getVerbosity() const { return verbosity_; }
    void setStrategy(int s) { strategy_ = s; }
    void setTolerance(double t) { tolerance_ = t; }
    // GF_MIXED (FP32 events, FP64 reductions; the default) or GF_FP64
    void setPrecision(int p) { precision_ = p; }
    // asymmetric MINOS errors of the free parameters after the fit (FitManagerMinuit2::fit,
    // src/goofit/FitManagerMinuit2.cpp:58-80)
    void setMinos(bool flag = true) { minos_ = flag; }
    // (negative, positive) MINOS error of each free parameter, in the order of PdfBase::getParameters
    std::vector<std::pair<double, double>> getMinosErrors() const { return minos_errors_; }
    // external covariance of the final Hesse, [n][n] over PdfBase::getParameters (zero rows for fixed ones)
    const std::vector<double> &getCovariance() const { return cov_; }
    operator bool() const { return valid_; }
    operator int() const { return valid_ ? 0 : 51; }
    const gf_fit_result &result() const { return last_; }

    gf_fit_result fit() {
        DataSet *ds = pdf_->getData();
        if(!ds)
            throw GeneralError("FitManager: the PDF has no data set (setData)");
        auto *unbinned = dynamic_cast<UnbinnedDataSet *>(ds);
        auto *binned   = dynamic_cast<BinnedDataSet *>(ds);
        if(!unbinned && !binned)
            throw GeneralError("FitManager: unsupported data set type");
        const FitControl &fc = *pdf_->getFitControl();
        if(binned && !fc.binnedFit())
            throw GeneralError("FitManager: a BinnedDataSet needs a binned fit control");
        if(unbinned && fc.binnedFit())
            throw GeneralError("FitManager: a binned fit control needs a BinnedDataSet");
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
        int64_t n = 0;
        if(binned) {
            soa = binned->engineColumns(f.obs, fc.binErrors());
            n   = (int64_t)binned->getNumBins();
        } else {
            n = (int64_t)unbinned->getNumEvents();
            for(auto &o : f.obs) {
                const auto &c = unbinned->column(o);
                soa.insert(soa.end(), c.begin(), c.end());
            }
        }
        gf_engine *eng = nullptr;
        detail::check(gf_engine_create(&eng, 0, precision_), nullptr);
        std::unique_ptr<gf_engine, int (*)(gf_engine *)> guard(eng, gf_engine_destroy);
        if(fc.metric() != GF_FIT_UNBINNED_NLL)
            detail::check(gf_set_fit_metric(eng, fc.metric()), eng);
        detail::check(gf_set_tree(eng, f.nodes.data(), (int)f.nodes.size(), ob.data(), (int)ob.size(), np, mask.data()),
                      eng);
        for(size_t i = 0; i < f.order.size(); ++i)
            f.order[i]->engineSetup(eng, (int)i);
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
        cov_.assign((size_t)np * np, 0.0);
        o.cov = cov_.data();
        detail::check(gf_fit(eng, 0, &o, x0.data(), x.data(), e.data(), &last_), eng);
        o.cov = nullptr;
        for(int i = 0; i < np; ++i) {
            Variable v = f.params[i];
            v.setValue(x[i] + v.state()->blind);
            v.setError(e[i]);
            v.setFitterIndex(i);
        }
        valid_ = last_.valid != 0;
        minos_errors_.clear();
        if(minos_ && valid_) {
            for(int i = 0; i < np; ++i)
                if(!fixed[i])
                    minos_errors_.emplace_back(minosSide(eng, o, x, e, lo, hi, limited, fixed, i, -1.0),
                                               minosSide(eng, o, x, e, lo, hi, limited, fixed, i, +1.0));
        }
        if(verbosity_ > 0) {
            std::printf("MIGRAD %s: fmin=%.10g edm=%.3g nfcn=%d\n", valid_ ? "valid" : "INVALID", last_.fmin, last_.edm,
                        last_.nfcn);
            for(auto &v : f.params)
                if(!v.IsFixed())
                    std::printf("   %s: %.8g +/- %.3g\n", v.getName().c_str(), v.getValue(), v.getError());
            if(!minos_errors_.empty()) {
                std::printf("1-sigma minos errors:\n");
                size_t k = 0;
                for(auto &v : f.params)
                    if(!v.IsFixed()) {
                        std::printf("%s: %.8g %.8g\n", v.getName().c_str(), minos_errors_[k].first,
                                    minos_errors_[k].second);
                        ++k;
                    }
            }
        }
        return last_;
    }

  private:
    // Signed MINOS error of parameter i on one side: the offset d at which the minimum over the other free
    // parameters of NLL(x_i = best + d) - fmin equals up (F. James, MINUIT's MINOS; the reference runs Minuit2's
    // MnMinos).  Each trial is a MIGRAD fit with x_i fixed, started at the best point; the offset is updated by
    // d <- d sqrt(up / delta), exact for a parabolic profile, until delta is within 1% of up.  A parameter limit
    // stops the search there.
    double minosSide(gf_engine *eng, gf_fit_options o, const std::vector<double> &best, const std::vector<double> &errs,
                     const std::vector<double> &lo, const std::vector<double> &hi, const std::vector<int32_t> &limited,
                     std::vector<int32_t> fixed, int i, double sgn) const {
        const double up = o.up;
        const int np    = (int)best.size();
        double d        = errs[i] > 0 ? errs[i] : std::max(std::fabs(o.err[i]), 1e-12);
        fixed[i]        = 1;
        o.fixed         = fixed.data();
        std::vector<double> x(np), xo(np), eo(np);
        gf_fit_result r{};
        for(int it = 0; it < 12; ++it) {
            x           = best;
            x[i]        = best[i] + sgn * d;
            bool atLimit = false;
            if(limited[i] && lo[i] < hi[i] && (x[i] <= lo[i] || x[i] >= hi[i])) {
                x[i]    = std::min(std::max(x[i], lo[i]), hi[i]);
                atLimit = true;
            }
            detail::check(gf_fit(eng, 0, &o, x.data(), xo.data(), eo.data(), &r), eng);
            const double delta = r.fmin - last_.fmin;
            if(atLimit && delta < up)
                return x[i] - best[i];
            if(!std::isfinite(delta) || delta <= 0) {
                d *= 2.0;
                continue;
            }
            if(std::fabs(delta - up) < 0.01 * up)
                return x[i] - best[i];
            d *= std::sqrt(up / delta);
        }
        return sgn * d;
    }
};
using FitManagerMinuit2 = FitManager;

} // namespace GooFit
