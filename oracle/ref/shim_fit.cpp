// Project-written link stand-ins for the Minuit2 side of the reference (FitManagerMinuit2.cpp, Params.cpp,
// FCN.cpp are not compiled: Minuit2 is an empty submodule of the reference).  PdfBase::fit names these
// symbols; nothing in the CPU build of the reference's likelihood calls them, and each fails loudly if it is.
#include <goofit/Error.h>
#include <goofit/fitting/FCN.h>
#include <goofit/fitting/FitManagerMinuit2.h>
#include <goofit/fitting/Params.h>

namespace GooFit {

Params::Params(PdfBase &pdf)
    : pdf_(&pdf), num_(0) {}
void Params::SetGooFitParams(const Minuit2::MnUserParameterState &) {}
auto Params::make_minuit_vector() const -> std::vector<double> { return {}; }
void Params::from_minuit_vector(const std::vector<double> &, bool) {}

FCN::FCN(Params &params)
    : params_(&params) {}
auto FCN::operator()(const std::vector<double> &) const -> double {
    throw GeneralError("the CPU build of the reference has no minimiser");
}
auto FCN::operator()() const -> double { throw GeneralError("the CPU build of the reference has no minimiser"); }
auto FCN::GetParams() -> Params * { return params_; }

FitManagerMinuit2::FitManagerMinuit2(PdfBase *dat)
    : upar_(*dat), fcn_(upar_) {}
auto FitManagerMinuit2::fit() -> ROOT::Minuit2::FunctionMinimum {
    throw GeneralError("the CPU build of the reference has no minimiser");
}
auto FitManagerMinuit2::getMnScan() -> ROOT::Minuit2::MnScan { return {}; }

} // namespace GooFit

// ---- the events the phase-space stand-in returns ----
#include <mcbooster/Generate.h>

namespace {
std::vector<mcbooster::GReal_t> g_events;
mcbooster::GLong_t g_n      = 0;
mcbooster::GInt_t g_ndaught = 0;
} // namespace

void mcbooster::SetGeneratedEvents(const GReal_t *p4, GLong_t n, GInt_t ndaughters) {
    g_events.assign(p4, p4 + (size_t)n * ndaughters * 4);
    g_n       = n;
    g_ndaught = ndaughters;
}

void mcbooster::PhaseSpace::Generate(const Vector4R &) {
    if(g_n <= 0 || g_ndaught != (GInt_t)masses_.size())
        throw std::runtime_error("phase-space stand-in: no supplied events for this decay");
    daughters_.assign(g_ndaught, Particles_d(g_n));
    for(GLong_t i = 0; i < g_n; ++i)
        for(GInt_t k = 0; k < g_ndaught; ++k) {
            const GReal_t *p = &g_events[((size_t)i * g_ndaught + k) * 4];
            daughters_[k][i] = Vector4R(p[0], p[1], p[2], p[3]);
        }
}
