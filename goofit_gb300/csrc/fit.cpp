// Minimiser C ABI and the native fit loops (FitManagerMinuit2::fit,
// src/goofit/FitManagerMinuit2.cpp:31-119; FCN::operator(),
// src/goofit/FCN.cpp:18-28; Params::from_minuit_vector,
// src/goofit/Params.cpp:47-57).
#include "../../include/gfengine.h"
#include "migrad.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

struct gf_minimizer {
    std::unique_ptr<gf::Minimizer> m;
    int n = 0;
};

namespace {

gf::MinConfig makeConfig(int n, const double *x0, const double *err, const double *lo, const double *hi,
                         const int32_t *limited, const int32_t *fixed, double up, int strategy, double tol, int maxfcn,
                         int use_grad, double fnoise_rel) {
    gf::MinConfig c;
    c.n = n;
    c.x0.assign(x0, x0 + n);
    c.err.assign(n, 0.0);
    c.lo.assign(n, 0.0);
    c.hi.assign(n, 0.0);
    c.limited.assign(n, 0);
    c.fixed.assign(n, 0);
    for(int i = 0; i < n; ++i) {
        if(err)
            c.err[i] = err[i];
        if(lo)
            c.lo[i] = lo[i];
        if(hi)
            c.hi[i] = hi[i];
        if(limited)
            c.limited[i] = limited[i];
        if(fixed)
            c.fixed[i] = fixed[i];
        if(c.limited[i] == 1 && !(c.hi[i] > c.lo[i]))
            c.limited[i] = 0;
    }
    c.up       = up > 0 ? up : 0.5;
    c.strategy = strategy;
    c.tol      = tol > 0 ? tol : 0.1;
    c.maxfcn   = maxfcn;
    c.use_grad = use_grad != 0;
    c.fnoise_rel = fnoise_rel > 0 ? fnoise_rel : 0.0;
    return c;
}

void fillResult(const gf::MinResult &r, gf_fit_result *res) {
    if(!res)
        return;
    res->fmin           = r.fmin;
    res->edm            = r.edm;
    res->nfcn           = r.nfcn;
    res->ngrad          = r.ngrad;
    res->valid          = r.valid() ? 1 : 0;
    res->above_max_edm  = r.converged ? 0 : 1;
    res->call_limit     = r.call_limit ? 1 : 0;
    res->has_covariance = r.has_cov ? 1 : 0;
    res->hesse_failed   = r.hesse_failed ? 1 : 0;
    res->made_posdef    = r.made_posdef ? 1 : 0;
    res->n_iter         = r.niter;
    res->reserved       = 0;
}

// Scatters the engine's gradient (one entry per masked parameter) over all parameters.
void scatterGrad(const std::vector<int> &gparam, const double *g, std::vector<double> &full) {
    std::fill(full.begin(), full.end(), 0.0);
    for(size_t s = 0; s < gparam.size(); ++s)
        full[gparam[s]] = g[s];
}

} // namespace

int gf_fit_batch_impl(gf_engine *eng, int toy, int n_toys, const gf_fit_options *o, const double *X0, double *X,
                      double *ERR, gf_fit_result *res);

extern "C" {

int gf_minimizer_create(gf_minimizer **out, int n, const double *x0, const double *err, const double *lo,
                        const double *hi, const int32_t *limited, const int32_t *fixed, double up, int strategy,
                        double tolerance, int maxfcn, int use_grad, double fnoise_rel) {
    if(!out || n < 0 || (n > 0 && !x0))
        return GF_ERR_INVALID;
    auto *m = new(std::nothrow) gf_minimizer();
    if(!m)
        return GF_ERR_OOM;
    m->n = n;
    m->m.reset(new gf::Minimizer(
        makeConfig(n, x0, err, lo, hi, limited, fixed, up, strategy, tolerance, maxfcn, use_grad, fnoise_rel)));
    *out = m;
    return GF_OK;
}

int gf_minimizer_ask(gf_minimizer *m, double *x, int32_t *need_grad) {
    if(!m || !x || !need_grad)
        return -GF_ERR_INVALID;
    int ng  = 0;
    bool r  = m->m->ask(x, &ng);
    *need_grad = ng;
    return r ? 1 : 0;
}

int gf_minimizer_tell(gf_minimizer *m, double f, const double *grad) {
    if(!m)
        return GF_ERR_INVALID;
    m->m->tell(f, grad);
    return GF_OK;
}

int gf_minimizer_result(const gf_minimizer *m, gf_fit_result *res, double *x, double *err, double *cov) {
    if(!m)
        return GF_ERR_INVALID;
    const gf::MinResult &r = m->m->result();
    fillResult(r, res);
    for(int i = 0; i < m->n; ++i) {
        if(x)
            x[i] = r.x[i];
        if(err)
            err[i] = r.err[i];
    }
    if(cov)
        std::memcpy(cov, r.cov.data(), sizeof(double) * r.cov.size());
    return GF_OK;
}

int gf_minimizer_destroy(gf_minimizer *m) {
    delete m;
    return GF_OK;
}

int gf_fit(gf_engine *eng, int toy, const gf_fit_options *o, const double *x0, double *x, double *err,
           gf_fit_result *res) {
    if(!eng || !o || !x0)
        return GF_ERR_INVALID;
    return gf_fit_batch_impl(eng, toy, 1, o, x0, x, err, res);
}

int gf_fit_batch(gf_engine *eng, int n_toys, const gf_fit_options *o, const double *X0, double *X, double *ERR,
                 gf_fit_result *res) {
    return gf_fit_batch_impl(eng, -1, n_toys, o, X0, X, ERR, res);
}

} // extern "C"

// toy >= 0: fit one toy of the engine; toy < 0: fit toys 0..n_toys-1 in lockstep.
int gf_fit_batch_impl(gf_engine *eng, int toy, int n_toys, const gf_fit_options *o, const double *X0, double *X,
                      double *ERR, gf_fit_result *res) {
    if(!eng || !o || !X0 || n_toys < 1)
        return GF_ERR_INVALID;
    const int np = gf_num_params(eng);
    const int ng = gf_num_grad(eng);
    std::vector<int32_t> gq(std::max(1, ng));
    gf_grad_params(eng, gq.data(), ng);
    std::vector<int> gp(gq.begin(), gq.begin() + ng);
    if(o->use_grad) {
        // every free parameter must have an analytic derivative
        std::vector<int> has(np, 0);
        for(int p : gp)
            has[p] = 1;
        for(int i = 0; i < np; ++i)
            if(!(o->fixed && o->fixed[i]) && !has[i])
                return GF_ERR_INVALID;
    }
    std::vector<std::unique_ptr<gf::Minimizer>> ms;
    for(int t = 0; t < n_toys; ++t)
        ms.emplace_back(new gf::Minimizer(makeConfig(np, X0 + (size_t)t * np, o->err, o->lo, o->hi, o->limited,
                                                     o->fixed, o->up, o->strategy, o->tolerance, o->maxfcn,
                                                     o->use_grad, o->fnoise_rel)));
    std::vector<double> xr(np), gfull(np), g(std::max(1, ng));
    int rc = GF_OK;
    if(toy >= 0) {
        int need = 0;
        while(ms[0]->ask(xr.data(), &need)) {
            double f = 0;
            int r    = gf_set_params(eng, toy, xr.data(), np);
            if(r == GF_OK)
                r = need ? gf_nll_grad(eng, toy, &f, g.data()) : gf_nll(eng, toy, &f);
            if(r == GF_ERR_CUDA || r == GF_ERR_OOM || r == GF_ERR_STATE || r == GF_ERR_INVALID) {
                rc = r;
                break;
            }
            if(r != GF_OK)
                f = NAN; // invalid normalisation at this trial point: the line search backs off
            if(need) {
                scatterGrad(gp, g.data(), gfull);
                ms[0]->tell(f, gfull.data());
            } else
                ms[0]->tell(f, nullptr);
        }
    } else {
        const int NT = gf_num_toys(eng);
        if(NT != n_toys)
            return GF_ERR_INVALID;
        std::vector<double> P((size_t)n_toys * np, 0.0), nll(n_toys), G((size_t)n_toys * std::max(1, ng));
        std::vector<int32_t> active(n_toys);
        std::vector<int> need(n_toys);
        for(int t = 0; t < n_toys; ++t)
            std::memcpy(&P[(size_t)t * np], X0 + (size_t)t * np, sizeof(double) * np);
        while(true) {
            bool any = false, anyGrad = false;
            for(int t = 0; t < n_toys; ++t) {
                active[t] = ms[t]->ask(&P[(size_t)t * np], &need[t]) ? 1 : 0;
                any |= active[t] != 0;
                anyGrad |= active[t] && need[t];
            }
            if(!any)
                break;
            int r = gf_nll_batch(eng, n_toys, P.data(), active.data(), nll.data(), anyGrad ? G.data() : nullptr);
            if(r == GF_ERR_CUDA || r == GF_ERR_OOM || r == GF_ERR_STATE || r == GF_ERR_INVALID) {
                rc = r;
                break;
            }
            for(int t = 0; t < n_toys; ++t) {
                if(!active[t])
                    continue;
                if(need[t]) {
                    scatterGrad(gp, &G[(size_t)t * std::max(1, ng)], gfull);
                    ms[t]->tell(nll[t], gfull.data());
                } else
                    ms[t]->tell(nll[t], nullptr);
            }
        }
    }
    for(int t = 0; t < n_toys; ++t) {
        const gf::MinResult &r = ms[t]->result();
        if(X)
            std::memcpy(X + (size_t)t * np, r.x.data(), sizeof(double) * np);
        if(ERR)
            std::memcpy(ERR + (size_t)t * np, r.err.data(), sizeof(double) * np);
        if(o->cov && r.cov.size() == (size_t)np * np)
            std::memcpy(o->cov + (size_t)t * np * np, r.cov.data(), sizeof(double) * np * np);
        fillResult(r, res ? res + t : nullptr);
    }
    return rc;
}
