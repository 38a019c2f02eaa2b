// MIGRAD-style variable-metric minimiser (see migrad.h for the conventions).
#include "migrad.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>

namespace gf {

namespace {
constexpr double kHuge = 1e300;
inline double finiteOr(double f) { return std::isfinite(f) ? f : kHuge; }
} // namespace

Minimizer::Minimizer(const MinConfig &cfg)
    : cfg_(cfg)
    , root_(Task{std::coroutine_handle<Task::promise_type>{}}) {
    // machine precision as MINUIT estimates it: eps ~ 4 DBL_EPSILON, eps2 = 2 sqrt(eps)
    eps_  = 4.0 * DBL_EPSILON;
    eps2_ = 2.0 * std::sqrt(eps_);
    for(int i = 0; i < cfg_.n; ++i)
        if(!cfg_.fixed[i])
            free_.push_back(i);
    nf_ = (int)free_.size();
    req_x_.assign(cfg_.n, 0.0);
    rep_g_.assign(cfg_.n, 0.0);
    res_.x   = cfg_.x0;
    res_.err.assign(cfg_.n, 0.0);
    res_.cov.assign((size_t)cfg_.n * cfg_.n, 0.0);
    root_ = run();
}

Minimizer::~Minimizer() = default;

bool Minimizer::done() const { return started_ && (!root_.h || root_.h.done()); }

bool Minimizer::ask(double *x, int *need_grad) {
    if(!started_) {
        started_ = true;
        root_.h.resume();
    }
    if(root_.h.done() || !pending_)
        return false;
    for(int i = 0; i < cfg_.n; ++i)
        x[i] = req_x_[i];
    *need_grad = req_grad_ ? 1 : 0;
    return true;
}

void Minimizer::tell(double f, const double *grad) {
    rep_f_ = f;
    if(grad)
        for(int i = 0; i < cfg_.n; ++i)
            rep_g_[i] = grad[i];
    auto h   = pending_;
    pending_ = {};
    if(h)
        h.resume();
}

// ---- parameter transforms (MINUIT internal coordinates) ----
double Minimizer::int2ext(int k, double v) const {
    int i = free_[k];
    switch(cfg_.limited[i]) {
    case 1: return cfg_.lo[i] + 0.5 * (cfg_.hi[i] - cfg_.lo[i]) * (std::sin(v) + 1.0);
    case 2: return cfg_.lo[i] - 1.0 + std::sqrt(v * v + 1.0);
    case 3: return cfg_.hi[i] + 1.0 - std::sqrt(v * v + 1.0);
    default: return v;
    }
}

double Minimizer::ext2int(int k, double v) const {
    int i = free_[k];
    switch(cfg_.limited[i]) {
    case 1: {
        const double piby2  = 2.0 * std::atan(1.0);
        const double distnn = 8.0 * std::sqrt(eps2_);
        double yy           = 2.0 * (v - cfg_.lo[i]) / (cfg_.hi[i] - cfg_.lo[i]) - 1.0;
        if(yy * yy > 1.0 - eps2_)
            return yy < 0 ? -piby2 + distnn : piby2 - distnn;
        return std::asin(yy);
    }
    case 2: {
        double yy = v - cfg_.lo[i] + 1.0;
        return yy * yy > 1.0 ? std::sqrt(yy * yy - 1.0) : 0.0;
    }
    case 3: {
        double yy = cfg_.hi[i] - v + 1.0;
        return yy * yy > 1.0 ? std::sqrt(yy * yy - 1.0) : 0.0;
    }
    default: return v;
    }
}

double Minimizer::dext(int k, double v) const {
    int i = free_[k];
    switch(cfg_.limited[i]) {
    case 1: return 0.5 * (cfg_.hi[i] - cfg_.lo[i]) * std::cos(v);
    case 2: return v / std::sqrt(v * v + 1.0);
    case 3: return -v / std::sqrt(v * v + 1.0);
    default: return 1.0;
    }
}

// MINUIT's conversion of an internal error to an external one.
double Minimizer::int2extError(int k, double v, double e) const {
    int i     = free_[k];
    double dx = e;
    if(cfg_.limited[i]) {
        double ui  = int2ext(k, v);
        double du1 = int2ext(k, v + dx) - ui;
        double du2 = int2ext(k, v - dx) - ui;
        if(cfg_.limited[i] == 1 && dx > 1.0)
            du1 = cfg_.hi[i] - cfg_.lo[i];
        dx = 0.5 * (std::fabs(du1) + std::fabs(du2));
    }
    return dx;
}

// Cholesky-based inversion of a symmetric matrix; if it is not positive
// definite the diagonal is shifted until it is (MINUIT's MnPosDef idea).
bool Minimizer::invertPosDef(std::vector<double> &A, int n, bool *made_posdef) {
    std::vector<double> a = A;
    for(int i = 0; i < n; ++i)
        for(int j = 0; j < i; ++j) {
            double s           = 0.5 * (a[i * n + j] + a[j * n + i]);
            a[i * n + j]       = s;
            a[j * n + i]       = s;
        }
    double dmin = std::numeric_limits<double>::max(), dmax = 0;
    for(int i = 0; i < n; ++i) {
        dmin = std::min(dmin, a[i * n + i]);
        dmax = std::max(dmax, std::fabs(a[i * n + i]));
    }
    auto chol = [&](std::vector<double> M, std::vector<double> &L) -> bool {
        L.assign((size_t)n * n, 0.0);
        for(int j = 0; j < n; ++j) {
            double s = M[j * n + j];
            for(int k = 0; k < j; ++k)
                s -= L[j * n + k] * L[j * n + k];
            if(!(s > 0))
                return false;
            L[j * n + j] = std::sqrt(s);
            for(int i = j + 1; i < n; ++i) {
                double t = M[i * n + j];
                for(int k = 0; k < j; ++k)
                    t -= L[i * n + k] * L[j * n + k];
                L[i * n + j] = t / L[j * n + j];
            }
        }
        return true;
    };
    std::vector<double> L;
    bool ok = chol(a, L);
    if(made_posdef)
        *made_posdef = false;
    if(!ok) {
        if(made_posdef)
            *made_posdef = true;
        double shift = std::max(1e-3 * dmax, 1e-12) + (dmin < 0 ? -dmin : 0);
        for(int tries = 0; tries < 60 && !ok; ++tries) {
            std::vector<double> b = a;
            for(int i = 0; i < n; ++i)
                b[i * n + i] += shift;
            ok = chol(b, L);
            shift *= 2;
        }
        if(!ok)
            return false;
    }
    // inverse from L: A^-1 = L^-T L^-1
    std::vector<double> Linv((size_t)n * n, 0.0);
    for(int i = 0; i < n; ++i) {
        Linv[i * n + i] = 1.0 / L[i * n + i];
        for(int j = 0; j < i; ++j) {
            double s = 0;
            for(int k = j; k < i; ++k)
                s -= L[i * n + k] * Linv[k * n + j];
            Linv[i * n + j] = s / L[i * n + i];
        }
    }
    for(int i = 0; i < n; ++i)
        for(int j = 0; j <= i; ++j) {
            double s = 0;
            for(int k = i; k < n; ++k)
                s += Linv[k * n + i] * Linv[k * n + j];
            A[i * n + j] = s;
            A[j * n + i] = s;
        }
    return true;
}

// One function (and optionally gradient) evaluation at internal point xi.
Minimizer::Task Minimizer::evalAt(const std::vector<double> &xi, bool grad) {
    req_x_ = cfg_.x0;
    for(int k = 0; k < nf_; ++k)
        req_x_[free_[k]] = int2ext(k, xi[k]);
    req_grad_ = grad;
    co_await Req{this};
    ++res_.nfcn;
    f_ = finiteOr(rep_f_);
    if(grad) {
        ++res_.ngrad;
        gi_.assign(nf_, 0.0);
        for(int k = 0; k < nf_; ++k)
            gi_[k] = rep_g_[free_[k]] * dext(k, xi[k]);
    }
}

// Two-point numerical derivatives with MINUIT's step control (strategy cycles).
Minimizer::Task Minimizer::numGrad(std::vector<double> &xi, double f0) {
    int ncycle      = cfg_.strategy <= 0 ? 2 : (cfg_.strategy == 1 ? 3 : 5);
    double stepTol  = cfg_.strategy <= 0 ? 0.5 : (cfg_.strategy == 1 ? 0.3 : 0.1);
    double gradTol  = cfg_.strategy <= 0 ? 0.1 : (cfg_.strategy == 1 ? 0.05 : 0.02);
    double dfmin    = 8.0 * eps2_ * (std::fabs(f0) + cfg_.up);
    double vrysml   = 8.0 * eps_ * eps_;
    for(int k = 0; k < nf_; ++k) {
        double xtf    = xi[k];
        double epspri = eps2_ + std::fabs(g_[k] * eps2_);
        double stepb4 = 0;
        for(int j = 0; j < ncycle; ++j) {
            double optstp = std::sqrt(dfmin / (std::fabs(g2_[k]) + epspri));
            double step   = std::max(optstp, std::fabs(0.1 * gstep_[k]));
            if(cfg_.limited[free_[k]])
                step = std::min(step, 0.5);
            double stpmax = 10.0 * std::fabs(gstep_[k]);
            step          = std::min(step, stpmax);
            double stpmin = std::max(vrysml, 8.0 * std::fabs(eps2_ * xi[k]));
            step          = std::max(step, stpmin);
            if(std::fabs((step - stepb4) / step) < stepTol)
                break;
            gstep_[k] = step;
            stepb4    = step;
            xi[k]     = xtf + step;
            co_await evalAt(xi, false);
            double fs1 = f_;
            xi[k]      = xtf - step;
            co_await evalAt(xi, false);
            double fs2 = f_;
            xi[k]      = xtf;
            double grdb4 = g_[k];
            g_[k]        = 0.5 * (fs1 - fs2) / step;
            g2_[k]       = (fs1 + fs2 - 2.0 * f0) / step / step;
            if(std::fabs(grdb4 - g_[k]) / (std::fabs(g_[k]) + dfmin / step) < gradTol)
                break;
        }
    }
}

// Second derivatives at the minimum: central differences of the analytic
// gradient, or MINUIT-style function-value differences.  Sets V_ on success.
Minimizer::Task Minimizer::hesse(std::vector<double> &xi, double f0) {
    int n = nf_;
    std::vector<double> H((size_t)n * n, 0.0);
    std::vector<double> d(n);
    for(int k = 0; k < n; ++k) {
        double s = V_[k * n + k] > 0 ? std::sqrt(V_[k * n + k]) : std::sqrt(2.0 * cfg_.up / std::max(std::fabs(g2_[k]), 1e-300));
        if(!std::isfinite(s) || s <= 0)
            s = 1e-3 * (std::fabs(xi[k]) + 1.0);
        d[k] = s;
    }
    if(cfg_.use_grad) {
        for(int k = 0; k < n; ++k) {
            double h = 0.05 * d[k], xk = xi[k];
            xi[k]    = xk + h;
            co_await evalAt(xi, true);
            std::vector<double> gp = gi_;
            xi[k] = xk - h;
            co_await evalAt(xi, true);
            std::vector<double> gm = gi_;
            xi[k] = xk;
            for(int j = 0; j < n; ++j)
                H[j * n + k] = (gp[j] - gm[j]) / (2.0 * h);
        }
    } else {
        std::vector<double> fp(n), fm(n);
        for(int k = 0; k < n; ++k) {
            double h = 0.3 * d[k], xk = xi[k];
            d[k]     = h;
            xi[k]    = xk + h;
            co_await evalAt(xi, false);
            fp[k] = f_;
            xi[k] = xk - h;
            co_await evalAt(xi, false);
            fm[k] = f_;
            xi[k] = xk;
            H[k * n + k] = (fp[k] + fm[k] - 2.0 * f0) / (h * h);
            g2_[k]       = H[k * n + k];
        }
        for(int k = 0; k < n; ++k)
            for(int j = k + 1; j < n; ++j) {
                double xk = xi[k], xj = xi[j];
                xi[k] += d[k];
                xi[j] += d[j];
                co_await evalAt(xi, false);
                xi[k] = xk;
                xi[j] = xj;
                double hkj   = (f_ + f0 - fp[k] - fp[j]) / (d[k] * d[j]);
                H[k * n + j] = hkj;
                H[j * n + k] = hkj;
            }
    }
    bool posdef = false;
    std::vector<double> V = H;
    if(invertPosDef(V, n, &posdef)) {
        V_                = V;
        res_.has_cov      = true;
        res_.made_posdef  = res_.made_posdef || posdef;
        res_.hesse_failed = false;
    } else {
        res_.hesse_failed = true;
    }
}

// Line search along `step` from f0 with directional derivative slope < 0.
// With function values only: parabolic interpolation / backtracking.  With an
// analytic gradient the directional derivative brackets the minimum (secant on
// g . step), which stays reliable when the value carries rounding noise of
// order fnoise_rel * |f| (sums of many FP32 terms); value changes below that
// noise are treated as ties.
Minimizer::Task Minimizer::lineSearch(const std::vector<double> &xi, double f0, const std::vector<double> &step,
                                      double slope) {
    const bool g      = cfg_.use_grad;
    const double ftol = cfg_.fnoise_rel * std::fabs(f0);
    auto at = [&](double lam) {
        std::vector<double> x = xi;
        for(int k = 0; k < nf_; ++k)
            x[k] += lam * step[k];
        return x;
    };
    auto dslope = [&]() {
        double s = 0;
        for(int k = 0; k < nf_; ++k)
            s += gi_[k] * step[k];
        return s;
    };
    ls_lambda_ = 0;
    ls_f_      = f0;
    co_await evalAt(at(1.0), g);
    double f1 = f_;
    std::vector<double> g1 = gi_;
    // approximate Wolfe conditions (Hager & Zhang): with an analytic gradient a step is acceptable when the
    // directional derivative has dropped to sigma*slope or below while not turning up by more than
    // (1 - 2 delta)|slope|, and the value has not risen beyond its rounding noise
    const bool wolfe = g && std::isfinite(f1) && f1 <= f0 + ftol && dslope() >= 0.9 * slope && dslope() <= -0.8 * slope;
    if(g && std::isfinite(f1) && (f1 <= f0 + ftol || wolfe)) {
        double s1  = dslope();
        ls_lambda_ = 1.0;
        ls_f_      = f1;
        ls_g_      = g1;
        // root of the linearly interpolated directional derivative
        double lsec = (s1 != slope) ? slope / (slope - s1) : 1.0;
        double ltry = 0;
        if(s1 >= 0 && lsec > 0.05 && lsec < 0.95)
            ltry = lsec;
        else if(s1 < 0 && s1 > slope)
            ltry = std::min(lsec, 4.0);
        if(ltry > 0 && std::fabs(ltry - 1.0) > 0.05) {
            co_await evalAt(at(ltry), g);
            double st = dslope();
            if(std::isfinite(f_) && f_ <= f1 + ftol && std::fabs(st) < std::fabs(s1)) {
                ls_lambda_ = ltry;
                ls_f_      = f_;
                ls_g_      = gi_;
            }
        }
        co_return;
    }
    if(!g && f1 < f0) {
        ls_lambda_  = 1.0;
        ls_f_       = f1;
        ls_g_       = g1;
        double den  = 2.0 * (f1 - f0 - slope);
        double lp   = den > 0 ? -slope / den : 4.0;
        double ltry = 0;
        if(lp > 1.5)
            ltry = std::min(lp, 4.0);
        else if(lp < 0.7 && lp > 0.05)
            ltry = lp;
        if(ltry > 0) {
            co_await evalAt(at(ltry), g);
            if(f_ < ls_f_) {
                ls_lambda_ = ltry;
                ls_f_      = f_;
                ls_g_      = gi_;
            }
        }
        co_return;
    }
    // backtracking: the trial point overshot (or was invalid)
    double lam = 1.0, fl = f1;
    double sl  = (g && std::isfinite(f1)) ? dslope() : 0.0;
    for(int it = 0; it < 12; ++it) {
        double ln;
        if(g && std::isfinite(fl) && sl > 0)
            ln = lam * slope / (slope - sl); // secant on the directional derivative
        else {
            double den = 2.0 * (fl - f0 - slope * lam);
            ln         = den > 0 && std::isfinite(fl) ? -slope * lam * lam / den : 0.5 * lam;
        }
        ln = std::min(std::max(ln, 0.1 * lam), 0.5 * lam);
        co_await evalAt(at(ln), g);
        if(std::isfinite(f_) && (f_ < f0 || (g && f_ <= f0 + ftol))) {
            ls_lambda_ = ln;
            ls_f_      = f_;
            ls_g_      = gi_;
            co_return;
        }
        lam = ln;
        fl  = f_;
        if(g)
            sl = dslope();
    }
}

Minimizer::Task Minimizer::run() {
    const int n = nf_;
    int maxfcn  = cfg_.maxfcn > 0 ? cfg_.maxfcn : 200 + 100 * n + 5 * n * n;
    double edmval = 0.002 * cfg_.tol * cfg_.up;
    std::vector<double> xi(n), dirin(n);
    for(int k = 0; k < n; ++k) {
        int i  = free_[k];
        xi[k]  = ext2int(k, cfg_.x0[i]);
        double e = std::fabs(cfg_.err[i]) > 0 ? std::fabs(cfg_.err[i]) : 0.1 * (std::fabs(cfg_.x0[i]) + 1.0);
        double up = cfg_.x0[i] + e, dn = cfg_.x0[i] - e;
        if(cfg_.limited[i] == 1 || cfg_.limited[i] == 3)
            up = std::min(up, cfg_.hi[i]);
        if(cfg_.limited[i] == 1 || cfg_.limited[i] == 2)
            dn = std::max(dn, cfg_.lo[i]);
        double d = 0.5 * (std::fabs(ext2int(k, up) - xi[k]) + std::fabs(ext2int(k, dn) - xi[k]));
        dirin[k] = d > 0 ? d : e;
    }
    g_.assign(n, 0.0);
    g2_.assign(n, 0.0);
    gstep_.assign(n, 0.0);
    V_.assign((size_t)n * n, 0.0);

    co_await evalAt(xi, cfg_.use_grad && n > 0);
    double f0 = f_;
    if(n == 0) {
        res_.fmin      = f0;
        res_.converged = true;
        res_.has_cov   = true;
        co_return;
    }
    auto resetV = [&]() {
        std::fill(V_.begin(), V_.end(), 0.0);
        for(int k = 0; k < n; ++k)
            V_[k * n + k] = g2_[k] > 0 ? 1.0 / g2_[k] : dirin[k] * dirin[k];
    };
    // ---- seed ----
    if(cfg_.use_grad) {
        g_ = gi_;
        std::vector<double> H((size_t)n * n, 0.0);
        for(int k = 0; k < n; ++k) {
            double h  = std::max(1e-3 * dirin[k], 1e-7 * (std::fabs(xi[k]) + 1.0));
            double xk = xi[k];
            xi[k]     = xk + h;
            co_await evalAt(xi, true);
            xi[k] = xk;
            for(int j = 0; j < n; ++j)
                H[j * n + k] = (gi_[j] - g_[j]) / h;
            g2_[k] = H[k * n + k];
        }
        std::vector<double> V = H;
        bool pd = false;
        if(invertPosDef(V, n, &pd) && !pd)
            V_ = V;
        else
            resetV();
    } else {
        for(int k = 0; k < n; ++k) {
            g2_[k]    = 2.0 * cfg_.up / (dirin[k] * dirin[k]);
            gstep_[k] = 0.1 * dirin[k];
        }
        co_await numGrad(xi, f0);
        resetV();
    }
    auto edmOf = [&](const std::vector<double> &g) {
        double e = 0;
        for(int i = 0; i < n; ++i)
            for(int j = 0; j < n; ++j)
                e += g[i] * V_[i * n + j] * g[j];
        return 0.5 * e;
    };
    double edm    = edmOf(g_);
    int hesseRuns = 0;
    bool justReset = false;
    while(true) {
        if(res_.nfcn >= maxfcn) {
            res_.call_limit = true;
            break;
        }
        if(edm < edmval) {
            if(hesseRuns >= 3) {
                res_.converged = true;
                break;
            }
            ++hesseRuns;
            co_await hesse(xi, f0);
            edm = edmOf(g_);
            if(edm < edmval || res_.hesse_failed) {
                res_.converged = edm < edmval;
                break;
            }
            continue;
        }
        std::vector<double> step(n, 0.0);
        for(int i = 0; i < n; ++i)
            for(int j = 0; j < n; ++j)
                step[i] -= V_[i * n + j] * g_[j];
        double slope = 0;
        for(int i = 0; i < n; ++i)
            slope += g_[i] * step[i];
        if(!(slope < 0)) {
            resetV();
            std::fill(step.begin(), step.end(), 0.0);
            for(int i = 0; i < n; ++i)
                for(int j = 0; j < n; ++j)
                    step[i] -= V_[i * n + j] * g_[j];
            slope = 0;
            for(int i = 0; i < n; ++i)
                slope += g_[i] * step[i];
            if(!(slope < 0))
                break;
        }
        co_await lineSearch(xi, f0, step, slope);
        if(ls_lambda_ == 0) {
            if(justReset)
                break;
            resetV();
            justReset = true;
            continue;
        }
        justReset = false;
        std::vector<double> xn(n), gn, gold = g_;
        for(int k = 0; k < n; ++k)
            xn[k] = xi[k] + ls_lambda_ * step[k];
        double fn = ls_f_;
        if(cfg_.use_grad)
            gn = ls_g_;
        else {
            co_await numGrad(xn, fn); // refines g_, g2_, gstep_ in place
            gn = g_;
        }
        // Davidon / BFGS rank-two update of the inverse Hessian
        std::vector<double> dx(n), dg(n), vg(n, 0.0);
        double delgam = 0, gvg = 0;
        for(int k = 0; k < n; ++k) {
            dx[k] = xn[k] - xi[k];
            dg[k] = gn[k] - gold[k];
            delgam += dx[k] * dg[k];
        }
        for(int i = 0; i < n; ++i)
            for(int j = 0; j < n; ++j)
                vg[i] += V_[i * n + j] * dg[j];
        for(int i = 0; i < n; ++i)
            gvg += dg[i] * vg[i];
        if(delgam > 0 && gvg > 0) {
            for(int i = 0; i < n; ++i)
                for(int j = 0; j < n; ++j)
                    V_[i * n + j] += dx[i] * dx[j] / delgam - vg[i] * vg[j] / gvg;
            if(delgam > gvg) {
                std::vector<double> fl(n);
                for(int i = 0; i < n; ++i)
                    fl[i] = dx[i] / delgam - vg[i] / gvg;
                for(int i = 0; i < n; ++i)
                    for(int j = 0; j < n; ++j)
                        V_[i * n + j] += gvg * fl[i] * fl[j];
            }
        }
        xi = xn;
        f0 = fn;
        g_ = gn;
        edm = edmOf(g_);
        ++res_.niter;
    }
    // ---- result in external coordinates ----
    res_.fmin = f0;
    res_.edm  = edm;
    res_.x    = cfg_.x0;
    for(int k = 0; k < n; ++k) {
        int i      = free_[k];
        res_.x[i]  = int2ext(k, xi[k]);
        double e   = V_[k * n + k] > 0 ? std::sqrt(V_[k * n + k]) : 0.0;
        res_.err[i] = int2extError(k, xi[k], e);
    }
    for(int a = 0; a < n; ++a)
        for(int b = 0; b < n; ++b)
            res_.cov[(size_t)free_[a] * cfg_.n + free_[b]] = dext(a, xi[a]) * V_[a * n + b] * dext(b, xi[b]);
}

} // namespace gf
