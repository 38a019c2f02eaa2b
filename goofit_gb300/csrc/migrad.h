// Variable-metric minimiser with the MIGRAD conventions of MINUIT (F. James,
// "MINUIT Function Minimization and Error Analysis", CERN D506): internal
// sine / square-root parameter transforms for limits, EDM = g^T V g / 2 with
// convergence at EDM < 0.002 * tolerance * up, Davidon-Fletcher-Powell /
// BFGS rank-two updates of the inverse Hessian, numerical 2-point gradients
// with strategy-dependent cycles, and a final Hesse step for the errors.
//
// It replaces the Minuit2 MnMigrad call of the reference
// (src/goofit/FitManagerMinuit2.cpp:45-53), which is not vendored with the
// reference sources.  Written as a coroutine so that a caller can drive it in
// ask/tell style: one minimiser per fit, many fits advanced in lockstep.
#pragma once

#include <coroutine>
#include <exception>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace gf {

struct MinConfig {
    int n = 0;
    std::vector<double> x0, err, lo, hi;
    std::vector<int> limited; // 0 none, 1 both, 2 lower, 3 upper
    std::vector<int> fixed;
    double up       = 0.5;
    int strategy    = 1;
    double tol      = 0.1;
    int maxfcn      = 0; // 0: 200 + 100 n + 5 n^2 (MINUIT default)
    bool use_grad   = false;
    double fnoise_rel = 0; // relative rounding noise of f: value changes below it are ties
};

struct MinResult {
    std::vector<double> x, err;
    std::vector<double> cov; // external, n x n (fixed rows/cols zero)
    double fmin = 0, edm = 0;
    int nfcn = 0, ngrad = 0, niter = 0;
    bool converged = false, has_cov = false, call_limit = false, hesse_failed = false, made_posdef = false;
    bool valid() const { return converged && has_cov && !call_limit; }
};

class Minimizer {
  public:
    explicit Minimizer(const MinConfig &cfg);
    ~Minimizer();
    Minimizer(const Minimizer &)            = delete;
    Minimizer &operator=(const Minimizer &) = delete;

    // true while a function value is requested; fills x (external, n) and need_grad
    bool ask(double *x, int *need_grad);
    // f and (if requested) the external gradient over all n parameters
    void tell(double f, const double *grad);
    bool done() const;
    const MinResult &result() const { return res_; }

    struct Task {
        struct promise_type {
            std::coroutine_handle<> cont;
            Task get_return_object() { return Task{std::coroutine_handle<promise_type>::from_promise(*this)}; }
            std::suspend_always initial_suspend() noexcept { return {}; }
            struct Final {
                bool await_ready() noexcept { return false; }
                std::coroutine_handle<> await_suspend(std::coroutine_handle<promise_type> h) noexcept {
                    auto c = h.promise().cont;
                    return c ? c : std::noop_coroutine();
                }
                void await_resume() noexcept {}
            };
            Final final_suspend() noexcept { return {}; }
            void return_void() {}
            void unhandled_exception() { std::terminate(); }
        };
        std::coroutine_handle<promise_type> h;
        explicit Task(std::coroutine_handle<promise_type> hh) : h(hh) {}
        Task(Task &&o) noexcept : h(std::exchange(o.h, {})) {}
        Task &operator=(Task &&o) noexcept {
            if(h)
                h.destroy();
            h = std::exchange(o.h, {});
            return *this;
        }
        ~Task() {
            if(h)
                h.destroy();
        }
        bool await_ready() { return false; }
        std::coroutine_handle<> await_suspend(std::coroutine_handle<> c) {
            h.promise().cont = c;
            return h;
        }
        void await_resume() {}
    };

  private:
    struct Req {
        Minimizer *m;
        bool await_ready() { return false; }
        void await_suspend(std::coroutine_handle<> h) { m->pending_ = h; }
        void await_resume() {}
    };

    Task run();
    Task evalAt(const std::vector<double> &xi, bool grad);   // -> f_, gi_ (internal)
    Task numGrad(std::vector<double> &xi, double f0);          // -> g_, g2_, gstep_
    Task hesse(std::vector<double> &xi, double f0);            // -> V_
    Task lineSearch(const std::vector<double> &xi, double f0, const std::vector<double> &step, double slope);

    double int2ext(int k, double v) const;
    double ext2int(int k, double v) const;
    double dext(int k, double v) const;
    double int2extError(int k, double v, double e) const;
    bool invertPosDef(std::vector<double> &A, int n, bool *made_posdef);

    MinConfig cfg_;
    std::vector<int> free_; // free parameter indices
    int nf_ = 0;
    // request / reply
    std::vector<double> req_x_;
    bool req_grad_ = false;
    double rep_f_  = 0;
    std::vector<double> rep_g_;
    std::coroutine_handle<> pending_;
    bool started_ = false;
    Task root_;
    // working state (internal coordinates)
    double f_ = 0;
    std::vector<double> gi_;              // gradient of last evalAt (if grad)
    std::vector<double> g_, g2_, gstep_;  // current gradient estimates
    std::vector<double> V_;               // inverse Hessian (nf x nf)
    double ls_lambda_ = 0, ls_f_ = 0;     // line search result
    std::vector<double> ls_g_;            // gradient at the line-search point (analytic mode)
    MinResult res_;
    double eps_, eps2_;
};

} // namespace gf
