// C entry points over the reference's own likelihood code, compiled for the CPU (Thrust OMP backend) from
// the reference's sources by oracle/ref/Makefile.  TEST INFRASTRUCTURE ONLY: it pins the FP64 restatement in
// oracle/oracle.cpp to the reference's arithmetic (tests/test_reference_build.py); the engine never uses it.
//
// Each entry point builds the benchmark configuration's PDF tree with the reference's classes and
// constructors, fills an UnbinnedDataSet, and evaluates GooPdf::calculateNLL (src/PDFs/GooPdf.cu:254-273)
// at every requested parameter point the way FCN::operator() does (src/goofit/FCN.cpp:18-28): the
// variables' values are set and marked changed, the parameters pushed with updateParameters(), the NLL
// computed.  Errors thrown by the reference come back as a non-zero status and a message.
#include <goofit/PDFs/GooPdf.h>
#include <goofit/PDFs/basic/ExpPdf.h>
#include <goofit/PDFs/basic/GaussianPdf.h>
#include <goofit/PDFs/basic/PolynomialPdf.h>
#include <goofit/PDFs/combine/AddPdf.h>
#include <goofit/PDFs/combine/ConvolutionPdf.h>
#include <goofit/PDFs/combine/ProdPdf.h>
#include <goofit/PDFs/physics/Amp3Body.h>
#include <goofit/PDFs/physics/Amp4Body.h>
#include <goofit/PDFs/physics/Amplitude.h>
#include <goofit/PDFs/physics/SpinFactors.h>
#include <goofit/PDFs/physics/detail/Dim5.h>
#include <goofit/PDFs/physics/lineshapes/RBW.h>
#include <goofit/PDFs/physics/lineshapes/SBW.h>
#include <goofit/PDFs/physics/resonances/RBW.h>
#include <goofit/UnbinnedDataSet.h>
#include <mcbooster/EvaluateArray.h>
#include <mcbooster/Generate.h>
#include <goofit/Variable.h>

#include <array>
#include <exception>
#include <string>
#include <vector>

namespace {

std::string g_err;

template <typename F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch(std::exception &e) {
        g_err = e.what();
        return 1;
    } catch(...) {
        g_err = "unknown exception";
        return 1;
    }
}

// One FCN evaluation of the reference: set the values, flag them changed, push them, compute the NLL.
double evaluate(GooFit::GooPdf &pdf, std::vector<GooFit::Variable> &vars, const double *p) {
    for(size_t i = 0; i < vars.size(); ++i) {
        vars[i].setValue(p[i]);
        vars[i].setChanged(true);
        pdf.updateVariable(vars[i], p[i]);
    }
    pdf.updateParameters();
    return pdf.calculateNLL();
}

void fill(GooFit::UnbinnedDataSet &data, GooFit::Observable &x, const double *xs, long n) {
    for(long i = 0; i < n; ++i) {
        x.setValue(xs[i]);
        data.addEvent();
    }
}

} // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

// C1: ExpPdf(x; alpha) on [lo, hi] (analytic normalisation).  P[k] = alpha of point k.
int ref_exp_nll(const double *xs, long n, double lo, double hi, const double *P, int npts, double *out) {
    return guarded([&] {
        GooFit::Observable x("x", lo, hi);
        GooFit::Variable alpha("alpha", P[0], 0.1, -10.0, 10.0);
        GooFit::ExpPdf pdf("exppdf", x, alpha);
        GooFit::UnbinnedDataSet data(x);
        fill(data, x, xs, n);
        pdf.setData(&data);
        std::vector<GooFit::Variable> vars{alpha};
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(pdf, vars, P + k);
    });
}

// C2: AddPdf(fsig; ConvolutionPdf(ExpPdf(alpha), GaussianPdf(mu, sigma)), PolynomialPdf(c0)) on
// [xlo, xhi] with `bins` normalisation bins and integration constants conv = (lo, hi, step).
// P[5 k ..] = (fsig, alpha, mu, sigma, c0) of point k.
int ref_c2_nll(const double *xs, long n, double xlo, double xhi, int bins, const double *conv, const double *P,
               int npts, double *out) {
    return guarded([&] {
        GooFit::Observable x("x", xlo, xhi);
        x.setNumBins(bins);
        GooFit::Variable fsig("fsig", P[0], 0.02, 0.0, 1.0);
        GooFit::Variable alpha("alpha", P[1], 0.05, -2.0, -0.1);
        GooFit::Variable mu("mu", P[2], 0.02, -1.0, 1.0);
        GooFit::Variable sigma("sigma", P[3], 0.02, 0.05, 1.0);
        GooFit::Variable c0("c0", P[4]);
        GooFit::ExpPdf model("model", x, alpha);
        GooFit::GaussianPdf resol("resolution", x, mu, sigma);
        GooFit::ConvolutionPdf sig("signal", x, &model, &resol);
        sig.setIntegrationConstants(conv[0], conv[1], conv[2]);
        GooFit::PolynomialPdf bkg("background", x, {c0}, 0);
        GooFit::AddPdf pdf("total", fsig, &sig, &bkg);
        GooFit::UnbinnedDataSet data(x);
        fill(data, x, xs, n);
        pdf.setData(&data);
        std::vector<GooFit::Variable> vars{fsig, alpha, mu, sigma, c0};
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(pdf, vars, P + 5 * k);
    });
}

// ProdPdf(GaussianPdf(x; mx, sx), ExpPdf(y; ay)) on x in [-5, 5], y in [0, 10]: separate observables, each
// factor normalised analytically.  P[3 k ..] = (mx, sx, ay).
int ref_prod_nll(const double *xs, const double *ys, long n, const double *P, int npts, double *out) {
    return guarded([&] {
        GooFit::Observable x("x", -5.0, 5.0), y("y", 0.0, 10.0);
        GooFit::Variable mx("mx", P[0], 0.01, -1, 1), sx("sx", P[1], 0.01, 0.1, 3), ay("ay", P[2], 0.01, -2, -0.01);
        GooFit::GaussianPdf g("gx", x, mx, sx);
        GooFit::ExpPdf e("ey", y, ay);
        GooFit::ProdPdf pdf("prod", {&g, &e});
        GooFit::UnbinnedDataSet data({x, y});
        for(long i = 0; i < n; ++i) {
            x.setValue(xs[i]);
            y.setValue(ys[i]);
            data.addEvent();
        }
        pdf.setData(&data);
        std::vector<GooFit::Variable> vars{mx, sx, ay};
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(pdf, vars, P + 3 * k);
    });
}

// ProdPdf(GaussianPdf(x; mx, sx), ExpPdf(x; ax)) on x in [-5, 5] with `bins` bins: the factors share x, so
// the product is normalised numerically.  P[3 k ..] = (mx, sx, ax).
int ref_prod_overlap_nll(const double *xs, long n, int bins, const double *P, int npts, double *out) {
    return guarded([&] {
        GooFit::Observable x("x", -5.0, 5.0);
        x.setNumBins(bins);
        GooFit::Variable mx("mx", P[0], 0.01, -1, 1), sx("sx", P[1], 0.01, 0.1, 3), ax("ax", P[2], 0.01, -2, 2);
        GooFit::GaussianPdf g("gx", x, mx, sx);
        GooFit::ExpPdf e("ex", x, ax);
        GooFit::ProdPdf pdf("prod", {&g, &e});
        GooFit::UnbinnedDataSet data(x);
        fill(data, x, xs, n);
        pdf.setData(&data);
        std::vector<GooFit::Variable> vars{mx, sx, ax};
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(pdf, vars, P + 3 * k);
    });
}

// Extended AddPdf({n_e, n_g}; ExpPdf(x; a), GaussianPdf(x; m, s)) on x in [0, 10].
// P[5 k ..] = (a, m, s, n_e, n_g).
int ref_extadd_nll(const double *xs, long n, const double *P, int npts, double *out) {
    return guarded([&] {
        GooFit::Observable x("x", 0.0, 10.0);
        GooFit::Variable a("a", P[0], 0.01, -3, -0.01), m("m", P[1], 0.01, 1, 8), sg("s", P[2], 0.01, 0.1, 3);
        GooFit::Variable ne("n_e", P[3], 10, 0, 1e6), ng("n_g", P[4], 10, 0, 1e6);
        GooFit::ExpPdf e("e", x, a);
        GooFit::GaussianPdf g("g", x, m, sg);
        GooFit::AddPdf pdf("ext", {ne, ng}, {&e, &g});
        GooFit::UnbinnedDataSet data(x);
        fill(data, x, xs, n);
        pdf.setData(&data);
        std::vector<GooFit::Variable> vars{a, m, sg, ne, ng};
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(pdf, vars, P + 5 * k);
    });
}

// C3: Amp3Body(m12, m13, eventNumber) of nres relativistic Breit-Wigner resonances (spin[r], daughter pair
// cyc[r]) with a constant multivariate PolynomialPdf efficiency; dec = (M, m1, m2, m3, meson radius,
// mother radius); `bins` normalisation bins per axis on [0, 3]^2.  P[4 nres k ..] = (Re c, Im c, mass, width)
// per resonance of point k.
int ref_amp3_nll(const double *m12s, const double *m13s, long n, int bins, const double *dec, int nres,
                 const int *spin, const int *cyc, const double *P, int npts, double *out) {
    return guarded([&] {
        GooFit::Observable m12("m12", 0.0, 3.0), m13("m13", 0.0, 3.0);
        m12.setNumBins(bins);
        m13.setNumBins(bins);
        GooFit::EventNumber evt("eventNumber");
        GooFit::DecayInfo3 d;
        d.motherMass         = dec[0];
        d.daug1Mass          = dec[1];
        d.daug2Mass          = dec[2];
        d.daug3Mass          = dec[3];
        d.meson_radius       = dec[4];
        d.mother_meson_radius = dec[5];
        std::vector<GooFit::Variable> vars;
        for(int r = 0; r < nres; ++r) {
            const std::string nm = "res" + std::to_string(r);
            GooFit::Variable ar(nm + "_re", P[4 * r], 0.001, 0, 0), ai(nm + "_im", P[4 * r + 1], 0.001, 0, 0);
            GooFit::Variable m(nm + "_mass", P[4 * r + 2]), w(nm + "_width", P[4 * r + 3]);
            d.resonances.push_back(new GooFit::Resonances::RBW(nm, ar, ai, m, w, spin[r], cyc[r]));
            vars.insert(vars.end(), {ar, ai, m, w});
        }
        GooFit::Variable one("constantOne", 1), z0("constantZero0", 0), z1("constantZero1", 0);
        auto *eff = new GooFit::PolynomialPdf("constantEff", {m12, m13}, {one}, {z0, z1}, 0);
        auto *pdf = new GooFit::Amp3Body("signalPDF", m12, m13, evt, d, eff);
        GooFit::UnbinnedDataSet data({m12, m13, evt});
        for(long i = 0; i < n; ++i) {
            m12.setValue(m12s[i]);
            m13.setValue(m13s[i]);
            evt.setValue((double)i);
            data.addEvent();
        }
        pdf->setDataSize(data.getNumEvents());
        pdf->setData(&data);
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(*pdf, vars, P + (size_t)4 * nres * k);
    });
}

// The reference's own Dim5 (include/goofit/PDFs/physics/detail/Dim5.h) through the array evaluation MCBooster
// would run: n events of 4 daughters (E, px, py, pz) -> out[5][n] = m12, m34, cos12, cos34, phi.
int ref_dim5(const double *p4, long n, double *out) {
    return guarded([&] {
        std::vector<mcbooster::Particles_d> d(4, mcbooster::Particles_d(n));
        for(long i = 0; i < n; ++i)
            for(int k = 0; k < 4; ++k) {
                const double *q = p4 + ((size_t)i * 4 + k) * 4;
                d[k][i]         = mcbooster::Vector4R(q[0], q[1], q[2], q[3]);
            }
        mcbooster::ParticlesSet_d pset{&d[0], &d[1], &d[2], &d[3]};
        std::vector<mcbooster::RealVector_d> v(5, mcbooster::RealVector_d(n));
        mcbooster::VariableSet_d vset{&v[0], &v[1], &v[2], &v[3], &v[4]};
        GooFit::Dim5 eval;
        mcbooster::EvaluateArray<GooFit::Dim5>(eval, pset, vset);
        for(int j = 0; j < 5; ++j)
            for(long i = 0; i < n; ++i)
                out[(size_t)j * n + i] = v[j][i];
    });
}

// C5: Amp4Body of the benchmark's six decay chains of D0 -> pi+ pi- K- pi+ (masses[5] = parent and daughters),
// constant multivariate PolynomialPdf efficiency, normalisation events `norm_p4` (nnorm events of 4 daughters,
// (E, px, py, pz), handed to the phase-space stand-in).  ev = [m12 | m34 | cos12 | cos34 | phi] of n events.
// P[22 k ..] = (rho, K*, K1, a1, f0 mass and width) x 5, then (Re c, Im c) of the six amplitudes.
int ref_amp4_nll(const double *ev, long n, const double *masses, const double *norm_p4, long nnorm, const double *P,
                 int npts, double *out) {
    return guarded([&] {
        using namespace GooFit;
        Observable m12("m12", 0, 3), m34("m34", 0, 3), c12("cos12", -1, 1), c34("cos34", -1, 1), phi("phi", -3.5, 3.5);
        EventNumber evt("eventNumber");
        DecayInfo4 d;
        d.particle_masses = {masses[0], masses[1], masses[2], masses[3], masses[4]};
        d.meson_radius    = 1.5;
        Variable rho_m("rho_mass", P[0]), rho_w("rho_width", P[1]), kst_m("Kst_mass", P[2]), kst_w("Kst_width", P[3]),
            k1_m("K1_mass", P[4]), k1_w("K1_width", P[5]), a1_m("a1_mass", P[6]), a1_w("a1_width", P[7]),
            f0_m("f0_mass", P[8]), f0_w("f0_width", P[9]);
        using LRBW = Lineshapes::RBW;
        using LSBW = Lineshapes::SBW;
        auto krho = [&]() -> std::vector<Lineshape *> {
            return {new LRBW("rho(770)", rho_m, rho_w, 1, M_12), new LRBW("K*(892)", kst_m, kst_w, 1, M_34),
                    new LRBW("rho(770)", rho_m, rho_w, 1, M_24), new LRBW("K*(892)", kst_m, kst_w, 1, M_13)};
        };
        const double mD = masses[0];
        auto sf = [&](SF_4Body kind, std::array<unsigned, 4> a, std::array<unsigned, 4> b) -> std::vector<SpinFactor *> {
            return {new SpinFactor("SF", kind, mD, a[0], a[1], a[2], a[3]),
                    new SpinFactor("SF", kind, mD, b[0], b[1], b[2], b[3])};
        };
        struct Chain {
            std::string name;
            std::vector<Lineshape *> ls;
            std::vector<SpinFactor *> sfs;
        };
        std::vector<Chain> chains = {
            {"K*rho_S", krho(), sf(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_S, {0, 1, 2, 3}, {3, 1, 2, 0})},
            {"K*rho_P", krho(), sf(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_P, {0, 1, 2, 3}, {3, 1, 2, 0})},
            {"K*rho_D", krho(), sf(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_D, {0, 1, 2, 3}, {3, 1, 2, 0})},
            {"K1rho",
             {new LSBW("K1(1270)", k1_m, k1_w, 0, M_12_3), new LRBW("rho(770)", rho_m, rho_w, 1, M_12),
              new LSBW("K1(1270)", k1_m, k1_w, 0, M_24_3), new LRBW("rho(770)", rho_m, rho_w, 1, M_24)},
             sf(SF_4Body::DtoAP1_AtoVP2_VtoP3P4, {3, 2, 0, 1}, {0, 2, 3, 1})},
            {"a1rho",
             {new LSBW("a1(1260)", a1_m, a1_w, 0, M_12_4), new LRBW("rho(770)", rho_m, rho_w, 1, M_12),
              new LSBW("a1(1260)", a1_m, a1_w, 0, M_24_1), new LRBW("rho(770)", rho_m, rho_w, 1, M_24)},
             sf(SF_4Body::DtoAP1_AtoVP2_VtoP3P4, {2, 3, 0, 1}, {2, 0, 3, 1})},
            {"K*f0",
             {new LRBW("K*(892)", kst_m, kst_w, 1, M_34), new LRBW("f0(500)", f0_m, f0_w, 0, M_12),
              new LRBW("K*(892)", kst_m, kst_w, 1, M_13), new LRBW("f0(500)", f0_m, f0_w, 0, M_24)},
             sf(SF_4Body::DtoVS_VtoP1P2_StoP3P4, {2, 3, 0, 1}, {2, 0, 3, 1})},
        };
        std::vector<Variable> vars{rho_m, rho_w, kst_m, kst_w, k1_m, k1_w, a1_m, a1_w, f0_m, f0_w};
        for(size_t k = 0; k < chains.size(); ++k) {
            Variable ar(chains[k].name + "_re", P[10 + 2 * k], 0.01, 0, 0);
            Variable ai(chains[k].name + "_im", P[11 + 2 * k], 0.01, 0, 0);
            d.amplitudes.push_back(new Amplitude(chains[k].name, ar, ai, chains[k].ls, chains[k].sfs, 2));
            vars.push_back(ar);
            vars.push_back(ai);
        }
        Variable one("constantOne", 1), z0("constantZero0", 0), z1("constantZero1", 0);
        auto *eff = new PolynomialPdf("constantEff", {m12, m34}, {one}, {z0, z1}, 0);
        mcbooster::SetGeneratedEvents(norm_p4, nnorm, 4);
        auto *pdf = new Amp4Body("DK3pi", {m12, m34, c12, c34, phi, evt}, d, eff, (unsigned)nnorm);
        UnbinnedDataSet data({m12, m34, c12, c34, phi, evt});
        for(long i = 0; i < n; ++i) {
            m12.setValue(ev[i]);
            m34.setValue(ev[n + i]);
            c12.setValue(ev[2 * n + i]);
            c34.setValue(ev[3 * n + i]);
            phi.setValue(ev[4 * n + i]);
            evt.setValue((double)i);
            data.addEvent();
        }
        pdf->setDataSize(data.getNumEvents());
        pdf->setData(&data);
        for(int k = 0; k < npts; ++k)
            out[k] = evaluate(*pdf, vars, P + (size_t)22 * k);
    });
}

} // extern "C"
