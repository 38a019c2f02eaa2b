// C++ host API check: the reference's own fit scenarios written against goofit_gb300.hpp.
//   1. tests/simple/BinningTest.cpp "Unbinned" section style: ExpPdf on mt19937(137) exponential(1.5) draws
//      (with MINOS errors the second time)
//   2. tests/simple/BinningTest.cpp "Binned" style: the same draws in a BinnedDataSet, BinnedNllFit and
//      BinnedChisqFit
//   3. the composite model: AddPdf(Convolution(Exp, Gauss), flat Polynomial) on given data
// Prints one line per fit: valid flag, then value and error of every free parameter.
#include "goofit_gb300.hpp"

#include <cstdio>
#include <fstream>
#include <random>

using namespace GooFit;

int main(int argc, char **argv) {
    const int precision = (argc > 1 && std::string(argv[1]) == "fp64") ? GF_FP64 : GF_MIXED;
    {
        std::mt19937 gen(137);
        std::exponential_distribution<> d(1.5);
        Observable xvar{"xvar", 0, 10};
        UnbinnedDataSet data{xvar};
        for(int i = 0; i < 100000; ++i) {
            double val = d(gen);
            if(val < 10) {
                xvar.setValue(val);
                data.addEvent();
            }
        }
        Variable alpha{"alpha", -2, 0.1, -10, 10};
        ExpPdf exppdf{"exppdf", xvar, alpha};
        exppdf.setData(&data);
        FitManager fitter{&exppdf};
        fitter.setVerbosity(0);
        fitter.setPrecision(precision);
        fitter.setTolerance(0.01);
        fitter.fit();
        std::printf("exp %d %.12g %.12g\n", bool(fitter) ? 1 : 0, alpha.getValue(), alpha.getError());

        // the same fit with MINOS errors
        alpha.setValue(-2);
        alpha.setError(0.1);
        FitManager mfitter{&exppdf};
        mfitter.setVerbosity(0);
        mfitter.setPrecision(precision);
        mfitter.setTolerance(0.01);
        mfitter.setMinos();
        mfitter.fit();
        const auto me = mfitter.getMinosErrors();
        std::printf("minos %d %.12g %.12g %.12g %.12g\n", bool(mfitter) ? 1 : 0, alpha.getValue(), alpha.getError(),
                    me.at(0).first, me.at(0).second);
    }
    {
        // tests/simple/BinningTest.cpp "Binned" style: the exponential draws filled into 100 bins, fitted with
        // the binned Poisson likelihood and with the chi-square
        for(int kind = 0; kind < 2; ++kind) {
            std::mt19937 gen(137);
            std::exponential_distribution<> d(1.5);
            Observable xvar{"xvar", 0, 10};
            BinnedDataSet data{xvar};
            for(int i = 0; i < 100000; ++i) {
                double val = d(gen);
                if(val < 10) {
                    xvar.setValue(val);
                    data.addEvent();
                }
            }
            Variable alpha{"alpha", -1.4, 0.1, -10, 10};
            ExpPdf exppdf{"exppdf", xvar, alpha};
            exppdf.setData(&data);
            if(kind == 1)
                exppdf.setFitControl(std::make_shared<BinnedChisqFit>());
            FitManager fitter{&exppdf};
            fitter.setVerbosity(0);
            fitter.setPrecision(precision);
            fitter.setTolerance(0.01);
            fitter.fit();
            std::printf("%s %d %.12g %.12g\n", kind ? "binned_chisq" : "binned_nll", bool(fitter) ? 1 : 0,
                        alpha.getValue(), alpha.getError());
        }
    }
    if(argc > 2) {
        // composite model on events read from a text file (one x per line)
        Observable x{"x", -5, 10};
        x.setNumBins(10000);
        UnbinnedDataSet data{x};
        std::ifstream in(argv[2]);
        double v;
        while(in >> v) {
            x.setValue(v);
            data.addEvent();
        }
        Variable alpha{"alpha", -0.6, 0.05, -2.0, -0.1};
        Variable mu{"mu", 0.05, 0.02, -1.0, 1.0};
        Variable sigma{"sigma", 0.35, 0.02, 0.05, 1.0};
        Variable c0{"c0", 1.0};
        Variable fsig{"fsig", 0.65, 0.02, 0.0, 1.0};
        ExpPdf model{"model", x, alpha};
        GaussianPdf resol{"resolution", x, mu, sigma};
        ConvolutionPdf conv{"signal", x, &model, &resol};
        conv.setIntegrationConstants(0.0, 10.0, 0.01);
        PolynomialPdf bkg{"background", x, {c0}, 0};
        AddPdf total{"total", fsig, &conv, &bkg};
        total.setData(&data);
        FitManager fitter{&total};
        fitter.setVerbosity(0);
        fitter.setPrecision(precision);
        fitter.setTolerance(0.01);
        fitter.fit();
        std::printf("composite %d %.12g %.12g %.12g %.12g %.12g %.12g %.12g %.12g\n", bool(fitter) ? 1 : 0,
                    fsig.getValue(), fsig.getError(), alpha.getValue(), alpha.getError(), mu.getValue(), mu.getError(),
                    sigma.getValue(), sigma.getError());
    }
    return 0;
}
