// C++ host API check for the 4-body amplitude classes of goofit_gb300.hpp: the D0 -> K- pi+ pi+ pi- model
// (six decay chains of Lineshapes::RBW / SBW and SpinFactor, two permutations each) built with Amp4Body,
// DecayInfo4 and Amplitude as user code of the reference's API would build it.
//
//   amp4_examples tree <coefs>                     the flattened gf_node tree, one node per line
//   amp4_examples dim5 <n> <p4.bin> <out.bin>      Dim5 of n events of four (px, py, pz, E) 4-vectors
//   amp4_examples gen <n> <seed> <out.bin>         n normalisation events of the model's Amp4Body, SoA 5 x n
//   amp4_examples fit <prec> <coefs> <n> <data.bin> <nn> <norm.bin>
//                                                  fits the free coefficients to n events (SoA 6 x n doubles)
//                                                  normalised over nn given events (SoA 5 x nn)
// <coefs> is a text file of the twelve (Re, Im) coefficients; the first chain's pair is fixed, the other pairs
// float and start at 1.05 times the given values.
#include "goofit_gb300.hpp"

#include <cstdio>
#include <fstream>

using namespace GooFit;

namespace {

const double M = 1.865, MPI = 0.13957, MK = 0.4937;

std::vector<double> readBin(const char *path, size_t n) {
    std::vector<double> v(n);
    std::ifstream in(path, std::ios::binary);
    in.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(double)));
    if(!in)
        throw GeneralError(std::string("cannot read ") + path);
    return v;
}
void writeBin(const char *path, const std::vector<double> &v) {
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
}

struct Model {
    Observable m12{"m12", 0, 3}, m34{"m34", 0, 3}, c12{"cos12", -1, 1}, c34{"cos34", -1, 1}, phi{"phi", -3.5, 3.5};
    EventNumber evt{"eventNumber"};
    Variable rho_m{"rho_mass", 0.775}, rho_w{"rho_width", 0.149}, kst_m{"Kst_mass", 0.892},
        kst_w{"Kst_width", 0.050}, k1_m{"K1_mass", 1.272}, k1_w{"K1_width", 0.090}, a1_m{"a1_mass", 1.230},
        a1_w{"a1_width", 0.400}, f0_m{"f0_mass", 0.500}, f0_w{"f0_width", 0.400};
    std::vector<std::unique_ptr<Lineshape>> ls;
    std::vector<std::unique_ptr<SpinFactor>> sf;
    std::vector<std::unique_ptr<Amplitude>> amps;
    std::vector<Variable> coefs;
    std::unique_ptr<PolynomialPdf> eff;
    std::unique_ptr<Amp4Body> pdf;

    Lineshape *rbw(const char *n, Variable &m, Variable &w, unsigned L, unsigned pair) {
        ls.emplace_back(new Lineshapes::RBW(n, m, w, L, pair));
        return ls.back().get();
    }
    Lineshape *sbw(const char *n, Variable &m, Variable &w, unsigned L, unsigned pair) {
        ls.emplace_back(new Lineshapes::SBW(n, m, w, L, pair));
        return ls.back().get();
    }
    std::vector<SpinFactor *> sfPair(SF_4Body kind, std::vector<unsigned> a, std::vector<unsigned> b) {
        sf.emplace_back(new SpinFactor("SF", kind, M, a[0], a[1], a[2], a[3]));
        sf.emplace_back(new SpinFactor("SF", kind, M, b[0], b[1], b[2], b[3]));
        return {sf[sf.size() - 2].get(), sf.back().get()};
    }
    std::vector<Lineshape *> krho() {
        return {rbw("rho(770)", rho_m, rho_w, 1, M_12), rbw("K*(892)", kst_m, kst_w, 1, M_34),
                rbw("rho(770)", rho_m, rho_w, 1, M_24), rbw("K*(892)", kst_m, kst_w, 1, M_13)};
    }

    Model(const std::vector<double> &c, bool start, unsigned nNorm) {
        DecayInfo4 d;
        d.particle_masses = {M, MPI, MPI, MK, MPI};
        d.meson_radius    = 1.5;
        const char *names[6] = {"K*rho_S", "K*rho_P", "K*rho_D", "K1rho", "a1rho", "K*f0"};
        std::vector<std::pair<std::vector<Lineshape *>, std::vector<SpinFactor *>>> chains;
        chains.push_back({krho(), sfPair(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_S, {0, 1, 2, 3}, {3, 1, 2, 0})});
        chains.push_back({krho(), sfPair(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_P, {0, 1, 2, 3}, {3, 1, 2, 0})});
        chains.push_back({krho(), sfPair(SF_4Body::DtoV1V2_V1toP1P2_V2toP3P4_D, {0, 1, 2, 3}, {3, 1, 2, 0})});
        chains.push_back({{sbw("K1(1270)", k1_m, k1_w, 0, M_12_3), rbw("rho(770)", rho_m, rho_w, 1, M_12),
                           sbw("K1(1270)", k1_m, k1_w, 0, M_24_3), rbw("rho(770)", rho_m, rho_w, 1, M_24)},
                          sfPair(SF_4Body::DtoAP1_AtoVP2_VtoP3P4, {3, 2, 0, 1}, {0, 2, 3, 1})});
        chains.push_back({{sbw("a1(1260)", a1_m, a1_w, 0, M_12_4), rbw("rho(770)", rho_m, rho_w, 1, M_12),
                           sbw("a1(1260)", a1_m, a1_w, 0, M_24_1), rbw("rho(770)", rho_m, rho_w, 1, M_24)},
                          sfPair(SF_4Body::DtoAP1_AtoVP2_VtoP3P4, {2, 3, 0, 1}, {2, 0, 3, 1})});
        chains.push_back({{rbw("K*(892)", kst_m, kst_w, 1, M_34), rbw("f0(500)", f0_m, f0_w, 0, M_12),
                           rbw("K*(892)", kst_m, kst_w, 1, M_13), rbw("f0(500)", f0_m, f0_w, 0, M_24)},
                          sfPair(SF_4Body::DtoVS_VtoP1P2_StoP3P4, {2, 3, 0, 1}, {2, 0, 3, 1})});
        for(int k = 0; k < 6; ++k) {
            const std::string n = names[k];
            const double f      = (start && k > 0) ? 1.05 : 1.0;
            if(k == 0) {
                coefs.emplace_back(n + "_re", c[0]);
                coefs.emplace_back(n + "_im", c[1]);
            } else {
                coefs.emplace_back(n + "_re", f * c[2 * k], 0.01, 0, 0);
                coefs.emplace_back(n + "_im", f * c[2 * k + 1], 0.01, 0, 0);
            }
            amps.emplace_back(new Amplitude(n, coefs[2 * k], coefs[2 * k + 1], chains[k].first, chains[k].second, 2));
            d.amplitudes.push_back(amps.back().get());
        }
        eff.reset(new PolynomialPdf("constantEff", std::vector<Observable>{m12, m34},
                                    std::vector<Variable>{Variable("constantOne", 1)},
                                    std::vector<Variable>{Variable("constantZero0", 0), Variable("constantZero1", 0)},
                                    0));
        pdf.reset(new Amp4Body("DK3pi", {m12, m34, c12, c34, phi, evt}, d, eff.get(), nNorm));
    }
};

std::vector<double> readCoefs(const char *path) {
    std::ifstream in(path);
    std::vector<double> c;
    double v;
    while(in >> v)
        c.push_back(v);
    if(c.size() != 12)
        throw GeneralError("expected twelve coefficients");
    return c;
}

} // namespace

int main(int argc, char **argv) {
    if(argc < 2)
        return 2;
    const std::string mode = argv[1];
    if(mode == "tree") {
        Model m(readCoefs(argv[2]), false, 1000);
        PdfBase::Flat f = m.pdf->flatten();
        for(auto &p : f.params)
            std::printf("param %s %.17g %d\n", p.getName().c_str(), p.getValue(), p.IsFixed() ? 1 : 0);
        for(auto &o : f.obs)
            std::printf("obs %s %.17g %.17g %d\n", o.getName().c_str(), o.getLowerLimit(), o.getUpperLimit(),
                        o.isEventNumber() ? 1 : 0);
        for(auto &n : f.nodes) {
            std::printf("node %d %d |", n.op, n.flags);
            for(int i = 0; i < n.n_params; ++i)
                std::printf(" %d", n.params[i]);
            std::printf(" |");
            for(int i = 0; i < n.n_consts; ++i)
                std::printf(" %.17g", n.consts[i]);
            std::printf(" |");
            for(int i = 0; i < n.n_obs; ++i)
                std::printf(" %d", n.obs[i]);
            std::printf(" |");
            for(int i = 0; i < n.n_children; ++i)
                std::printf(" %d", n.children[i]);
            std::printf("\n");
        }
        return 0;
    }
    if(mode == "dim5") {
        const size_t n = std::stoul(argv[2]);
        const auto p4  = readBin(argv[3], 16 * n);
        std::vector<double> out(5 * n);
        for(size_t i = 0; i < n; ++i) {
            detail::P4 d[4];
            for(int j = 0; j < 4; ++j)
                d[j] = {p4[16 * i + 4 * j], p4[16 * i + 4 * j + 1], p4[16 * i + 4 * j + 2], p4[16 * i + 4 * j + 3]};
            double v[5];
            detail::dim5(d, v);
            for(int c = 0; c < 5; ++c)
                out[c * n + i] = v[c];
        }
        writeBin(argv[4], out);
        return 0;
    }
    if(mode == "gen") {
        const size_t n = std::stoul(argv[2]);
        writeBin(argv[4], detail::normEvents4({M, MPI, MPI, MK, MPI}, n, std::stoull(argv[3])));
        return 0;
    }
    if(mode == "fit") {
        const int precision = std::string(argv[2]) == "fp64" ? GF_FP64 : GF_MIXED;
        Model m(readCoefs(argv[3]), true, 1000);
        const size_t n = std::stoul(argv[4]), nn = std::stoul(argv[6]);
        const auto ev  = readBin(argv[5], 6 * n);
        m.pdf->setNormEvents(readBin(argv[7], 5 * nn));
        UnbinnedDataSet data({m.m12, m.m34, m.c12, m.c34, m.phi, m.evt});
        std::vector<double> row(6);
        for(size_t i = 0; i < n; ++i) {
            for(int c = 0; c < 6; ++c)
                row[c] = ev[c * n + i];
            data.addEvent(row);
        }
        m.pdf->setData(&data);
        FitManager fitter{m.pdf.get()};
        fitter.setVerbosity(0);
        fitter.setPrecision(precision);
        fitter.setTolerance(0.01);
        fitter.fit();
        std::printf("valid %d %.17g\n", bool(fitter) ? 1 : 0, fitter.result().fmin);
        for(auto &v : m.coefs)
            if(!v.IsFixed())
                std::printf("%s %.17g %.17g\n", v.getName().c_str(), v.getValue(), v.getError());
        return 0;
    }
    return 2;
}
