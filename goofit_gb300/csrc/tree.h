// Tree analysis for the likelihood engine: normalisation plan, gradient
// dependencies, convolution geometry and numeric-grid layout of one PDF tree.
#pragma once

#include "../../include/gfengine.h"

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace gf {

// How a node's normalisation factor is obtained on every FCN call.
enum NormKind {
    NK_ONE     = 0, // combine nodes (AddPdf/ProdPdf) and subtrees forced to 1 by
                    // recursiveSetNormalization (src/goofit/PdfBase.cpp:29-38)
    NK_EXP     = 1, // ExpPdf::integrate        (src/PDFs/basic/ExpPdf.cu:121-132)
    NK_GAUSS   = 2, // GaussianPdf::integrate   (src/PDFs/basic/GaussianPdf.cu:28-35)
    NK_NUMERIC = 3, // grid sum                 (src/PDFs/GooPdf.cu:366-395)
    NK_AMP3    = 4, // Amp3Body::normalize: c^H I c over the cached resonance integrals
                    // (src/PDFs/physics/Amp3Body.cu:238-359), evaluated on the host
    NK_AMP4    = 5  // Amp4Body::normalize: c^H G c / N over the flat phase-space events
                    // (src/PDFs/physics/Amp4Body.cu:398-558), evaluated on the host
};

struct TNode {
    int op = 0, flags = 0;
    std::vector<int> params;
    std::vector<double> consts;
    std::vector<int> obs;
    std::vector<int> children;
    int ibins = 0;
};

// Geometry of one ConvolutionPdf (src/PDFs/combine/ConvolutionPdf.cu:228-282).
struct ConvInfo {
    int node = -1, model = -1, resol = -1, obs = -1;
    double lo = 0, hi = 0, step = 0;
    double ic[6]  = {0, 0, 0, 0, 0, 0}; // host_iConsts
    int nM = 0, nR = 0, offset = 0;
    int kmin = 0, kmax = 0, nK = 0; // bin-offset range of x in [obs.lo, obs.hi]
    std::vector<int> dep;           // gradient slots the table depends on
};

// A floated resonance / line-shape parameter of an amplitude node with an analytic gradient: the amplitudes
// that depend on it get one derivative column each (dA_a / dparam per event), and the normalisation one
// matrix H_ab = sum over normalisation points of dA_a/dparam conj(A_b) (times the efficiency for Amp3Body).
struct AmpTheta {
    int slot = -1, param = -1;
    std::vector<int> amps; // dependent amplitudes (indices within the node)
    int col0 = 0;          // first derivative column
};

// One Amp3Body node (src/PDFs/physics/Amp3Body.cu:127-196): resonances, efficiency, decay constants and
// the normalisation grid (m12^2 x m13^2 bin centres; the m13 bin count is read from the m12 slot as
// src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:72 does).
struct Amp3Info {
    int node = -1, nRes = 0, eff = -1, o12 = -1, o13 = -1;
    std::vector<int> res;     // resonance nodes
    int col0 = 0;             // first amplitude column of this node
    double M = 0, m1 = 0, m2 = 0, m3 = 0, r = 0, rm = 0;
    int nb12 = 0, nb13 = 0, nb13q = 0;
    double area = 0;          // bin size of m12 times bin size of m13
    std::vector<int> cache_params; // parameters the cached amplitudes and integrals depend on
    std::vector<uint32_t> grid;    // in-Dalitz normalisation bins, b12 | b13 << 16 (FP64 inDalitz)
    std::vector<AmpTheta> theta;
};

// One Amp4Body node (src/PDFs/physics/Amp4Body.cu:94-292): amplitudes built from line shapes and spin
// factors, both de-duplicated by value across amplitudes as the constructor does (lines 122-158).
struct Amp4Info {
    int node = -1, nAmp = 0, eff = -1;
    int obs[5] = {-1, -1, -1, -1, -1}; // m12, m34, cos12, cos34, phi
    double M = 0, m[4] = {0, 0, 0, 0};
    std::vector<int> ls, sf; // representative node of every distinct line shape / spin factor
    struct Amp {
        int node = -1, nPerm = 1;
        std::vector<int> ls, sf; // indices into Amp4Info::ls / sf, in the amplitude's child order
    };
    std::vector<Amp> amps;
    int col0 = 0;                  // first amplitude column of this node
    std::vector<int> cache_params; // line-shape (and efficiency) parameters
    std::vector<AmpTheta> theta;
};

// inDalitz (src/PDFs/physics/DalitzPlotHelpers.cu:14-59), FP64 without contraction.
bool in_dalitz(double m12, double m13, double bigM, double dm1, double dm2, double dm3);

// One numerically normalised node: grid over its observables.
struct NumInfo {
    int node = -1;
    std::vector<int> obs;
    std::vector<int> nbins;
    int64_t total  = 1;
    double volume  = 1;
    std::vector<int> convs;       // conv nodes inside the subtree
    std::vector<int> conv_axis;   // axis of each conv's observable in this grid
    std::vector<int64_t> kgrid_off; // offset of each conv's per-axis-bin k table in the kgrid buffer
};

struct Tree {
    std::vector<TNode> nodes;
    std::vector<gf_observable> obs;
    int n_params = 0;
    std::vector<int> gslot; // parameter -> gradient slot or -1
    std::vector<int> gparam; // gradient slot -> parameter
    int NG = 0;

    std::vector<int> nk;
    std::vector<std::vector<int>> dep_val, dep_norm; // sorted gradient slots
    std::vector<ConvInfo> convs;
    std::vector<int> conv_of; // node -> index in convs or -1
    std::vector<NumInfo> nums;
    std::vector<int> num_of; // node -> index in nums or -1
    std::vector<int> kgrid;  // host copy of all grid k tables
    int fit_metric = GF_FIT_UNBINNED_NLL; // binned metrics: the last two observables are content and volume/error
    std::vector<Amp3Info> amp3s;
    std::vector<int> amp3_of; // node -> index in amp3s or -1
    std::vector<Amp4Info> amp4s;
    std::vector<int> amp4_of; // node -> index in amp4s or -1
    // amplitude nodes of both kinds share one numbering: Amp3Body nodes first, then Amp4Body nodes
    int n_amp_nodes() const { return (int)(amp3s.size() + amp4s.size()); }
    int amp_index(int node) const {
        return amp3_of[node] >= 0 ? amp3_of[node] : (amp4_of[node] >= 0 ? (int)amp3s.size() + amp4_of[node] : -1);
    }
    int amp_count(int k) const { return k < (int)amp3s.size() ? amp3s[k].nRes : amp4s[k - amp3s.size()].nAmp; }
    int amp_node(int k) const { return k < (int)amp3s.size() ? amp3s[k].node : amp4s[k - amp3s.size()].node; }
    int amp_col0(int k) const { return k < (int)amp3s.size() ? amp3s[k].col0 : amp4s[k - amp3s.size()].col0; }
    const std::vector<int> &amp_cache_params(int k) const {
        return k < (int)amp3s.size() ? amp3s[k].cache_params : amp4s[k - amp3s.size()].cache_params;
    }
    const std::vector<AmpTheta> &amp_theta(int k) const {
        return k < (int)amp3s.size() ? amp3s[k].theta : amp4s[k - amp3s.size()].theta;
    }
    int n_amp_cols = 0;       // complex amplitude columns per toy
    bool extended_root = false;

    // Returns "" on success, else the reason the tree is rejected.
    std::string build(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                      const int32_t *grad_mask);

    std::vector<int> subtreeObs(int i) const;
    bool inSubtree(int root, int i) const;
    bool prodOverlaps(int i) const;
};

// ConvolutionPdf bin offset of x (src/PDFs/combine/ConvolutionPdf.cu:40-43), in FP64.
inline int conv_offset_in_bins(double x0, double loBound, double step) {
    double lowerBoundOffset = loBound / step;
    lowerBoundOffset -= std::floor(lowerBoundOffset);
    return (int)std::floor(x0 / step - lowerBoundOffset);
}

// Bin centre of the binned MetricTaker (src/PDFs/MetricTaker.cu:76-82), in FP64.
inline double bin_centre(double lo, double hi, int nbins, int b) {
    double x = hi - lo;
    x /= nbins;
    x *= (b + 0.5);
    x += lo;
    return x;
}

// Where every normalisation factor lives during an evaluation.
//   record (type R, one per toy): [0, n_params) parameters, then the analytic factors the host computes
//   from the parameters before each launch (ExpPdf::integrate and GaussianPdf::integrate run on the host
//   in the reference too, src/PDFs/basic/ExpPdf.cu:121-132, src/PDFs/basic/GaussianPdf.cu:28-35);
//   numeric array (type R, one per toy): the factors of numerically normalised nodes, written by the
//   finishing CTA of the grid kernel.
struct NormLayout {
    // every factor N is kept as hi + lo (lo = N - hi rounded; 0 in FP64), so that FP32 products v * N carry
    // no systematic rounding of N
    struct Analytic {
        int node = -1, kind = 0, slotN = -1, slotNL = -1;
        std::vector<std::pair<int, int>> dN; // (gradient slot, record index)
    };
    int npr = 0; // record length
    std::vector<Analytic> analytic;
    int nq = 0;                                        // numeric slots per toy
    std::vector<int> qN;                               // per numeric node q: slot of N
    std::vector<int> qNL;                              // per numeric node q: slot of the low part of N
    std::vector<std::vector<std::pair<int, int>>> qdN; // per q: (gradient slot, slot of dN)
};
NormLayout norm_layout(const Tree &t);

// Generates the CUDA source of the fused kernel set for a tree.
struct KernelPlan {
    std::string source;
    size_t evt_smem_grad = 0, evt_smem_nograd = 0; // dynamic shared memory of the event kernels
    bool recompute_kernels = false; // gf_evt_gr and gf_gramr were generated (amplitude recompute mode)
    size_t evt_smem_gr     = 0;     // dynamic shared memory of gf_evt_gr
    size_t conv_smem_grad = 0, conv_smem_nograd = 0;
    int conv_tk = 64;      // table entries per conv CTA
    int conv_blocks = 0;   // CTAs per (toy, conv) of the table kernel
    int grid_bins_per_block = 256; // 1024 for batches of toys
    int conv_kp             = 1;   // table k-tiles per staged model and resolution (batches of toys)
    std::vector<int> grid_blocks; // per numeric node
    int max_grid_blocks = 0;      // also covers the conv kernel's folded grid sums
    // A numeric node that is a ConvolutionPdf on a 1-D grid has the grid sum sum_b T[k(b)] = sum_k n_k T[k]
    // (n_k: grid bins with bin offset k): in kernels shaped for batches of toys the conv kernel accumulates
    // it and finishes the node's normalisation, and the grid kernel skips the node.
    std::vector<int> conv_fold_q; // per conv: folded numeric node or -1
    std::vector<char> num_folded; // per numeric node
    bool grid_needs_conv = false; // an unfolded numeric node reads a convolution table
    int64_t ctab_per_toy_grad = 0, ctab_per_toy_nograd = 0; // table elements per toy
    std::vector<int64_t> ctab_off_grad, ctab_off_nograd;    // per conv
    // mixed precision, one toy: the low parts of conv 0's values (the table's value column holds the high parts
    // of unevaluated FP32 pairs), at this element offset of the toy's table block; -1 when not kept
    int64_t ctab_lo_off_grad = -1, ctab_lo_off_nograd = -1;
    std::vector<int> ctab_cp_grad, ctab_cp_nograd;          // per conv: padded components per table row
    std::vector<int> obs_used_evt;                          // observables the event kernel loads
    // Amp3Body integrals: pairs (i <= j) of each node split into tiles; one CTA row per tile
    struct GramTile {
        int amp, p0, p1; // node index in Tree::amp3s, pair range
    };
    std::vector<GramTile> gram_tiles;
    int gram_pairs_max = 0;                                 // most pairs in one tile
    std::vector<int64_t> dgrid_off;                         // per Amp3Body: offset of its bins in the bin list
    // the root's normalisation is applied on the host: the event pass returns sum -log P, sum -dP/P and the
    // count of events with P > 0 (out[2 + NG]); the host adds count * (-log N) and count * (-dN/N)
    bool factor_root = false;
    // one toy: the whole evaluation as one cooperative launch (gf_fcn_g / gf_fcn_n), [nograd, grad]
    bool fused = false;
    bool fused_tab = false;             // its event pass gathers per-k tabulated terms (event function of k alone)
    size_t fused_smem[2] = {0, 0};      // dynamic shared memory, staged events included
    size_t fused_stage_off[2] = {0, 0}; // where the staged events start (after the tables' working space)
    size_t fused_stage_cap[2] = {0, 0}; // and the bytes of them that fit
    int fused_row[2] = {0, 0};          // doubles per chunk row it writes to host memory (components, status)
    NormLayout nl;
};

// batch: kernels shaped for many toys per launch (fewer, larger table and grid CTAs)
// Launch shapes the autotuner varies (0: the generator's default): table k-tiles per staged model and resolution
// (batches of toys), numeric-grid bins per CTA.
struct Shapes {
    int conv_kp  = 0;
    int grid_bpb = 0;
};
KernelPlan generate_kernels(const Tree &t, bool mixed, int evt_block, bool batch, const Shapes &shapes = Shapes());

} // namespace gf
