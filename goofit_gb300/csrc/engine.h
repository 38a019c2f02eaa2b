// Internal state of a likelihood engine handle.
#pragma once

#include "../../include/gfengine.h"
#include "tree.h"

#include <cuda_runtime.h>

#include <string>
#include <vector>

struct GfArgs {
    const double *P;
    const int *active;
    const void *const *col;
    const int *const *kcol;
    void *ctab;
    const int *kgrid;
    double *gsum;
    double *gpartial;
    unsigned *gcounter;
    double *partial;
    unsigned *counter;
    double *out;
    const long long *chunks;
    const int *toy_chunk0;
    const int *toy_nchunks;
    const long long *toy_nevents;
    double *vals;
    const void *Pr;
    void *Nq;
    int *qflag;
    const void *const *acol;
    const double *const *dcol;
    const unsigned *dgrid;
    double *gram;
    const int *dirty;
    const double *const *nevt;
    const long long *nnorm;
    void *const *nscr;
    int n_chunks;
    int n_toys;
    int metric;
    int gtoy;
    long long chunk;      // events per chunk
    long long nevt0;      // events of toy 0
    unsigned *gbar;       // grid barrier words of the one-launch evaluation [arrivals, unused, error]
    unsigned long long bar_ns; // longest barrier wait (ns) before the one-launch kernel gives up
    int rec_n;            // one-launch evaluation: the toy's record (rec_n R values) passed by value in rec
    int stage_off;        // one-launch evaluation: shared-memory offset and room (bytes) of the staged events
    unsigned stage_cap;
    unsigned bar_target;  // the arrival count at which this launch's grid barrier opens
    double *hpart;        // one-launch evaluation: per-chunk [components..., status] rows in page-locked memory
    const int *ksort;     // one-launch tabulated path: toy 0's bin offsets sorted by bin (null: read kcol)
    alignas(16) unsigned char rec[512];
    const void *p0[192];  // toy 0: observable columns, bin-offset columns, amplitude columns (one toy only)
};

struct GfToy {
    int64_t n    = 0;
    int64_t npad = 0;
    double total = 0; // number of events: n, or the summed bin contents of binned data
    void *cols[16] = {nullptr};
    int *kcols[8]  = {nullptr};
    int *ksort     = nullptr;           // one-launch tabulated path: the bin offsets of conv 0 sorted by bin
    bool ksort_valid = false;
    unsigned *khist = nullptr;          // the sort's histogram (khist_n bins)
    int khist_n      = 0;
    void *abase    = nullptr;           // cached resonance amplitudes and FP64 Dalitz columns (one allocation)
    void *acols[128] = {nullptr};       // R2 per event: amplitude columns, then derivative columns
    double *dcols[16] = {nullptr};      // FP64 event columns of the Dalitz variables
    bool loaded    = false;
    bool amp_valid  = false;            // the per-event amplitude columns match amp_params and the events
    bool norm_valid = false;            // the integrals (amp_I, amp_H) match amp_params
    std::vector<double> amp_params;     // parameter values the cache and integrals were built with
    std::vector<std::vector<double>> amp_I; // per amplitude node: n x n complex integrals, interleaved
    std::vector<std::vector<double>> amp_H; // per amplitude node: (derivative rows) x n complex, interleaved
};

struct GfModule {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t conv_g = nullptr, conv_n = nullptr, grid_g = nullptr, grid_n = nullptr;
    cudaKernel_t evt_g = nullptr, evt_n = nullptr, val_n = nullptr;
    cudaKernel_t amp = nullptr, ampn = nullptr, gram = nullptr;
    cudaKernel_t evt_gr = nullptr, gramr = nullptr; // amplitude recompute mode (gradient pass, integrals)
    cudaKernel_t fcn_g = nullptr, fcn_n = nullptr; // one toy: the whole evaluation in one cooperative launch
};

struct gf_engine {
    int device    = 0;
    int precision = GF_MIXED;
    int sm_count  = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    bool has_tree = false;
    gf::Tree tree;
    gf::KernelPlan plan;
    GfModule mod;
    int block = 256;
    int chunk = 8192;
    bool chunk_fixed = false;
    int evt_ctas_per_sm = 4;      // resident event CTAs per SM: the gradient event kernel's occupancy
    bool evt_ctas_fixed = false;
    bool batch_kernels  = false;  // kernels generated for a batch of toys (n_toys > 1)
    bool tune_pending   = false;  // the next evaluation runs the event-chunking autotuner
    int tuned_chunk     = 0;      // chunk size the autotuner chose (0: not tuned)
    int chunk_cap       = 0;      // chunks the chunk list and partials have room for

    // amplitude derivatives (enum gf_amp_mode): stored per event and per normalisation point, or recomputed
    // where they are used; auto recomputes when storing them would take more than amp_budget bytes (0: a
    // quarter of the free device memory).  Decided at the first event upload after gf_set_tree.
    int amp_mode         = GF_AMP_AUTO;
    int64_t amp_budget   = 0;
    bool amp_recompute   = false;
    bool amp_decided     = false;

    // launch shapes (gf_tune_shapes): the generator's table k-tiles and grid bins per CTA, and the tensor-core
    // Gram kernel's slice width (0: the defaults)
    gf::Shapes shapes;
    int gram_w = 0;

    int fit_metric = GF_FIT_UNBINNED_NLL;
    int n_toys = 1;
    std::vector<GfToy> toys;

    // device buffers
    double *d_P = nullptr;
    int *d_active = nullptr;
    void **d_cols = nullptr;
    int **d_kcols = nullptr;
    void *d_ctab = nullptr;
    int *d_kgrid = nullptr;
    double *d_gsum = nullptr, *d_gpartial = nullptr;
    unsigned *d_gcounter = nullptr;
    double *d_partial = nullptr;
    unsigned *d_counter = nullptr;
    double *d_out = nullptr;
    long long *d_chunks = nullptr;
    int *d_toy_chunk0 = nullptr, *d_toy_nchunks = nullptr;
    long long *d_toy_nevents = nullptr;
    double *d_vals = nullptr;
    int64_t vals_cap = 0;
    double *d_stage = nullptr; // FP64 staging of uploads (grow-only)
    int64_t stage_cap = 0;
    int *h_uperr = nullptr;
    void **d_acols = nullptr;    // [toy][amplitude column]
    double **d_dcols = nullptr;  // [toy][observable]
    unsigned *d_dgrid = nullptr; // in-Dalitz bins of every Amp3Body
    double *d_gram = nullptr;    // integral partials [toy][tile][CTA][2 * pairs]
    double *h_gram = nullptr;
    int *d_dirty = nullptr, *h_dirty = nullptr;
    int gram_blocks = 0;
    // Amp4Body normalisation events, one FP64 SoA [5][n] buffer per Amp4Body node (gf_set_norm_events)
    std::vector<double *> norm_buf;
    std::vector<int64_t> norm_n;
    double **d_nevt = nullptr;
    long long *d_nnorm = nullptr;
    // normalisation-point columns per amplitude node (values, derivatives, efficiency) of one toy at a time
    // tensor-core Gram (mixed precision): per-CTA FP64 partials, the summed real Gram matrix, a status word
    bool gram_tc         = false;
    double *d_gtc_part   = nullptr;
    double *d_gtc_out    = nullptr;
    int *d_gtc_err       = nullptr;
    size_t gtc_part_n    = 0, gtc_out_n = 0;
    std::vector<double> h_gtc;
    std::vector<void *> nscr;
    std::vector<size_t> nscr_bytes;
    void **d_nscr = nullptr;
    void *d_Nq = nullptr;   // [toy][nq] R numeric normalisation factors
    int *d_qflag = nullptr; // [toy]
    // pinned host mirrors; h_P is one block: [toy][n_params] FP64, then [toy][npr] R records
    double *h_P = nullptr;
    size_t pblock_bytes = 0;
    size_t active_off   = 0; // byte offset of the active flags inside the parameter block
    std::vector<int> host_flag; // per toy: status bits from host-computed analytic factors
    std::vector<double> root_N, root_dN; // per toy: the root's normalisation and its derivatives, FP64
    int *h_active = nullptr;
    double *h_out = nullptr;

    int n_chunks = 0;
    bool layout_ready = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // device time of the last evaluation (CUDA events around it); after a one-launch evaluation whose rows the
    // host read before the launch ended, it is read from the events when first asked for
    mutable double last_ms_total = 0;
    double last_ms_evt = 0;
    mutable bool timing_pending = false;
    bool use_graph = true;
    bool fused_direct = false; // GF_FUSED_DIRECT=1: the one-launch kernel is launched directly, not replayed from a graph
    std::vector<double> fsum; // the host's sums of the one-launch rows
    bool wait_sync = false;   // GF_WAIT_SYNC=1: the host synchronises the stream before it reads the one-launch rows
    bool use_pdl   = true;
    // one-launch evaluation (one toy, unbinned NLL): resident CTAs of the cooperative launch, the barrier
    // words it synchronises on and the longest barrier wait before it gives up (GF_FUSED=0: three launches)
    bool use_fused        = true;
    bool use_stage        = true; // GF_STAGE=0: the one-launch kernel reads events from global memory
    bool use_ksort        = true; // GF_KSORT=0: its tabulated event pass reads the offsets in upload order
    int fcn_grid          = 0;
    unsigned *d_gbar      = nullptr;
    unsigned long long bar_ns = 1000000000ull;
    unsigned long long gram_ns = 0; // per-stage wait limit of the tensor-core Gram kernel (0: its 2 s default)
    unsigned bar_epoch        = 0; // one-launch evaluations run since the barrier words were cleared
    bool fused_graph_ok   = true; // false: the cooperative launch is not captured into a graph here
    // captured one-launch graphs [nograd, grad]: the source graph, its kernel node and that node's launch
    // parameters, whose arguments (the toy's record by value) are replaced before every graph launch
    cudaGraph_t graph_src[2]         = {nullptr, nullptr};
    cudaGraphNode_t fused_node[2]    = {nullptr, nullptr};
    cudaKernelNodeParams fused_kp[2] = {};
    // the one-launch kernel's per-chunk rows (mapped page-locked memory), chunk_cap rows of fused_row doubles
    double *h_fpart = nullptr, *d_fpart = nullptr;
    int fused_row   = 0;
};

// helpers shared between translation units
int gf_fail(gf_engine *e, int code, const std::string &msg);

// tensor-core Gram matrix of ncol complex FP32 columns (gram_tc.cu): real columns per slice (16, 32 or 64),
// 0 when 2 ncol > 64
int gf_gram_tc_width(int ncol);
size_t gf_gram_tc_part_doubles(int ncol, int grid);
// G (2 ncol x 2 ncol, FP64) = sum_{p < npts} x_r(p) eff(p) x_s(p) of the columns sc[c * nst + p] (nst a
// multiple of 4, sc and eff 16-byte aligned) into out; part holds gf_gram_tc_part_doubles(ncol, sm_count)
// doubles; *err gets bit 0 when a bounded wait ran out; width: real columns per slice (16, 32 or 64, at least
// gf_gram_tc_width(ncol)), 0 for the narrowest; wait_ns: the limit of each per-stage mbarrier wait (0: 2 s; the
// wait for the last committed MMAs before the tensor memory is freed is always 2 s); stall >= 0: a test of the
// failure path, in which the wait for stage `stall` also waits on a barrier that never completes
cudaError_t gf_gram_tc_launch(const float2 *sc, long long npts, long long nst, int ncol, const float *eff,
                              int sm_count, double *part, double *out, int *err, cudaStream_t s, int width = 0,
                              unsigned long long wait_ns = 0, int stall = -1);
int gf_cuda_check(gf_engine *e, cudaError_t r, const char *what);
int gf_run(gf_engine *e, bool grad, int metric_values_toy, int metric);
