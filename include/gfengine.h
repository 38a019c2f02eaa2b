/*
 * gfengine.h — C ABI of the GB300 likelihood engine (libgfengine.so).
 *
 * This is the drop-in boundary for GooFit's fit path.  In the reference every
 * PDF registers a device function pointer (`device_function_ptr`,
 * include/goofit/PDFs/detail/Globals.h:12) into a process-global table that a
 * Thrust functor (MetricTaker, src/PDFs/MetricTaker.cu:17-44) calls per event,
 * and the host drives it through PdfBase/GooPdf (`setData`
 * src/PDFs/PdfBase.cu:329-438, `normalize` src/PDFs/GooPdf.cu:340-396,
 * `calculateNLL` src/PDFs/GooPdf.cu:254-273) and Minuit2 (`FCN::operator()`
 * src/goofit/FCN.cpp:18-28).
 *
 * Here a PDF tree is handed over once as a flat node list (`gf_node`, one
 * entry per PdfBase object in the same depth-first order that
 * PdfBase::populateArrays flattens it, src/PDFs/PdfBase.cu:268-311).  The
 * engine generates one fused kernel set for that tree, keeps events resident
 * in HBM as structure-of-arrays columns, and answers NLL / gradient queries.
 *
 * Conventions: every function returns GF_OK (0) or a gf_status code and never
 * throws or aborts; gf_last_error() gives the message.  Host arrays are
 * caller-owned and copied.  Sizes are element counts.
 */
#ifndef GFENGINE_H
#define GFENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (GooFit::abort sites: src/PDFs/GooPdf.cu:260-271,381-391) ---- */
enum gf_status {
    GF_OK              = 0,
    GF_ERR_INVALID     = 1,  /* bad argument / size / index */
    GF_ERR_CUDA        = 2,  /* CUDA runtime error */
    GF_ERR_COMPILE     = 3,  /* runtime code generation failed */
    GF_ERR_NAN_NORM    = 4,  /* "NaN in normalization" */
    GF_ERR_NONPOS_NORM = 5,  /* "non-positive normalization" */
    GF_ERR_ZERO_NLL    = 6,  /* "zero NLL" */
    GF_ERR_OOM         = 7,
    GF_ERR_TIMEOUT     = 8,
    GF_ERR_BAD_TREE    = 9,
    GF_ERR_STATE       = 10, /* call order (no tree / no data) */
    GF_ERR_NO_DEVICE   = 11
};

/* ---- arithmetic of the per-event path ---- */
enum gf_precision {
    GF_FP64  = 0, /* every event, workspace and reduction in FP64 (the plain path) */
    GF_MIXED = 1  /* FP32 events and per-event PDF math, FP64 reductions and normalisations */
};

/* ---- node operators: one per reference device function ---- */
enum gf_op {
    GF_OP_EXP               = 1,  /* device_Exp            src/PDFs/basic/ExpPdf.cu:7-17      params [alpha] */
    GF_OP_EXP_OFFSET        = 2,  /* device_ExpOffset      src/PDFs/basic/ExpPdf.cu:19-30     params [x0, alpha] */
    GF_OP_EXP_POLY          = 3,  /* device_ExpPoly        src/PDFs/basic/ExpPdf.cu:32-46     params [w0..wn] */
    GF_OP_EXP_POLY_OFFSET   = 4,  /* device_ExpPolyOffset  src/PDFs/basic/ExpPdf.cu:48-63     params [x0, w..] */
    GF_OP_GAUSSIAN          = 5,  /* device_Gaussian       src/PDFs/basic/GaussianPdf.cu:7-17 params [mean, sigma] */
    GF_OP_POLYNOMIAL        = 6,  /* device_Polynomial     src/PDFs/basic/PolynomialPdf.cu:8-26  consts [lowestDegree] params [c..] */
    GF_OP_POLYNOMIAL_OFFSET = 7,  /* device_OffsetPolynomial src/PDFs/basic/PolynomialPdf.cu:28-44 consts [lowestDegree] params [c.., x0] */
    GF_OP_ADD               = 8,  /* device_AddPdfs        src/PDFs/combine/AddPdf.cu:16-51   params [f1..f(n-1)] children n */
    GF_OP_ADD_EXT           = 9,  /* device_AddPdfsExt     src/PDFs/combine/AddPdf.cu:53-80   params [N1..Nn] children n */
    GF_OP_PROD              = 10, /* device_ProdPdfs       src/PDFs/combine/ProdPdf.cu:9-26   consts [nComps] children n */
    GF_OP_CONVOLUTION       = 11, /* device_ConvolvePdfs   src/PDFs/combine/ConvolutionPdf.cu:27-75 consts [lo, hi, step] children [model, resolution] */
    GF_OP_AMP3BODY          = 12, /* device_DalitzPlot     src/PDFs/physics/Amp3Body.cu:60-122
                                     consts [nRes, cache, M, m1, m2, m3, mesonRadius, motherRadius]
                                     params [Re c0, Im c0, Re c1, ...] obs [m12^2, m13^2, eventNumber]
                                     children [resonance 0 .. n-1, efficiency] */
    GF_OP_AMP4BODY          = 13, /* device_DP             src/PDFs/physics/Amp4Body.cu:53-90
                                     consts [M, m1, m2, m3, m4, cache] params [Re c0, Im c0, ...]
                                     obs [m12, m34, cos12, cos34, phi, eventNumber]
                                     children [amplitude 0 .. n-1, efficiency]; normalised over the flat
                                     phase-space events given with gf_set_norm_events */
    GF_OP_MULTIPOLYNOMIAL   = 14, /* device_MultiPolynomial src/PDFs/basic/PolynomialPdf.cu:46-107
                                     consts [maxDegree] params [offsets (one per observable), coefficients] */
    GF_OP_RES_RBW           = 20, /* plainBW<1|2>          src/PDFs/physics/resonances/RBW.cu:9-86
                                     params [mass, width] consts [spin, cyclic index, norm, symmetric] */
    GF_OP_RES_NONRES        = 21, /* nonres                src/PDFs/physics/resonances/NonRes.cu:8-11
                                     amplitude 1 + 0i; no parameters */
    GF_OP_AMPLITUDE         = 15, /* Amplitude             src/PDFs/physics/Amplitude.cu:11-31, AmpCalc
                                     src/PDFs/physics/detail/AmpCalc.cu:14-59
                                     consts [nPerm, nLS, nSF] children [line shapes..., spin factors...] */
    GF_OP_LS_RBW            = 22, /* BW (ptr_to_BW_DP4)    src/PDFs/physics/lineshapes/BW.cu:14-68
                                     params [mass, width] consts [Mpair (DP4Pair), L, FF, radius] */
    GF_OP_LS_SBW            = 23, /* SBW                   src/PDFs/physics/lineshapes/BW.cu:70-110 (as GF_OP_LS_RBW) */
    GF_OP_SPINFACTOR        = 24  /* SpinFactor            src/PDFs/physics/SpinFactors.cu:83-568
                                     consts [SF_4Body kind, mD0, P0, P1, P2, P3] */
};

/* node flags */
#define GF_FLAG_COMMON_NORM   1 /* PdfBase::setCommonNorm   include/goofit/PdfBase.h:228 */
#define GF_FLAG_SEPARATE_NORM 2 /* PdfBase::setSeparateNorm include/goofit/PdfBase.h:229 */

/* One PdfBase object.  `params` index the engine parameter vector (one slot
 * per distinct Variable), `obs` index the observable columns, `children`
 * index this node list (children always come after their parent). */
typedef struct gf_node {
    int32_t op;
    int32_t flags;
    int32_t n_params;
    int32_t n_consts;
    int32_t n_obs;
    int32_t n_children;
    const int32_t *params;
    const double *consts;
    const int32_t *obs;
    const int32_t *children;
    int32_t integration_bins; /* PdfBase::setIntegrationFineness, 0 = observable bins */
    int32_t reserved;
} gf_node;

/* One Observable (include/goofit/Variable.h:109-140). */
typedef struct gf_observable {
    double lo;
    double hi;
    int32_t nbins;
    int32_t is_event_number;
} gf_observable;

/* What a per-event evaluation returns (include/goofit/FitControl.h:11). */
enum gf_metric { GF_METRIC_EVAL = 0, GF_METRIC_NLL = 1, GF_METRIC_PROB = 2 };

/* What the fit minimises (the FitControl classes, include/goofit/FitControl.h:40-76, and their metric functions
   src/PDFs/MetricPointer.cu:13-58).  The binned metrics take bins as events: the observable columns hold the bin
   centres, followed by two more columns, the bin content and the bin volume (GF_FIT_BINNED_ERROR: the bin
   error), as PdfBase::setData lays out a BinnedDataSet (src/PDFs/PdfBase.cu:439-495).  The expected number of
   events of a bin is c_totalEvents * P * norm * volume with c_totalEvents = the number of bins, as the
   reference sets it (src/PDFs/PdfBase.cu:527). */
enum gf_fit_metric {
    GF_FIT_UNBINNED_NLL = 0, /* UnbinnedNllFit: -sum log(P norm) */
    GF_FIT_BINNED_NLL   = 1, /* BinnedNllFit (BinAvg): sum (mu - n log mu), mu = T P norm V */
    GF_FIT_BINNED_ERROR = 2, /* BinnedErrorFit (BinWithError): sum ((P - n) / err)^2, P unnormalised */
    GF_FIT_BINNED_CHISQ = 3  /* BinnedChisqFit (Chisq): sum (T P norm V - n)^2 / max(n, 1) */
};


typedef struct gf_engine gf_engine;

/* ---- engine lifetime ---- */
int gf_engine_create(gf_engine **out, int device, int precision);
int gf_engine_destroy(gf_engine *eng);
const char *gf_last_error(const gf_engine *eng);
const char *gf_version(void);

/* ---- tree and data (PdfBase::setIndices / setData, src/PDFs/PdfBase.cu:313-438) ---- */
/* n_params: length of the parameter vector.  grad_mask[n_params] (may be NULL)
 * marks the parameters that get an analytic derivative. */
int gf_set_tree(gf_engine *eng,
                const gf_node *nodes,
                int n_nodes,
                const gf_observable *obs,
                int n_obs,
                int n_params,
                const int32_t *grad_mask);
/* Selects the fit metric (enum gf_fit_metric, default GF_FIT_UNBINNED_NLL).  A binned metric adds the two bin
   columns to the observables of the next gf_set_tree (call it before gf_set_tree). */
int gf_set_fit_metric(gf_engine *eng, int fit_metric);

/* Number of independent datasets ("toys"), each with its own parameter vector. */
int gf_set_num_toys(gf_engine *eng, int n_toys);

/* Events of one toy as SoA FP64 columns: soa[o * n_events + e] (replaces PdfBase::setData,
 * src/PDFs/PdfBase.cu:329-438).  Page-locked host memory is read in place by the conversion kernel; other
 * host memory is staged through a device buffer.  Returns when the device columns are ready;
 * GF_ERR_INVALID when an event lies outside a ConvolutionPdf's table range. */
int gf_upload_events(gf_engine *eng, int toy, const double *soa, int64_t n_events);

/* ---- evaluation: FCN::operator() + GooPdf::calculateNLL ---- */
int gf_set_params(gf_engine *eng, int toy, const double *params, int n_params);
/* Returns once the result is on the host. In the one-launch form the engine's kernel may still be ending on
 * the engine's stream at that point (its result rows are read as they arrive); later engine calls are ordered
 * after it, and gf_last_timing waits for it. */
int gf_nll(gf_engine *eng, int toy, double *nll);
/* grad has one entry per parameter whose grad_mask is set, in parameter order */
int gf_nll_grad(gf_engine *eng, int toy, double *nll, double *grad);
/* All toys in one launch sequence: P[n_toys][n_params] -> nll[n_toys], grad[n_toys][n_grad] (grad may be NULL).
 * active[n_toys] (may be NULL) skips toys whose entry is 0. */
int gf_nll_batch(gf_engine *eng, int n_toys, const double *P, const int32_t *active, double *nll, double *grad);
int gf_num_grad(const gf_engine *eng);
int gf_num_params(const gf_engine *eng);
int gf_num_toys(const gf_engine *eng);
/* Parameter index of every gradient slot: out[0..gf_num_grad-1]; returns the count. */
int gf_grad_params(const gf_engine *eng, int32_t *out, int cap);

/* Normalisation of every node (GooPdf::normalize, src/PDFs/GooPdf.cu:340-396):
 * integral[n] is the value normalize() returns, norm[n] the factor applied
 * (1/integral, or 1 for forced/combine nodes). */
int gf_normalize(gf_engine *eng, int toy, double *integral, double *norm);

/* Per-event values of node `node` treated as the root (GooPdf::evaluate_with_metric,
 * src/PDFs/GooPdf.cu:112-173): out[e] for the toy's events. */
int gf_eval_events(gf_engine *eng, int toy, int node, int metric, double *out, int64_t n_out);

/* Device time of the last evaluation's kernels in milliseconds (CUDA events). */
int gf_last_timing(const gf_engine *eng, double *ms_total, double *ms_event_kernel);
/* Device time of each kernel of one evaluation launched alone (no graph, no overlap), with CUDA events on
 * the engine's stream; a kernel a tree does not need reports 0.  toy = -1: every toy active. */
int gf_time_kernels(gf_engine *eng, int toy, int with_grad, double *ms_conv, double *ms_grid, double *ms_event);
/* Number of kernel launches issued by one gf_nll_grad / gf_nll_batch call. */
int gf_launches_per_eval(const gf_engine *eng, int with_grad);
/* Events per chunk of the event pass (chosen from the occupancy, then by the autotuner at the first
   evaluation of a layout unless GF_AUTOTUNE=0 or GF_CHUNK is set); 0 before the first evaluation. */
int64_t gf_event_chunk(const gf_engine *eng);
/* Longest wait, in nanoseconds of the GPU's global timer, at the grid barrier of the one-launch evaluation
 * (one toy: tables, grids and event pass in one cooperative launch); ns = 0 restores the default of 1 s.
 * A wait that runs out stops the launch, the call returns GF_ERR_TIMEOUT and the engine stays usable.
 * No counterpart in the reference (its Thrust reductions have no device-side waits). */
int gf_set_wait_limit(gf_engine *eng, uint64_t ns);
/* Longest wait, in nanoseconds of the GPU's global timer, of each pipeline-stage mbarrier wait of the mixed
 * engine's tensor-core Gram kernel (the normalisation integrals of Amp3Body / Amp4Body); ns = 0 restores the
 * default of 2 s.  The kernel's wait for its last committed MMAs before it frees its tensor memory always keeps
 * the 2 s limit.  A wait that runs out makes the integral rebuild return GF_ERR_CUDA; the engine stays usable
 * and rebuilds the integrals at the next evaluation.  No counterpart in the reference (its integrals are
 * Thrust reductions, src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:52-121, without device-side waits). */
int gf_set_gram_wait_limit(gf_engine *eng, uint64_t ns);

/* Where the derivatives of the amplitudes by floated resonance / line-shape parameters live (Amp3Body, Amp4Body).
   GF_AMP_STORE: per-event columns and per-normalisation-point scratch columns, as the reference caches its
   line shapes, spin factors and amplitudes (src/PDFs/physics/Amp4Body.cu:348-395).  GF_AMP_RECOMPUTE: only the
   amplitude values are cached per event; the gradient pass recomputes dA/dt per event, and the integrals are
   reduced from amplitudes recomputed at every normalisation point (no per-point storage).  GF_AMP_AUTO (the
   default) recomputes when storing would take more than budget_bytes (0: a quarter of the free device memory).
   Takes effect at the next gf_set_tree, or at the first gf_upload_events after it; GF_ERR_STATE once events
   are uploaded. */
enum gf_amp_mode { GF_AMP_AUTO = 0, GF_AMP_STORE = 1, GF_AMP_RECOMPUTE = 2 };
int gf_set_amp_mode(gf_engine *eng, int mode, int64_t budget_bytes);
/* 1: the engine recomputes amplitude derivatives, 0: it stores them (or the tree has none), -1: not decided yet
   (no events uploaded since gf_set_tree). */
int gf_amp_recomputing(const gf_engine *eng);
/* Device bytes the store mode keeps for the derivative columns of the uploaded events and the normalisation
   scratch columns (what the recompute mode does without); 0 without amplitude nodes or events. */
int64_t gf_amp_store_bytes(const gf_engine *eng);

/* Launch-shape autotuner (the counterpart of the reference's grain-size sweep, scripts/find_optimal.py): times
   one gradient evaluation of every toy (device time, L2 flushed) for each candidate and keeps the fastest.
   Candidates: the table kernel's k-tiles per staged model and resolution (1, 2, 4, 8; batches of toys with a
   convolution), the numeric-grid bins per CTA (128 ... 2048; grids not folded into a table), then the
   tensor-core Gram kernel's slice width (16, 32, 64 real columns; the integral rebuild timed).  Each table or
   grid candidate recompiles the tree.  Needs uploaded events; results are remembered for the process, keyed by
   tree, precision, toy count and events. */
int gf_tune_shapes(gf_engine *eng);
/* The shapes in use: table k-tiles, grid bins per CTA, Gram slice width (0: no tensor-core Gram). */
int gf_get_shapes(const gf_engine *eng, int32_t *conv_kp, int32_t *grid_bpb, int32_t *gram_w);

/* ---- minimiser (Minuit2 MnMigrad surface, src/goofit/FitManagerMinuit2.cpp:31-119) ---- */
typedef struct gf_minimizer gf_minimizer;

/* limited[i]: 0 none, 1 both bounds, 2 lower only, 3 upper only.  fixed[i] != 0 keeps x0[i].
 * use_grad != 0: the caller supplies gradients (FCNGradientBase); else numerical (2-point, strategy cycles). */
/* fnoise_rel: see gf_fit_options */
int gf_minimizer_create(gf_minimizer **out,
                        int n,
                        const double *x0,
                        const double *err,
                        const double *lo,
                        const double *hi,
                        const int32_t *limited,
                        const int32_t *fixed,
                        double up,
                        int strategy,
                        double tolerance,
                        int maxfcn,
                        int use_grad,
                        double fnoise_rel);
/* Returns 1 and fills x[n] (external values) when a function value is needed;
 * *need_grad says whether the gradient is wanted too.  Returns 0 when finished. */
int gf_minimizer_ask(gf_minimizer *m, double *x, int32_t *need_grad);
/* grad[n] over all parameters (entries of fixed ones are ignored); NULL if not asked. */
int gf_minimizer_tell(gf_minimizer *m, double f, const double *grad);

typedef struct gf_fit_result {
    double fmin;
    double edm;
    int32_t nfcn;
    int32_t ngrad;
    int32_t valid;          /* IsValid && HasCovariance && !IsAboveMaxEdm && !HasReachedCallLimit */
    int32_t above_max_edm;
    int32_t call_limit;
    int32_t has_covariance;
    int32_t hesse_failed;
    int32_t made_posdef;
    int32_t n_iter;
    int32_t reserved;
} gf_fit_result;

/* x[n], err[n] external; cov[n*n] external covariance (may be NULL). */
int gf_minimizer_result(const gf_minimizer *m, gf_fit_result *res, double *x, double *err, double *cov);
int gf_minimizer_destroy(gf_minimizer *m);

/* ---- native fit loop: MIGRAD against the engine without leaving C++ ---- */
typedef struct gf_fit_options {
    const double *err;       /* [n_params] initial step / error */
    const double *lo;        /* [n_params] */
    const double *hi;        /* [n_params] */
    const int32_t *limited;  /* [n_params] */
    const int32_t *fixed;    /* [n_params] */
    double up;               /* 0.5 for NLL (include/goofit/fitting/FCN.h:26) */
    double tolerance;        /* MnMigrad tolerance, EDM < 0.002 * tolerance * up */
    int32_t strategy;        /* MnStrategy(1) by default */
    int32_t maxfcn;
    int32_t use_grad;        /* analytic gradient from the adjoint path */
    int32_t reserved;
    double fnoise_rel;       /* relative rounding noise of the NLL (0: exact FP64 sums); the line search
                                treats value changes below fnoise_rel * |NLL| as ties and follows the gradient */
    double *cov;             /* optional out: [n_toys][n_params][n_params] external covariance of the final
                                Hesse (Minuit2's FunctionMinimum::UserCovariance); NULL: not returned */
} gf_fit_options;

/* Fits toy `toy` starting from x0[n_params]; x/err receive the result. */
int gf_fit(gf_engine *eng, int toy, const gf_fit_options *opt, const double *x0, double *x, double *err,
           gf_fit_result *res);
/* Fits toys 0..n_toys-1 in lockstep (one batched launch sequence per round).
 * X0/X/ERR are [n_toys][n_params]; res[n_toys]. */
int gf_fit_batch(gf_engine *eng, int n_toys, const gf_fit_options *opt, const double *X0, double *X, double *ERR,
                 gf_fit_result *res);

/* ---- NLL without device allocation ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they evaluate the likelihood (a host whose device memory is owned
 * by another allocator or a fixed budget; latency-critical code where
 * cudaMalloc/cudaFree may synchronise the device).  Computes, on `stream`
 * (a cudaStream_t, NULL = default stream), the NLL of ExpPdf(x; alpha) with its
 * analytic normalisation over [lo, hi] for n_events FP32 values x (device
 * memory), writing out[0] = NLL and out[1] = dNLL/dalpha (device memory, two
 * doubles).  Allocates nothing: its reduction scratch is a fixed device array
 * inside the library (24 KB per device, kept until exit) that limits a call to
 * 8,388,608 events; larger counts return GF_ERR_INVALID, and so does an alpha
 * whose normalisation integral is not finite and positive.  The first call on a
 * device looks up that array's device address (make that first call before any
 * stream capture).  All calls share the array, so calls that overlap on the
 * GPU (other streams, other host threads) race: order them on one stream.
 * Asynchronous: errors that only the device can see (NaN events) show in out[].
 * gf_noalloc_last_error() describes the last failure of this entry point. */
int gf_nll_exp_noalloc(const float *x, int64_t n_events, double alpha, double lo, double hi, double *out,
                       void *stream);
const char *gf_noalloc_last_error(void);

/* Normalisation integrals of an amplitude node at the toy's current parameters, n x n complex interleaved
   [re, im] row-major; `cap` counts doubles (>= 2 n^2).  Amp3Body: I_ij = sum over in-Dalitz bins of
   B_i conj(B_j) eff, before the bin size factor (the integrals Amp3Body::normalize caches,
   src/PDFs/physics/Amp3Body.cu:304-330).  Amp4Body: G_ab = sum over the normalisation events of
   A_a conj(A_b), before the 1/N (NormIntegrator's sum, src/PDFs/physics/detail/NormIntegrator.cu:15-68,
   taken apart by amplitude pairs). */
int gf_amp3_integrals(gf_engine *eng, int toy, int node, double *out, int cap);

/* Cached amplitude of resonance / amplitude `res` of an Amp3Body or Amp4Body node for every event of the toy,
   complex interleaved (2 n doubles; FP32 values widened in GF_MIXED): Amp3Body::getCachedWave
   (include/goofit/PDFs/physics/Amp3Body.h:61) and Amp4Body's cachedAMPs (src/PDFs/physics/Amp4Body.cu:381-386). */
int gf_amp3_cached_wave(gf_engine *eng, int toy, int node, int res, double *out, int64_t n_out);

/* Flat phase-space normalisation events of an Amp4Body node, SoA [m12 | m34 | cos12 | cos34 | phi], n each
   (copied).  Replaces the MCBooster generation inside the Amp4Body constructor
   (src/PDFs/physics/Amp4Body.cu:243-290); call after gf_set_tree, before evaluating. */
int gf_set_norm_events(gf_engine *eng, int node, const double *soa5, int64_t n);

/* ---- diagnostics: code generation without a device ---- */
/* Generated CUDA source for a tree (precision as in gf_engine_create); *len gets the full length. */
int gf_generated_source(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                        const int32_t *grad_mask, int precision, char *buf, int64_t cap, int64_t *len);
/* Compiles a tree's kernels for sm_103a without loading them; *cubin_bytes gets the image size. */
int gf_compile_tree(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                    const int32_t *grad_mask, int precision, int64_t *cubin_bytes);
/* The same for the kernel shapes an engine uses with more than one toy (gf_set_num_toys > 1). */
int gf_compile_tree_batch(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                          const int32_t *grad_mask, int precision, int64_t *cubin_bytes);

#ifdef __cplusplus
}
#endif

#endif /* GFENGINE_H */
