// An NLL entry point that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the moment they evaluate
// the likelihood.  Examples are hosts whose whole device memory is owned by
// another allocator (a framework's caching allocator, or a service that runs
// under a fixed memory budget and hands out pre-sized buffers only), and code
// on latency-critical paths, where cudaMalloc / cudaFree may synchronise the
// device.  The regular engine (gf_engine_create + gf_nll_grad) allocates its
// buffers when a tree and data are set; this entry point instead takes the
// caller's device buffers and keeps its own reduction scratch in a fixed,
// file-scope device array.
//
// What it computes: the NLL of one ExpPdf over an FP32 event column with its
// analytic normalisation over [lo, hi], and the derivative with respect to
// alpha.  The arithmetic is its own, simpler than the generated event kernels':
// per event FP32 (v = exp(a x) with a = alpha rounded to FP32, the term -log v
// and its alpha derivative -x), plain FP32 sums of each thread's 32 events, FP64
// across warps and CTAs.  Events with v = 0 (underflow) contribute nothing, as
// in the reference's NLL metric (terms with P <= 0 are skipped); NaN events
// reach the sums.  The normalisation N = 1/I is computed in FP64 at the same
// rounded a and applied once, in FP64, by the finishing CTA: count * (-log N)
// for the NLL and count * dI/I for the derivative, count being the number of
// events that contributed.  A single FP32 factor per event would move the NLL in
// steps of up to n * 2^-24 as alpha varies.
#include "../../include/gfengine.h"

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

namespace {

constexpr int kThreads       = 256;
constexpr int kChunk         = 8192;                   // events per CTA
constexpr int kMaxBlocks     = 1024;                   // CTAs whose partial sums fit in the scratch
constexpr long long kMaxEvts = (long long)kChunk * kMaxBlocks; // 8,388,608 events per call

struct NoAllocScratch {
    double partial[kMaxBlocks][3]; // per-CTA sums of -log v, -x and the count of contributing events
    unsigned int done;             // CTAs finished in the current call
};

// One copy per device that loads this library, held until the process exits.
// Every call of gf_nll_exp_noalloc on a device uses this same array.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_mu;
NoAllocScratch *g_scratch_addr[128] = {nullptr}; // device address of the array, per device ordinal
thread_local std::string g_err;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads)
    gf_exp_nll_noalloc_kernel(const float *__restrict__ x, long long n, float a, double logN, double dIoverI,
                              NoAllocScratch *scr, double *out) {
    __shared__ double red[kThreads / 32][3];
    __shared__ int last;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const long long b0 = (long long)blockIdx.x * kChunk;
    const long long e0 = b0 + kChunk < n ? b0 + kChunk : n;
    float av = 0.f, ag = 0.f;
    int cnt = 0;
    for(long long i = b0 + tid; i < e0; i += kThreads) {
        const float xv = x[i];
        const float v  = expf(a * xv);
        if(!(v <= 0.f)) { // v = 0 is skipped like a P <= 0 term; NaN passes into the sums
            av -= logf(v);
            ag -= xv;
            ++cnt;
        }
    }
    double t0 = warp_sum((double)av), t1 = warp_sum((double)ag), t2 = warp_sum((double)cnt);
    if(lane == 0) {
        red[wid][0] = t0;
        red[wid][1] = t1;
        red[wid][2] = t2;
    }
    __syncthreads();
    if(tid < 3) {
        double s = 0;
        for(int w = 0; w < kThreads / 32; ++w)
            s += red[w][tid];
        scr->partial[blockIdx.x][tid] = s;
    }
    __threadfence();
    __syncthreads();
    if(tid == 0)
        last = atomicAdd(&scr->done, 1u) == gridDim.x - 1;
    __syncthreads();
    if(last && tid == 0) {
        __threadfence();
        double s0 = 0, s1 = 0, c = 0;
        for(unsigned int b = 0; b < gridDim.x; ++b) {
            s0 += scr->partial[b][0];
            s1 += scr->partial[b][1];
            c += scr->partial[b][2];
        }
        // -log(v N) summed = -sum log v - count log N;  d/dalpha: -x - N'/N = -x + I'/I
        out[0]    = s0 - c * logN;
        out[1]    = s1 + c * dIoverI;
        scr->done = 0u;
    }
}

// ExpPdf::integrate over [lo, hi] at alpha, I = (e^{alpha hi} - e^{alpha lo}) / alpha, and dI/dalpha,
// written with expm1 so that small |alpha| loses no precision: with w = hi - lo and u = alpha w,
// I = e^{alpha lo} w g(u), g(u) = expm1(u) / u, and dI/dalpha = lo I + e^{alpha lo} w^2 g'(u),
// g'(u) = (expm1(u) (u - 1) + u) / u^2 (its Taylor series 1/2 + u/3 + u^2/8 + u^3/30 + u^4/144 below
// |u| = 1e-2, where the closed form cancels).
void expIntegral(double alpha, double lo, double hi, double *I, double *dI) {
    const double w = hi - lo, u = alpha * w, el = std::exp(alpha * lo);
    double g, gp;
    if(std::fabs(u) < 1e-2) {
        g  = 1.0 + u * (1.0 / 2 + u * (1.0 / 6 + u * (1.0 / 24 + u * (1.0 / 120 + u / 720))));
        gp = 1.0 / 2 + u * (1.0 / 3 + u * (1.0 / 8 + u * (1.0 / 30 + u / 144)));
    } else {
        const double em = std::expm1(u);
        g  = em / u;
        gp = (em * (u - 1.0) + u) / (u * u);
    }
    *I  = el * w * g;
    *dI = lo * (*I) + el * w * w * gp;
}

// Device address of the scratch array for the current device, resolved once per device.
int scratchForCurrentDevice(NoAllocScratch **p) {
    int dev = 0;
    cudaError_t r = cudaGetDevice(&dev);
    if(r != cudaSuccess) {
        g_err = std::string("cudaGetDevice: ") + cudaGetErrorString(r);
        return GF_ERR_CUDA;
    }
    if(dev < 0 || dev >= 128) {
        g_err = "device ordinal beyond 127";
        return GF_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if(!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        r         = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if(r != cudaSuccess || !ptr) {
            g_err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(r);
            return GF_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<NoAllocScratch *>(ptr);
    }
    *p = g_scratch_addr[dev];
    return GF_OK;
}

} // namespace

extern "C" {

int gf_nll_exp_noalloc(const float *x, int64_t n_events, double alpha, double lo, double hi, double *out,
                       void *stream) {
    if(!out || (n_events > 0 && !x)) {
        g_err = "gf_nll_exp_noalloc: null device pointer";
        return GF_ERR_INVALID;
    }
    if(n_events < 1 || n_events > kMaxEvts) {
        g_err = "gf_nll_exp_noalloc: n_events must be in 1.." + std::to_string(kMaxEvts) +
                " (the scratch array holds partial sums for " + std::to_string(kMaxBlocks) + " blocks of " +
                std::to_string(kChunk) + " events)";
        return GF_ERR_INVALID;
    }
    if(!(hi > lo) || !std::isfinite(lo) || !std::isfinite(hi)) {
        g_err = "gf_nll_exp_noalloc: need finite lo < hi";
        return GF_ERR_INVALID;
    }
    // the kernel evaluates exp(a x) at a = alpha rounded to FP32; the normalisation uses the same a
    const float a = (float)alpha;
    double I = 0, dI = 0;
    if(std::isfinite(alpha) && std::isfinite(a))
        expIntegral((double)a, lo, hi, &I, &dI);
    if(!(std::isfinite(I) && I > 0 && std::isfinite(dI))) {
        g_err = "gf_nll_exp_noalloc: alpha must give a finite, positive normalisation integral (alpha = " +
                std::to_string(alpha) + ")";
        return GF_ERR_INVALID;
    }
    NoAllocScratch *scr = nullptr;
    int rc              = scratchForCurrentDevice(&scr);
    if(rc)
        return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the completion counter must start at zero; the partial sums are overwritten by every call
    cudaError_t r = cudaMemsetAsync(&scr->done, 0, sizeof(unsigned int), s);
    if(r == cudaSuccess) {
        const unsigned blocks = (unsigned)((n_events + kChunk - 1) / kChunk);
        gf_exp_nll_noalloc_kernel<<<blocks, kThreads, 0, s>>>(x, (long long)n_events, a, -std::log(I), dI / I,
                                                                 scr, out);
        r = cudaGetLastError();
    }
    if(r != cudaSuccess) {
        g_err = std::string("gf_nll_exp_noalloc: ") + cudaGetErrorString(r);
        return GF_ERR_CUDA;
    }
    return GF_OK;
}

const char *gf_noalloc_last_error(void) { return g_err.c_str(); }

} // extern "C"
