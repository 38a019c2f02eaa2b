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
// analytic normalisation, and the derivative with respect to alpha; the same
// per-event arithmetic and chunked reduction as the event kernel the engine
// generates for that tree (mixed precision: FP32 per event, FP64 partials).
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
    double partial[kMaxBlocks][2]; // per-CTA (NLL, dNLL/dalpha) partial sums
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
    gf_exp_nll_noalloc_kernel(const float *__restrict__ x, long long n, double alpha, double lo, double hi,
                              NoAllocScratch *scr, double *out) {
    __shared__ double red[kThreads / 32][2];
    __shared__ int last;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // analytic normalisation of ExpPdf over [lo, hi] (ExpPdf::integrate) and its alpha derivative
    double I, dI;
    if(alpha == 0) {
        I  = hi - lo;
        dI = 0.5 * (hi * hi - lo * lo);
    } else {
        const double eh = exp(alpha * hi), el = exp(alpha * lo);
        I  = (eh - el) / alpha;
        dI = (hi * eh - lo * el) / alpha - I / alpha;
    }
    const double Nd = 1.0 / I;
    const float N   = (float)Nd;
    const float dN  = (float)(-Nd * Nd * dI);
    const float a   = (float)alpha;
    const long long b0 = (long long)blockIdx.x * kChunk;
    const long long e0 = b0 + kChunk < n ? b0 + kChunk : n;
    float av = 0.f, ag = 0.f;
    for(long long i = b0 + tid; i < e0; i += kThreads) {
        const float xv = x[i];
        const float v  = expf(a * xv);
        const float pv = v * N;
        if(pv > 0.f) {
            av -= logf(pv);
            ag -= (xv * v * N + v * dN) / pv;
        }
    }
    double t0 = warp_sum((double)av), t1 = warp_sum((double)ag);
    if(lane == 0) {
        red[wid][0] = t0;
        red[wid][1] = t1;
    }
    __syncthreads();
    if(tid < 2) {
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
    if(last && tid < 2) {
        __threadfence();
        double s = 0;
        for(unsigned int b = 0; b < gridDim.x; ++b)
            s += scr->partial[b][tid];
        out[tid] = s;
        if(tid == 0)
            scr->done = 0u;
    }
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
    if(!(hi > lo)) {
        g_err = "gf_nll_exp_noalloc: need lo < hi";
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
        gf_exp_nll_noalloc_kernel<<<blocks, kThreads, 0, s>>>(x, (long long)n_events, alpha, lo, hi, scr, out);
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
