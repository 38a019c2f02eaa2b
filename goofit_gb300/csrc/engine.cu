// Likelihood engine runtime: the C ABI of include/gfengine.h.
//
// Replaces the reference's process-global device state (d_parameters,
// d_constants, d_observables, d_normalizations, d_function_table,
// dev_event_array: src/PDFs/detail/Globals.cu:9-26, src/goofit/Globals.cpp:11)
// with per-handle buffers: per-toy SoA event columns in HBM, a pinned
// parameter/result exchange area, and one captured CUDA graph per
// evaluation kind that runs   H2D(params) -> conv tables -> grid sums ->
// event pass -> D2H(result)   in a single graph launch.
#include "engine.h"
#include "rtc.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <complex>
#include <cstring>
#include <new>

namespace {

thread_local std::string g_create_err;

struct ConvertArgs {
    const double *soa;
    long long n, npad;
    int n_obs, n_conv;
    void *cols[16];
    int *kcols[8];
    int conv_obs[8];
    double conv_lo[8], conv_step[8], conv_lbo[8];
    float conv_inv_step[8], conv_lbo_f[8];
    int conv_kmin[8], conv_kmax[8];
    double pad_val[16];
    int *err;
};

// FP64 SoA -> engine columns (FP32 or FP64) plus the ConvolutionPdf bin
// offset of every event (src/PDFs/combine/ConvolutionPdf.cu:40-43, FP64),
// which is all the convolution needs of x: one event (or padding slot) i.
template <typename R>
__device__ __forceinline__ void gf_convert_one(const ConvertArgs &a, long long i) {
    // every value is read once (the source may be page-locked host memory read over the interconnect),
    // all loads issued before the first store
    double xs[16];
#pragma unroll
    for(int o = 0; o < 16; ++o)
        if(o < a.n_obs)
            xs[o] = i < a.n ? a.soa[(long long)o * a.n + i] : a.pad_val[o];
#pragma unroll
    for(int o = 0; o < 16; ++o)
        if(o < a.n_obs)
            reinterpret_cast<R *>(a.cols[o])[i] = (R)xs[o];
    for(int c = 0; c < a.n_conv; ++c) {
        int k;
        if(i < a.n) {
            double x0 = 0.0;
#pragma unroll
            for(int o = 0; o < 16; ++o)
                if(o == a.conv_obs[c])
                    x0 = xs[o];
            // FP32 estimate of x0/step - frac(lo/step); its error is below 3e-7 (|q| + 1), so away from
            // a bin edge its floor is the FP64 result, and near an edge the FP64 division decides
            const float qf = fmaf((float)x0, a.conv_inv_step[c], -a.conv_lbo_f[c]);
            const float kf = floorf(qf);
            const float d  = qf - kf;
            const float th = 4e-7f * (fabsf(qf) + 1.0f);
            if(d > th && d < 1.0f - th)
                k = (int)kf;
            else
                k = (int)floor(x0 / a.conv_step[c] - a.conv_lbo[c]);
            if(k < a.conv_kmin[c] || k > a.conv_kmax[c]) {
                *a.err = 1; // page-locked host flag: every writer stores the same value
                k = a.conv_kmin[c];
            }
        } else
            k = a.conv_kmin[c];
        a.kcols[c][i] = k;
    }
}

// One thread per event or padding slot.
template <typename R>
__global__ void gf_convert_events(const ConvertArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if(i < a.npad)
        gf_convert_one<R>(a, i);
}

size_t rsize(const gf_engine *e) { return e->precision == GF_MIXED ? 4 : 8; }

// Counting sort of one toy's convolution bin offsets (the one-launch tabulated path, where an event's terms
// depend on the event only through its bin offset, so the order in which the events are summed is free):
// the histogram of the offsets, then every sorted position takes the bin whose prefix range holds it.  With the
// events in bin order every warp's gathers from the per-bin term table hit one or two rows (shared-memory
// broadcasts instead of bank conflicts), and each CTA's events span a few bins only.
__global__ void __launch_bounds__(1024) gf_khist(const int *__restrict__ k, long long n, int kmin, int nK, unsigned *__restrict__ hist) {
    extern __shared__ unsigned sh[];
    const bool local = nK <= 8192;
    if(local)
        for(int i = threadIdx.x; i < nK; i += blockDim.x)
            sh[i] = 0;
    __syncthreads();
    for(long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int b = k[e] - kmin;
        if(b >= 0 && b < nK)
            atomicAdd(local ? &sh[b] : &hist[b], 1u);
    }
    __syncthreads();
    if(local)
        for(int i = threadIdx.x; i < nK; i += blockDim.x)
            if(sh[i])
                atomicAdd(&hist[i], sh[i]);
}

// Block b writes bin b's run of the sorted column (coalesced stores, no search). The run starts at the sum of
// the counts of the bins below b, which each block reduces itself from the histogram in L2 (no separate scan
// launch: 2e6 offsets, 1501 bins, scan + fill 9.8 us before). The last block also fills the padding from n up
// to npad with the first bin; the counts add up to n (the conversion clamps offsets into the table), and the
// stores are bounded by npad all the same.
__global__ void __launch_bounds__(256) gf_kfill(const unsigned *__restrict__ hist, int nK, int kmin, long long n,
                                                long long npad, int *__restrict__ out) {
    __shared__ long long part[8];
    const int b = blockIdx.x, tid = threadIdx.x;
    long long s = 0;
    for(int i = tid; i < b; i += 256)
        s += hist[i];
    for(int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if((tid & 31) == 0)
        part[tid >> 5] = s;
    __syncthreads();
    long long start = 0;
    for(int w = 0; w < 8; ++w)
        start += part[w];
    const long long end = min(start + (long long)hist[b], npad);
    for(long long i = start + tid; i < end; i += 256)
        out[i] = kmin + b;
    if(b == nK - 1)
        for(long long i = n + tid; i < npad; i += 256)
            out[i] = kmin;
}

// The sort's histogram of toy 0, allocated on first use and kept across uploads.
cudaError_t ensureKHist(GfToy &ty, int nK) {
    if(ty.khist_n >= nK)
        return cudaSuccess;
    if(ty.khist)
        cudaFree(ty.khist);
    ty.khist      = nullptr;
    ty.khist_n    = 0;
    cudaError_t r = cudaMalloc((void **)&ty.khist, sizeof(unsigned) * nK);
    if(r == cudaSuccess)
        ty.khist_n = nK;
    return r;
}

// Sorted copy of toy 0's offsets of convolution 0: histogram and fill, all on the device and
// asynchronous on the engine's stream (the upload's own range check has already rejected offsets outside the
// table); the sorted column is allocated on first use and kept across uploads of the same size. (The histogram
// built inside the conversion kernel instead, with warp-aggregated atomics and a last-CTA scan, made the 2e6-event
// upload 2.5x slower.)
int buildKSort(gf_engine *e) {
    GfToy &ty = e->toys[0];
    if(!ty.loaded || e->tree.convs.empty())
        return GF_OK;
    const gf::ConvInfo &cv = e->tree.convs[0];
    const int nK           = cv.nK;
    cudaError_t r          = cudaSuccess;
    if(!ty.ksort)
        r = cudaMalloc((void **)&ty.ksort, sizeof(int) * (size_t)std::max<int64_t>(8, ty.npad));
    if(r == cudaSuccess)
        r = ensureKHist(ty, nK);
    // one CTA of 1024 threads per SM: half the CTAs of 2 x 256 per SM, so half the global additions of per-CTA
    // counts onto the same bins (2e6 offsets: 6.8 us against 10.1 us; 152 x 512: 8.8 us, 76 x 1024: 9.2 us)
    const int grid = std::max(1, e->sm_count);
    if(r == cudaSuccess)
        r = cudaMemsetAsync(ty.khist, 0, sizeof(unsigned) * nK, e->stream);
    if(r == cudaSuccess) {
        gf_khist<<<grid, 1024, nK <= 8192 ? sizeof(unsigned) * nK : 0, e->stream>>>(ty.kcols[0], ty.n, cv.kmin, nK, ty.khist);
        gf_kfill<<<nK, 256, 0, e->stream>>>(ty.khist, nK, cv.kmin, ty.n, ty.npad, ty.ksort);
        r = cudaGetLastError();
    }
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "sorting the bin offsets");
    ty.ksort_valid = true;
    return GF_OK;
}

void freeToy(GfToy &t) {
    for(int o = 0; o < 16; ++o)
        if(t.cols[o]) {
            if(o == 0)
                cudaFree(t.cols[0]);
            t.cols[o] = nullptr;
        }
    for(int c = 0; c < 8; ++c)
        t.kcols[c] = nullptr;
    if(t.ksort)
        cudaFree(t.ksort);
    if(t.khist)
        cudaFree(t.khist);
    t.ksort       = nullptr;
    t.khist       = nullptr;
    t.khist_n     = 0;
    t.ksort_valid = false;
    if(t.abase)
        cudaFree(t.abase);
    t.abase = nullptr;
    for(auto &p : t.acols)
        p = nullptr;
    for(auto &p : t.dcols)
        p = nullptr;
    t.loaded     = false;
    t.amp_valid  = false;
    t.norm_valid = false;
    t.amp_I.clear();
    t.n = t.npad = 0;
}

template <typename T>
void dfree(T *&p) {
    if(p)
        cudaFree((void *)p);
    p = nullptr;
}
template <typename T>
void hfree(T *&p) {
    if(p)
        cudaFreeHost((void *)p);
    p = nullptr;
}

void dropGraphs(gf_engine *e) {
    for(auto &g : e->graph)
        if(g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    for(int i = 0; i < 2; ++i) {
        if(e->graph_src[i])
            cudaGraphDestroy(e->graph_src[i]);
        e->graph_src[i]  = nullptr;
        e->fused_node[i] = nullptr;
    }
}

void freeLayout(gf_engine *e) {
    dropGraphs(e);
    dfree(e->d_P);
    e->d_active = nullptr; // inside d_P
    dfree(e->d_cols);
    dfree(e->d_kcols);
    dfree(e->d_ctab);
    dfree(e->d_kgrid);
    dfree(e->d_gsum);
    dfree(e->d_gpartial);
    dfree(e->d_gcounter);
    dfree(e->d_partial);
    dfree(e->d_counter);
    dfree(e->d_gbar);
    hfree(e->h_fpart);
    e->d_fpart   = nullptr;
    e->chunk_cap = 0;
    e->d_out = nullptr; // inside h_out
    dfree(e->d_chunks);
    e->chunk_cap = 0;
    dfree(e->d_toy_chunk0);
    dfree(e->d_toy_nchunks);
    dfree(e->d_toy_nevents);
    dfree(e->d_Nq);
    dfree(e->d_qflag);
    dfree(e->d_acols);
    dfree(e->d_dcols);
    dfree(e->d_dgrid);
    dfree(e->d_gram);
    dfree(e->d_gtc_part);
    dfree(e->d_gtc_out);
    dfree(e->d_gtc_err);
    e->gtc_part_n = e->gtc_out_n = 0;
    dfree(e->d_dirty);
    hfree(e->h_gram);
    hfree(e->h_dirty);
    hfree(e->h_P);
    e->h_active = nullptr; // inside h_P
    hfree(e->h_out);
    e->layout_ready = false;
}

void freeNormEvents(gf_engine *e) {
    for(auto &p : e->nscr)
        if(p)
            cudaFree(p);
    e->nscr.clear();
    e->nscr_bytes.clear();
    dfree(e->d_nscr);
    for(auto &b : e->norm_buf)
        dfree(b);
    e->norm_buf.clear();
    e->norm_n.clear();
    dfree(e->d_nevt);
    dfree(e->d_nnorm);
}

void freeModule(gf_engine *e) {
    if(e->mod.lib)
        cudaLibraryUnload(e->mod.lib);
    e->mod = GfModule();
}

template <typename T>
int dalloc(gf_engine *e, T *&p, size_t count, bool zero = true) {
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t r = cudaMalloc((void **)&p, bytes);
    if(r != cudaSuccess)
        return gf_fail(e, GF_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(r));
    if(zero)
        cudaMemset((void *)p, 0, bytes);
    return GF_OK;
}

// complex scratch columns of amplitude node k: its amplitudes, then one derivative column per (theta, amplitude)
int ampColumns(const gf::Tree &T, int k) {
    int nd = 0;
    for(auto &th : T.amp_theta(k))
        nd += (int)th.amps.size();
    return T.amp_count(k) + nd;
}

// Chunk tables for event chunks of `chunk` events (a chunk never spans two toys): the chunk list, each toy's
// first chunk and chunk count, and the chunk partials, grown when needed.  Captured graphs are dropped.
int setChunks(gf_engine *e, int chunk) {
    const int NT = e->n_toys, NGp = 1 + e->tree.NG;
    std::vector<long long> chunks;
    std::vector<int> c0(NT), nc(NT);
    for(int t = 0; t < NT; ++t) {
        const int64_t n = e->toys[t].n;
        const int k     = (int)std::max<int64_t>(1, (n + chunk - 1) / chunk);
        c0[t]           = (int)(chunks.size() / 3);
        nc[t]           = k;
        for(int c = 0; c < k; ++c) {
            chunks.push_back(t);
            chunks.push_back((long long)c * chunk);
            chunks.push_back(std::min<long long>((long long)(c + 1) * chunk, n));
        }
    }
    const int n = (int)(chunks.size() / 3);
    int rc      = GF_OK;
    if(n > e->chunk_cap) {
        dfree(e->d_chunks);
        dfree(e->d_partial);
        hfree(e->h_fpart);
        e->d_fpart   = nullptr;
        e->chunk_cap = 0;
        if((rc = dalloc(e, e->d_chunks, (size_t)3 * n, false)) || (rc = dalloc(e, e->d_partial, (size_t)n * (NGp + 1), false)))
            return rc;
        // rows of the one-launch kernel: [value, gradient..., count, status] per chunk, written by the kernel
        // into mapped page-locked memory and added up on the host
        e->fused_row = NGp + 2;
        if(cudaHostAlloc((void **)&e->h_fpart, sizeof(double) * (size_t)n * e->fused_row, cudaHostAllocMapped) !=
               cudaSuccess ||
           cudaHostGetDevicePointer((void **)&e->d_fpart, e->h_fpart, 0) != cudaSuccess) {
            cudaGetLastError();
            return gf_fail(e, GF_ERR_OOM, "cudaHostAlloc chunk rows");
        }
        e->chunk_cap = n;
    }
    cudaError_t r = cudaMemcpy(e->d_chunks, chunks.data(), sizeof(long long) * chunks.size(), cudaMemcpyHostToDevice);
    if(r == cudaSuccess)
        r = cudaMemcpy(e->d_toy_chunk0, c0.data(), sizeof(int) * NT, cudaMemcpyHostToDevice);
    if(r == cudaSuccess)
        r = cudaMemcpy(e->d_toy_nchunks, nc.data(), sizeof(int) * NT, cudaMemcpyHostToDevice);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "chunk tables");
    e->chunk    = chunk;
    e->n_chunks = n;
    dropGraphs(e);
    return GF_OK;
}

bool autotuneEnabled() {
    const char *v = std::getenv("GF_AUTOTUNE");
    return !(v && v[0] == '0');
}

int buildLayout(gf_engine *e) {
    if(e->layout_ready)
        return GF_OK;
    freeLayout(e);
    const gf::Tree &T = e->tree;
    const int NT = e->n_toys, NO = (int)T.obs.size(), NC = (int)T.convs.size(), NQ = (int)T.nums.size();
    const int NGp = 1 + T.NG;
    for(int t = 0; t < NT; ++t)
        if(!e->toys[t].loaded)
            return gf_fail(e, GF_ERR_STATE, "toy " + std::to_string(t) + " has no events");
    // chunk size: one chunk per resident event CTA (SMs x the event kernel's occupancy), so that a single
    // wave covers every SM with equal work; a multiple of 256 events (a warp's pass at 8 events per thread)
    if(!e->chunk_fixed) {
        int64_t total = 0;
        for(int t = 0; t < NT; ++t)
            total += e->toys[t].n;
        const int64_t target = (int64_t)std::max(1, e->sm_count) * e->evt_ctas_per_sm;
        int64_t ch           = (total + target - 1) / target;
        ch                   = (ch + 255) / 256 * 256;
        e->chunk             = (int)std::min<int64_t>(std::max<int64_t>(ch, 256), 1 << 20);
    }
    // the first evaluation times the event kernel at a few chunk sizes around this one and keeps the best
    e->tune_pending = !e->chunk_fixed && autotuneEnabled();
    std::vector<long long> ne(NT);
    for(int t = 0; t < NT; ++t)
        ne[t] = e->toys[t].n;
    int rc      = GF_OK;
    auto chk    = [&](int r) {
        if(r != GF_OK && rc == GF_OK)
            rc = r;
    };
    const gf::NormLayout &nl = e->plan.nl;
    // one host-to-device block per evaluation: [toy][param] FP64, [toy][record] R, then the active flags
    e->pblock_bytes = sizeof(double) * (size_t)NT * std::max(1, T.n_params) + rsize(e) * (size_t)NT * std::max(1, nl.npr);
    e->pblock_bytes = (e->pblock_bytes + 15) / 16 * 16;
    e->active_off   = e->pblock_bytes;
    e->pblock_bytes = (e->pblock_bytes + sizeof(int) * (size_t)NT + 15) / 16 * 16;
    chk(dalloc(e, e->d_P, e->pblock_bytes / sizeof(double)));
    {
        void *p = nullptr;
        if(cudaMalloc(&p, rsize(e) * (size_t)NT * std::max(1, nl.nq)) != cudaSuccess)
            chk(gf_fail(e, GF_ERR_OOM, "cudaMalloc numeric factors"));
        e->d_Nq = p;
    }
    chk(dalloc(e, e->d_qflag, NT));
    e->d_active = reinterpret_cast<int *>(reinterpret_cast<char *>(e->d_P) + e->active_off);
    chk(dalloc(e, e->d_cols, (size_t)NT * NO));
    chk(dalloc(e, e->d_kcols, (size_t)NT * std::max(1, NC)));
    int64_t ctab = std::max(e->plan.ctab_per_toy_grad, e->plan.ctab_per_toy_nograd);
    {
        void *p = nullptr;
        size_t bytes = (size_t)std::max<int64_t>(1, NT * ctab) * rsize(e);
        if(cudaMalloc(&p, bytes) != cudaSuccess)
            chk(gf_fail(e, GF_ERR_OOM, "cudaMalloc conv tables"));
        else
            cudaMemset(p, 0, bytes);
        e->d_ctab = p;
    }
    chk(dalloc(e, e->d_kgrid, std::max<size_t>(1, T.kgrid.size())));
    chk(dalloc(e, e->d_gsum, (size_t)NT * std::max(1, NQ)));
    chk(dalloc(e, e->d_gpartial, (size_t)NT * std::max(1, NQ) * std::max(1, e->plan.max_grid_blocks) * NGp));
    chk(dalloc(e, e->d_gcounter, (size_t)NT * std::max(1, NQ)));
    chk(dalloc(e, e->d_counter, NT));
    chk(dalloc(e, e->d_gbar, 4));
    e->bar_epoch = 0;
    chk(dalloc(e, e->d_toy_chunk0, NT));
    chk(dalloc(e, e->d_toy_nchunks, NT));
    chk(dalloc(e, e->d_toy_nevents, NT));
    const int NA = T.n_amp_cols, NTILE = (int)e->plan.gram_tiles.size();
    size_t ngrid = 0;
    for(auto &A : T.amp3s)
        ngrid += A.grid.size();
    e->gram_blocks = 2 * std::max(1, e->sm_count);
    chk(dalloc(e, e->d_acols, (size_t)NT * std::max(1, NA)));
    chk(dalloc(e, e->d_dcols, (size_t)NT * NO));
    chk(dalloc(e, e->d_dgrid, std::max<size_t>(1, ngrid)));
    chk(dalloc(e, e->d_gram, (size_t)NT * std::max(1, NTILE) * e->gram_blocks * std::max(1, 2 * e->plan.gram_pairs_max)));
    chk(dalloc(e, e->d_dirty, NT));
    // the integrals of the mixed-precision engine go through the tensor-core Gram kernel when every amplitude
    // node has at most 32 complex columns (values and derivatives); GF_GRAM=cuda keeps the CUDA-core kernel
    e->gram_tc = false;
    if(e->precision == GF_MIXED && T.n_amp_nodes() > 0) {
        const char *g = std::getenv("GF_GRAM");
        e->gram_tc    = !(g && std::string(g) == "cuda");
        size_t np = 0, no = 0;
        for(int k = 0; k < T.n_amp_nodes(); ++k) {
            const int nc = ampColumns(T, k);
            if(gf_gram_tc_width(nc) == 0)
                e->gram_tc = false;
            np = std::max(np, gf_gram_tc_part_doubles(nc, std::max(1, e->sm_count)));
            no = std::max(no, (size_t)4 * nc * nc);
        }
        if(e->gram_tc) {
            chk(dalloc(e, e->d_gtc_part, np));
            chk(dalloc(e, e->d_gtc_out, no));
            chk(dalloc(e, e->d_gtc_err, 1));
            e->gtc_part_n = np;
            e->gtc_out_n  = no;
            e->h_gtc.assign(no, 0.0);
        }
    }
    if(rc != GF_OK)
        return rc;
    if(cudaMallocHost((void **)&e->h_gram, sizeof(double) * (size_t)NT * std::max(1, NTILE) * e->gram_blocks *
                                               std::max(1, 2 * e->plan.gram_pairs_max)) != cudaSuccess ||
       cudaMallocHost((void **)&e->h_dirty, sizeof(int) * NT) != cudaSuccess)
        return gf_fail(e, GF_ERR_OOM, "cudaMallocHost");
    {
        std::vector<void *> ac((size_t)NT * std::max(1, NA), nullptr);
        std::vector<double *> dc((size_t)NT * NO, nullptr);
        for(int t = 0; t < NT; ++t) {
            for(int c = 0; c < NA; ++c)
                ac[(size_t)t * NA + c] = e->toys[t].acols[c];
            for(int o = 0; o < NO; ++o)
                dc[(size_t)t * NO + o] = e->toys[t].dcols[o];
        }
        std::vector<unsigned> g;
        g.reserve(ngrid);
        for(auto &A : T.amp3s)
            g.insert(g.end(), A.grid.begin(), A.grid.end());
        cudaMemcpy(e->d_acols, ac.data(), sizeof(void *) * ac.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(e->d_dcols, dc.data(), sizeof(double *) * dc.size(), cudaMemcpyHostToDevice);
        if(!g.empty())
            cudaMemcpy(e->d_dgrid, g.data(), sizeof(unsigned) * g.size(), cudaMemcpyHostToDevice);
    }
    // results: the event kernel's finishing CTA stores them straight into mapped page-locked memory (no
    // copy back at the end of each evaluation)
    if(cudaMallocHost((void **)&e->h_P, e->pblock_bytes) != cudaSuccess ||
       cudaHostAlloc((void **)&e->h_out, sizeof(double) * (size_t)NT * (NGp + 2), cudaHostAllocMapped) != cudaSuccess ||
       cudaHostGetDevicePointer((void **)&e->d_out, e->h_out, 0) != cudaSuccess)
        return gf_fail(e, GF_ERR_OOM, "cudaMallocHost");
    std::memset(e->h_out, 0, sizeof(double) * (size_t)NT * (NGp + 2));
    std::memset(e->h_P, 0, e->pblock_bytes);
    e->h_active = reinterpret_cast<int *>(reinterpret_cast<char *>(e->h_P) + e->active_off);
    e->host_flag.assign(NT, 0);
    for(int t = 0; t < NT; ++t)
        e->h_active[t] = 1;
    std::vector<void *> cols((size_t)NT * NO, nullptr);
    std::vector<int *> kcols((size_t)NT * std::max(1, NC), nullptr);
    for(int t = 0; t < NT; ++t) {
        for(int o = 0; o < NO; ++o)
            cols[(size_t)t * NO + o] = e->toys[t].cols[o];
        for(int c = 0; c < NC; ++c)
            kcols[(size_t)t * NC + c] = e->toys[t].kcols[c];
    }
    cudaMemcpy(e->d_cols, cols.data(), sizeof(void *) * cols.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_kcols, kcols.data(), sizeof(int *) * kcols.size(), cudaMemcpyHostToDevice);
    if(!T.kgrid.empty())
        cudaMemcpy(e->d_kgrid, T.kgrid.data(), sizeof(int) * T.kgrid.size(), cudaMemcpyHostToDevice);
    e->chunk_cap = 0;
    if((rc = setChunks(e, e->chunk)))
        return rc;
    cudaMemcpy(e->d_toy_nevents, ne.data(), sizeof(long long) * NT, cudaMemcpyHostToDevice);
    cudaError_t r = cudaDeviceSynchronize();
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "layout upload");
    if(e->plan.fused_tab && e->n_toys == 1 && e->use_ksort && !e->toys[0].ksort_valid)
        if(int rk = buildKSort(e))
            return rk;
    e->layout_ready = true;
    return GF_OK;
}

GfArgs makeArgs(gf_engine *e) {
    GfArgs a{};
    a.P           = e->d_P;
    a.active      = e->d_active;
    a.col         = (const void *const *)e->d_cols;
    a.kcol        = (const int *const *)e->d_kcols;
    a.ctab        = e->d_ctab;
    a.kgrid       = e->d_kgrid;
    a.gsum        = e->d_gsum;
    a.gpartial    = e->d_gpartial;
    a.gcounter    = e->d_gcounter;
    a.partial     = e->d_partial;
    a.counter     = e->d_counter;
    a.out         = e->d_out;
    a.chunks      = e->d_chunks;
    a.toy_chunk0  = e->d_toy_chunk0;
    a.toy_nchunks = e->d_toy_nchunks;
    a.toy_nevents = e->d_toy_nevents;
    a.vals        = e->d_vals;
    a.Pr          = (const char *)e->d_P + sizeof(double) * (size_t)e->n_toys * std::max(1, e->tree.n_params);
    a.Nq          = e->d_Nq;
    a.qflag       = e->d_qflag;
    a.acol        = (const void *const *)e->d_acols;
    a.dcol        = (const double *const *)e->d_dcols;
    a.dgrid       = e->d_dgrid;
    a.gram        = e->d_gram;
    a.dirty       = e->d_dirty;
    a.nevt        = (const double *const *)e->d_nevt;
    a.nnorm       = e->d_nnorm;
    a.nscr        = (void *const *)e->d_nscr;
    a.gtoy        = 0;
    a.chunk       = e->chunk;
    a.nevt0       = e->toys.empty() ? 0 : e->toys[0].n;
    if(!e->toys.empty()) {
        // toy 0's column pointers by value: the kernels of a single fit read no pointer table
        const gf::Tree &T = e->tree;
        const int NO = (int)T.obs.size(), NC = (int)T.convs.size(), NA = T.n_amp_cols;
        const GfToy &t0 = e->toys[0];
        for(int o = 0; o < NO && o < 192; ++o)
            a.p0[o] = t0.cols[o];
        for(int c = 0; c < NC && NO + c < 192; ++c)
            a.p0[NO + c] = t0.kcols[c];
        for(int c = 0; c < NA && NO + NC + c < 192; ++c)
            a.p0[NO + NC + c] = t0.acols[c];
    }
    a.n_chunks    = e->n_chunks;
    a.n_toys      = e->n_toys;
    a.metric      = 1;
    a.gbar        = e->d_gbar;
    a.bar_ns      = e->bar_ns;
    return a;
}

cudaError_t launch(cudaKernel_t k, dim3 g, dim3 b, size_t smem, cudaStream_t s, GfArgs &a, bool pdl = false) {
    void *args[] = {&a};
    if(!pdl)
        return cudaLaunchKernel((const void *)k, g, b, args, smem, s);
    // programmatic dependent launch: the kernel may start while the previous kernel of the stream is
    // finishing; it waits (griddepcontrol.wait) before it reads that kernel's results
    cudaLaunchAttribute attr[1];
    attr[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim          = g;
    cfg.blockDim         = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream           = s;
    cfg.attrs            = attr;
    cfg.numAttrs         = 1;
    return cudaLaunchKernelExC(&cfg, (const void *)k, args);
}

// Enqueues the prep kernels (conv tables, grid sums) for one variant.
// Enqueues the prep kernels (conv tables, grid sums) for one variant; returns whether a kernel was the last
// operation, so that the next kernel can be chained programmatically.
bool gridWork(const gf_engine *e) {
    for(char f : e->plan.num_folded)
        if(!f)
            return true;
    return false;
}

cudaError_t enqueuePrep(gf_engine *e, bool grad, GfArgs &a, bool *kernelLast = nullptr) {
    const gf::Tree &T = e->tree;
    cudaError_t r     = cudaSuccess;
    bool prevKernel   = false;
    auto conv = [&]() {
        dim3 g(e->plan.conv_blocks, e->n_toys, (unsigned)T.convs.size());
        r = launch(grad ? e->mod.conv_g : e->mod.conv_n, g, dim3(e->block),
                   grad ? e->plan.conv_smem_grad : e->plan.conv_smem_nograd, e->stream, a, prevKernel && e->use_pdl);
        prevKernel = true;
    };
    auto grid = [&]() {
        dim3 g(e->plan.max_grid_blocks, e->n_toys, (unsigned)T.nums.size());
        r = launch(grad ? e->mod.grid_g : e->mod.grid_n, g, dim3(e->block), 0, e->stream, a, prevKernel && e->use_pdl);
        prevKernel = true;
    };
    const bool hasConv = !T.convs.empty(), hasGrid = !T.nums.empty() && gridWork(e);
    if(hasConv && hasGrid && !e->plan.grid_needs_conv) {
        // the grid needs no table (a convolution's own grid sum is folded into the table kernel): the table
        // kernel starts while the grid kernel runs, and waits for it only before it completes
        grid();
        if(r == cudaSuccess)
            conv();
    } else {
        if(hasConv)
            conv();
        if(r == cudaSuccess && hasGrid)
            grid();
    }
    if(kernelLast)
        *kernelLast = prevKernel;
    return r;
}

int evtGrid(const gf_engine *e) { return std::max(1, std::min(e->n_chunks, e->sm_count * e->evt_ctas_per_sm)); }

// An event record that a captured graph keeps as a node (external record) or a plain one outside capture.
cudaError_t recordEvent(gf_engine *e, cudaEvent_t ev) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if(cudaStreamIsCapturing(e->stream, &st) == cudaSuccess && st == cudaStreamCaptureStatusActive)
        return cudaEventRecordWithFlags(ev, e->stream, cudaEventRecordExternal);
    return cudaEventRecord(ev, e->stream);
}

// The gradient event kernel of the engine's amplitude mode, and its dynamic shared memory.
cudaKernel_t evtGradKernel(const gf_engine *e) { return e->amp_recompute ? e->mod.evt_gr : e->mod.evt_g; }
size_t evtGradSmem(const gf_engine *e) { return e->amp_recompute ? e->plan.evt_smem_gr : e->plan.evt_smem_grad; }

// One toy with the one-launch kernels loaded and enabled: the evaluation is a single cooperative launch
// (the store mode's kernels only: recomputed amplitude derivatives use the separate gradient event kernel).
bool fusedPath(const gf_engine *e) {
    return e->use_fused && e->n_toys == 1 && !e->batch_kernels && e->mod.fcn_g && e->mod.fcn_n && e->fcn_grid > 0 &&
           e->h_fpart && !e->amp_recompute;
}

// Arguments of the one-launch kernel: the toy's record (parameters as R, analytic factors) by value when it
// fits, so that no CTA reads it from host memory; the page-locked block in place otherwise; no activity flag
// (the one toy is evaluated whatever its flag says); the chunk rows in mapped host memory.
GfArgs fusedArgs(gf_engine *e, bool grad) {
    GfArgs a    = makeArgs(e);
    a.stage_off = (int)e->plan.fused_stage_off[grad ? 1 : 0];
    a.stage_cap = e->use_stage ? (unsigned)e->plan.fused_stage_cap[grad ? 1 : 0] : 0u;
    const size_t poff = sizeof(double) * (size_t)e->n_toys * std::max(1, e->tree.n_params);
    char *hp          = nullptr;
    if(cudaHostGetDevicePointer((void **)&hp, e->h_P, 0) == cudaSuccess) {
        a.P  = (const double *)hp;
        a.Pr = hp + poff;
    } else
        cudaGetLastError();
    a.active        = nullptr;
    a.hpart         = e->d_fpart;
    a.bar_target    = (e->bar_epoch + 1u) * (unsigned)e->fcn_grid;
    a.ksort         = e->plan.fused_tab && e->toys[0].ksort_valid ? e->toys[0].ksort : nullptr;
    const size_t rb = rsize(e) * (size_t)e->plan.nl.npr;
    a.rec_n         = 0;
    if(rb > 0 && rb <= sizeof(a.rec)) {
        std::memcpy(a.rec, reinterpret_cast<const char *>(e->h_P) + poff, rb);
        a.rec_n = e->plan.nl.npr;
    }
    return a;
}

cudaError_t enqueueEval(gf_engine *e, bool grad) {
    if(fusedPath(e)) {
        // tables, grids and the event pass in one cooperative launch (all CTAs resident, grid barrier)
        GfArgs a      = fusedArgs(e, grad);
        cudaError_t r = recordEvent(e, e->ev[0]);
        if(r == cudaSuccess) {
            void *args[] = {&a};
            cudaLaunchAttribute attr[1];
            attr[0].id              = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cudaLaunchConfig_t cfg{};
            cfg.gridDim          = dim3(e->fcn_grid);
            cfg.blockDim         = dim3(e->block);
            cfg.dynamicSmemBytes = e->plan.fused_smem[grad ? 1 : 0];
            cfg.stream           = e->stream;
            cfg.attrs            = attr;
            cfg.numAttrs         = 1;
            r = cudaLaunchKernelExC(&cfg, (const void *)(grad ? e->mod.fcn_g : e->mod.fcn_n), args);
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if(r == cudaSuccess && cudaStreamIsCapturing(e->stream, &cs) == cudaSuccess &&
               cs == cudaStreamCaptureStatusNone)
                ++e->bar_epoch;
        }
        if(r == cudaSuccess)
            r = recordEvent(e, e->ev[3]);
        return r;
    }
    GfArgs a = makeArgs(e);
    // qflag is zero between evaluations: the event kernel's finisher clears it after reading it
    cudaError_t r = recordEvent(e, e->ev[0]);
    // one toy: the kernels read the parameter block from page-locked host memory in place (no copy
    // node at the head of the graph; C2 FCN 33.8 -> 33.0 us); batches keep the copy (1024 toys' records
    // read over the interconnect by every CTA made the lockstep round 3% slower)
    bool inPlace = false;
    if(e->n_toys == 1) {
        char *hp = nullptr;
        if(cudaHostGetDevicePointer((void **)&hp, e->h_P, 0) == cudaSuccess) {
            a.P      = (const double *)hp;
            a.Pr     = hp + sizeof(double) * (size_t)e->n_toys * std::max(1, e->tree.n_params);
            a.active = (const int *)(hp + e->active_off);
            inPlace  = true;
        } else
            cudaGetLastError();
    }
    if(!inPlace && r == cudaSuccess)
        r = cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
    bool kernelLast = false;
    if(r == cudaSuccess)
        r = enqueuePrep(e, grad, a, &kernelLast);
    if(r == cudaSuccess)
        r = launch(grad ? evtGradKernel(e) : e->mod.evt_n, dim3(evtGrid(e)), dim3(e->block),
                   grad ? evtGradSmem(e) : e->plan.evt_smem_nograd, e->stream, a, kernelLast && e->use_pdl);
    if(r == cudaSuccess)
        r = recordEvent(e, e->ev[3]);
    return r;
}

int statusOf(double st) {
    int s = (int)st;
    if(s & 1)
        return GF_ERR_NAN_NORM;
    if(s & 2)
        return GF_ERR_NONPOS_NORM;
    if(s & 4)
        return GF_ERR_ZERO_NLL;
    if(s & 8)
        return GF_ERR_TIMEOUT;
    return GF_OK;
}

int loadModule(gf_engine *e) {
    std::vector<char> cubin;
    std::string log;
    std::string arch = "sm_103a";
    if(const char *a = std::getenv("GF_ARCH"))
        arch = a;
    if(!gf::rtc_compile(e->plan.source, arch, cubin, log))
        return gf_fail(e, GF_ERR_COMPILE, log);
    freeModule(e);
    cudaError_t r = cudaLibraryLoadData(&e->mod.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "cudaLibraryLoadData");
    auto get = [&](cudaKernel_t &k, const char *name, bool need) -> int {
        cudaError_t rr = cudaLibraryGetKernel(&k, e->mod.lib, name);
        if(rr != cudaSuccess) {
            k = nullptr;
            cudaGetLastError();
            if(need)
                return gf_cuda_check(e, rr, name);
        }
        return GF_OK;
    };
    bool hasConv = !e->tree.convs.empty(), hasGrid = !e->tree.nums.empty();
    int rc = GF_OK;
    if((rc = get(e->mod.conv_g, "gf_conv_g", hasConv)) || (rc = get(e->mod.conv_n, "gf_conv_n", hasConv)) ||
       (rc = get(e->mod.grid_g, "gf_grid_g", hasGrid)) || (rc = get(e->mod.grid_n, "gf_grid_n", hasGrid)) ||
       (rc = get(e->mod.evt_g, "gf_evt_g", true)) || (rc = get(e->mod.evt_n, "gf_evt_n", true)) ||
       (rc = get(e->mod.val_n, "gf_val_n", true)))
        return rc;
    const bool hasAmp = e->tree.n_amp_nodes() > 0;
    if((rc = get(e->mod.amp, "gf_amp", hasAmp)) || (rc = get(e->mod.ampn, "gf_ampn", hasAmp)) ||
       (rc = get(e->mod.gram, "gf_gram", hasAmp)))
        return rc;
    if((rc = get(e->mod.fcn_g, "gf_fcn_g", e->plan.fused)) || (rc = get(e->mod.fcn_n, "gf_fcn_n", e->plan.fused)))
        return rc;
    if((rc = get(e->mod.evt_gr, "gf_evt_gr", e->plan.recompute_kernels)) ||
       (rc = get(e->mod.gramr, "gf_gramr", e->plan.recompute_kernels)))
        return rc;
    auto smem = [&](cudaKernel_t k, size_t bytes) -> int {
        if(!k || bytes <= 48 * 1024)
            return GF_OK;
        return gf_cuda_check(e,
                             cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                             (int)bytes, e->device),
                             "dynamic shared memory attribute");
    };
    if((rc = smem(e->mod.conv_g, e->plan.conv_smem_grad)) || (rc = smem(e->mod.conv_n, e->plan.conv_smem_nograd)) ||
       (rc = smem(e->mod.evt_g, e->plan.evt_smem_grad)) || (rc = smem(e->mod.evt_n, e->plan.evt_smem_nograd)) ||
       (rc = smem(e->mod.evt_gr, e->plan.evt_smem_gr)) ||
       (rc = smem(e->mod.val_n, e->plan.evt_smem_nograd)) || (rc = smem(e->mod.fcn_g, e->plan.fused_smem[1])) ||
       (rc = smem(e->mod.fcn_n, e->plan.fused_smem[0])))
        return rc;
    const size_t maxSmem = 227 * 1024;
    if(e->plan.conv_smem_grad > maxSmem || e->plan.evt_smem_grad > maxSmem)
        return gf_fail(e, GF_ERR_BAD_TREE, "convolution workspaces exceed shared memory");
    return GF_OK;
}

// Scale of an amplitude node's quadratic form: binSizeFactor of Amp3Body::normalize
// (src/PDFs/physics/Amp3Body.cu:350-353), or 1 / (number of normalisation events) for Amp4Body
// (src/PDFs/physics/Amp4Body.cu:542-545).
double ampScale(const gf_engine *e, int node) {
    const gf::Tree &T = e->tree;
    if(T.amp3_of[node] < 0) {
        const int k4 = T.amp4_of[node];
        return k4 < (int)e->norm_n.size() && e->norm_n[k4] > 0 ? 1.0 / (double)e->norm_n[k4] : NAN;
    }
    const gf::Amp3Info &A = T.amp3s[T.amp3_of[node]];
    const gf_observable &o12 = T.obs[A.o12], &o13 = T.obs[A.o13];
    double f = 1;
    f *= (o12.hi - o12.lo) / o12.nbins;
    f *= (o13.hi - o13.lo) / o13.nbins;
    return f;
}

// Normalisation integral of an amplitude node (Amp3Body.cu:334-356, Amp4Body.cu:531-545): the real part
// of sum_ij c_i conj(c_j) I_ij times the node's scale, from the cached integrals; dQ[k] receives the
// derivative of the real part with respect to the k-th entry of an.dN (before the scale).
double ampIntegral(const gf_engine *e, int t, int node, const double *P, const gf::NormLayout::Analytic &an,
                   double *dQ) {
    typedef std::complex<double> C;
    const gf::Tree &T   = e->tree;
    const gf::TNode &nd = T.nodes[node];
    const int ai        = T.amp_index(node);
    const int n         = T.amp_count(ai);
    // integrals not built yet for this toy, or their last rebuild failed (the rebuild empties them first)
    if((int)e->toys[t].amp_I.size() <= ai || e->toys[t].amp_I[ai].empty()) {
        for(size_t k = 0; k < an.dN.size() && k < 64; ++k)
            dQ[k] = 0;
        return NAN;
    }
    const std::vector<double> &I = e->toys[t].amp_I[ai];
    auto Iij = [&](int i, int j) { return C(I[2 * (i * n + j)], I[2 * (i * n + j) + 1]); };
    C sum(0, 0);
    for(int i = 0; i < n; ++i) {
        C ai_(P[nd.params[2 * i]], P[nd.params[2 * i + 1]]);
        for(int j = 0; j < n; ++j) {
            C aj(P[nd.params[2 * j]], -P[nd.params[2 * j + 1]]);
            sum += ai_ * aj * Iij(i, j);
        }
    }
    const auto &theta = T.amp_theta(ai);
    const std::vector<double> &H =
        e->toys[t].amp_H.size() > (size_t)ai && !e->toys[t].amp_H[ai].empty() ? e->toys[t].amp_H[ai] : I;
    for(size_t k = 0; k < an.dN.size() && k < 64; ++k) {
        const int p = T.gparam[an.dN[k].first];
        // a resonance / line-shape parameter: dQ = 2 Re sum_{a dep} sum_b c_a conj(c_b) H_ab
        int row = 0, th = -1;
        for(size_t q = 0; q < theta.size(); ++q) {
            if(theta[q].param == p) {
                th = (int)q;
                break;
            }
            row += (int)theta[q].amps.size();
        }
        if(th >= 0) {
            C d(0, 0);
            for(size_t j = 0; j < theta[th].amps.size(); ++j) {
                const int a = theta[th].amps[j];
                C ca(P[nd.params[2 * a]], P[nd.params[2 * a + 1]]);
                for(int b = 0; b < n; ++b) {
                    C cb(P[nd.params[2 * b]], P[nd.params[2 * b + 1]]);
                    const size_t h = 2 * ((size_t)(row + (int)j) * n + b);
                    d += ca * std::conj(cb) * C(H[h], H[h + 1]);
                }
            }
            dQ[k] = 2 * d.real();
            continue;
        }
        std::vector<C> dc(n);
        for(int i = 0; i < n; ++i)
            dc[i] = C(nd.params[2 * i] == p ? 1.0 : 0.0, nd.params[2 * i + 1] == p ? 1.0 : 0.0);
        C d(0, 0);
        for(int i = 0; i < n; ++i) {
            C ci(P[nd.params[2 * i]], P[nd.params[2 * i + 1]]);
            for(int j = 0; j < n; ++j) {
                C cj(P[nd.params[2 * j]], P[nd.params[2 * j + 1]]);
                d += (dc[i] * std::conj(cj) + ci * std::conj(dc[j])) * Iij(i, j);
            }
        }
        dQ[k] = d.real();
    }
    double ret = sum.real();
    ret *= ampScale(e, node);
    return ret;
}

// Host part of every evaluation: the per-toy records the kernels read (parameters as R, then the
// analytic normalisation factors, computed here from the FP64 parameters exactly as ExpPdf::integrate
// and GaussianPdf::integrate do on the host in the reference).
template <typename R>
void fillRecordsT(gf_engine *e) {
    const gf::Tree &T        = e->tree;
    const gf::NormLayout &nl = e->plan.nl;
    const int NT = e->n_toys, np = T.n_params;
    R *rec = reinterpret_cast<R *>(reinterpret_cast<char *>(e->h_P) + sizeof(double) * (size_t)NT * std::max(1, np));
    e->root_N.assign(NT, 1.0);
    e->root_dN.assign((size_t)NT * std::max(1, T.NG), 0.0);
    static const double rootPi = std::sqrt(std::atan2(0.0, -1.0)), root2 = std::sqrt(2.0);
    for(int t = 0; t < NT; ++t) {
        e->host_flag[t] = 0;
        if(!e->h_active[t])
            continue;
        // the kernels see the parameters rounded to R; the factors computed here use the same rounded values,
        // so that the NLL is one function of the rounded parameters (an event part evaluated at rounded and a
        // normalisation at unrounded parameters would differ by steps of n * ulp * |d(event part)/dp|)
        std::vector<double> Pq(std::max(1, np));
        R *r = rec + (size_t)t * nl.npr;
        for(int j = 0; j < np; ++j) {
            r[j]  = (R)e->h_P[(size_t)t * np + j];
            Pq[j] = (double)r[j];
        }
        const double *P = Pq.data();
        for(auto &an : nl.analytic) {
            const gf::TNode &nd = T.nodes[an.node];
            if(an.kind == gf::NK_AMP3 || an.kind == gf::NK_AMP4) {
                double dQ[64];
                const double Iv = ampIntegral(e, t, an.node, P, an, dQ);
                const double f  = ampScale(e, an.node);
                const double N  = 1.0 / Iv;
                r[an.slotN]     = (R)N;
                r[an.slotNL]    = (R)(N - (double)(R)N);
                for(size_t k = 0; k < an.dN.size(); ++k)
                    r[an.dN[k].second] = (R)(-N * N * f * dQ[k]);
                if(an.node == 0) {
                    e->root_N[t] = N;
                    for(size_t k = 0; k < an.dN.size(); ++k)
                        e->root_dN[(size_t)t * std::max(1, T.NG) + an.dN[k].first] = -N * N * f * dQ[k];
                }
                if(an.node == 0) {
                    if(std::isnan(Iv))
                        e->host_flag[t] |= 1;
                    else if(!(N > 0))
                        e->host_flag[t] |= 2;
                }
                continue;
            }
            double I = 1, dI;
            if(an.kind == gf::NK_EXP) {
                const gf_observable &o = T.obs[nd.obs[0]];
                const double al        = P[nd.params[0]];
                if(0 == al) {
                    I *= o.hi - o.lo;
                    dI = 0.5 * (o.hi * o.hi - o.lo * o.lo);
                } else {
                    const double eh = std::exp(al * o.hi), el = std::exp(al * o.lo);
                    double v        = eh - el;
                    v /= al;
                    I *= v;
                    dI = (o.hi * eh - o.lo * el) / al - I / al;
                }
            } else {
                double sg = P[nd.params[1]];
                sg *= root2 * rootPi;
                I *= sg;
                dI = root2 * rootPi;
            }
            const double N = 1.0 / I;
            r[an.slotN]    = (R)N;
            r[an.slotNL]   = (R)(N - (double)(R)N);
            for(auto &d : an.dN)
                r[d.second] = (R)(-N * N * dI);
            if(an.node == 0) {
                e->root_N[t] = N;
                for(auto &d : an.dN)
                    e->root_dN[(size_t)t * std::max(1, T.NG) + d.first] = -N * N * dI;
            }
            if(an.node == 0) {
                if(std::isnan(I))
                    e->host_flag[t] |= 1;
                else if(!(N > 0))
                    e->host_flag[t] |= 2;
            }
        }
    }
}

void fillRecords(gf_engine *e) {
    if(e->precision == GF_MIXED)
        fillRecordsT<float>(e);
    else
        fillRecordsT<double>(e);
}

// Number of normalisation points of amplitude node k: in-Dalitz bins (Amp3Body) or phase-space events.
int64_t ampPoints(const gf_engine *e, int k) {
    const gf::Tree &T = e->tree;
    if(k < (int)T.amp3s.size())
        return (int64_t)T.amp3s[k].grid.size();
    const int k4 = k - (int)T.amp3s.size();
    return k4 < (int)e->norm_n.size() ? e->norm_n[k4] : 0;
}

// column stride of the scratch columns: the points rounded up to a multiple of 4
int64_t ampStride(const gf_engine *e, int k) { return (std::max<int64_t>(1, ampPoints(e, k)) + 3) / 4 * 4; }

// Bytes the store mode keeps for amplitude derivatives and normalisation points: the derivative columns of every
// toy's events (npad events each) and the normalisation scratch columns.
size_t ampStoreBytes(const gf_engine *e, int64_t npad) {
    const gf::Tree &T = e->tree;
    const size_t rs   = rsize(e);
    size_t nd = 0, scr = 0;
    for(int k = 0; k < T.n_amp_nodes(); ++k) {
        int ndk = 0;
        for(auto &th : T.amp_theta(k))
            ndk += (int)th.amps.size();
        nd += (size_t)ndk;
        scr += (size_t)ampStride(e, k) * ((T.amp_count(k) + ndk) * 2 * rs + rs);
    }
    return (size_t)e->n_toys * (size_t)npad * nd * 2 * rs + scr;
}

// Fixes the amplitude mode of the engine's events (once per tree and toy count, at the first upload).
void decideAmpMode(gf_engine *e, int64_t npad) {
    if(e->amp_decided)
        return;
    bool rc = false;
    if(e->plan.recompute_kernels && e->mod.evt_gr && e->mod.gramr) {
        if(e->amp_mode == GF_AMP_RECOMPUTE)
            rc = true;
        else if(e->amp_mode == GF_AMP_AUTO) {
            size_t budget = (size_t)std::max<int64_t>(0, e->amp_budget);
            if(budget == 0) {
                size_t fr = 0, tot = 0;
                if(cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
                    cudaGetLastError();
                    fr = 0;
                }
                budget = fr / 4;
            }
            rc = ampStoreBytes(e, npad) > budget;
        }
    }
    e->amp_recompute = rc;
    e->amp_decided   = true;
}

// Scratch columns of the normalisation pass: per amplitude node, (values + derivatives) R2 columns and an R
// efficiency column over its points.
int ensureScratch(gf_engine *e) {
    const gf::Tree &T = e->tree;
    const int NK      = T.n_amp_nodes();
    const size_t rs   = rsize(e);
    if((int)e->nscr.size() != NK) {
        for(auto &p : e->nscr)
            if(p)
                cudaFree(p);
        e->nscr.assign(NK, nullptr);
        e->nscr_bytes.assign(NK, 0);
        dfree(e->d_nscr);
        if(int rc = dalloc(e, e->d_nscr, std::max(1, NK)))
            return rc;
    }
    bool changed = false;
    for(int k = 0; k < NK; ++k) {
        int nd = 0;
        for(auto &th : T.amp_theta(k))
            nd += (int)th.amps.size();
        const size_t bytes = (size_t)ampStride(e, k) * ((T.amp_count(k) + nd) * 2 * rs + rs) + 256;
        if(bytes == e->nscr_bytes[k])
            continue;
        if(e->nscr[k])
            cudaFree(e->nscr[k]);
        e->nscr[k]       = nullptr;
        e->nscr_bytes[k] = 0;
        cudaError_t r    = cudaMalloc(&e->nscr[k], bytes);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "cudaMalloc normalisation scratch");
        e->nscr_bytes[k] = bytes;
        changed          = true;
    }
    if(changed) {
        cudaError_t r = cudaMemcpy(e->d_nscr, e->nscr.data(), sizeof(void *) * NK, cudaMemcpyHostToDevice);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "scratch table");
    }
    return GF_OK;
}

// Rebuilds the resonance amplitude caches and the normalisation integrals of the active toys whose
// resonance or efficiency parameters changed since the last build (Amp3Body::normalize's redoIntegral
// logic, src/PDFs/physics/Amp3Body.cu:263-330).  Runs outside the captured evaluation graph; the
// evaluations that follow read the caches and the host copies of the integrals.
int updateAmpCaches(gf_engine *e) {
    const gf::Tree &T = e->tree;
    const int NAN_    = T.n_amp_nodes();
    if(NAN_ == 0)
        return GF_OK;
    for(size_t k = 0; k < T.amp4s.size(); ++k)
        if(k >= e->norm_n.size() || e->norm_n[k] <= 0)
            return gf_fail(e, GF_ERR_STATE, "Amp4Body node " + std::to_string(T.amp4s[k].node) +
                                                " has no normalisation events (gf_set_norm_events)");
    const int NT = e->n_toys, np = T.n_params, NTILE = (int)e->plan.gram_tiles.size();
    const int PM2 = 2 * e->plan.gram_pairs_max;
    std::vector<int> cp;
    for(int k = 0; k < NAN_; ++k)
        cp.insert(cp.end(), T.amp_cache_params(k).begin(), T.amp_cache_params(k).end());
    std::sort(cp.begin(), cp.end());
    cp.erase(std::unique(cp.begin(), cp.end()), cp.end());
    // new events invalidate only the per-event columns, new normalisation points only the integrals, a
    // changed resonance / line-shape / efficiency parameter both
    bool anyData = false, anyNorm = false;
    int64_t maxpad = 8;
    std::vector<std::vector<double>> snap(NT);
    std::vector<char> normDirty(NT, 0);
    for(int t = 0; t < NT; ++t) {
        e->h_dirty[t] = 0;
        if(!e->h_active[t])
            continue;
        const double *P = e->h_P + (size_t)t * np;
        for(int p : cp)
            snap[t].push_back(P[p]);
        GfToy &ty       = e->toys[t];
        const bool pchg = ty.amp_params != snap[t];
        if(pchg || !ty.amp_valid) {
            e->h_dirty[t] = 1;
            anyData       = true;
            maxpad        = std::max<int64_t>(maxpad, ty.npad);
        }
        if(pchg || !ty.norm_valid) {
            normDirty[t] = 1;
            anyNorm      = true;
        }
        if(pchg) {
            ty.amp_valid  = false;
            ty.norm_valid = false;
        }
    }
    if(!anyData && !anyNorm)
        return GF_OK;
    fillRecords(e); // R copies of the parameters for the efficiency in the integral kernel
    int rc = e->amp_recompute ? GF_OK : ensureScratch(e);
    if(rc)
        return rc;
    GfArgs a      = makeArgs(e);
    cudaError_t r = cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
    if(r == cudaSuccess)
        r = cudaMemcpyAsync(e->d_dirty, e->h_dirty, sizeof(int) * NT, cudaMemcpyHostToDevice, e->stream);
    if(r == cudaSuccess && anyData) {
        const int64_t bx = std::min<int64_t>((maxpad + 255) / 256, (int64_t)std::max(1, e->sm_count) * 8);
        r = launch(e->mod.amp, dim3((unsigned)bx, NT, (unsigned)NAN_), dim3(256), 0, e->stream, a);
    }
    if(r == cudaSuccess && anyData && !anyNorm)
        r = cudaStreamSynchronize(e->stream);
    if(r == cudaSuccess)
        for(int t = 0; t < NT; ++t)
            if(e->h_dirty[t]) {
                e->toys[t].amp_valid  = true;
                e->toys[t].amp_params = snap[t];
            }
    int64_t maxpts = 1;
    for(int k = 0; k < NAN_; ++k)
        maxpts = std::max<int64_t>(maxpts, ampPoints(e, k));
    const int64_t bn    = std::min<int64_t>((maxpts + 255) / 256, (int64_t)std::max(1, e->sm_count) * 8);
    const size_t gbytes = sizeof(double) * (size_t)NTILE * e->gram_blocks * PM2;
    for(int t = 0; t < NT && r == cudaSuccess; ++t) {
        if(!normDirty[t])
            continue;
        // the normalisation points of this toy: amplitudes (and derivatives), then their reduction (recompute
        // mode: one kernel that evaluates the amplitudes at every point and reduces them in place)
        a.gtoy = t;
        if(!e->amp_recompute)
            r = launch(e->mod.ampn, dim3((unsigned)bn, 1, (unsigned)NAN_), dim3(256), 0, e->stream, a);
        GfToy &ty = e->toys[t];
        ty.amp_I.assign(NAN_, {});
        ty.amp_H.assign(NAN_, {});
        if(e->gram_tc && !e->amp_recompute) {
            // tensor cores: the real Gram matrix G of each node's columns, then I and H from its blocks
            for(int k = 0; k < NAN_ && r == cudaSuccess; ++k) {
                const int n = T.amp_count(k), nc = ampColumns(T, k), m = 2 * nc;
                const int64_t npts = ampPoints(e, k), nst = ampStride(e, k);
                const float2 *sc   = reinterpret_cast<const float2 *>(e->nscr[k]);
                const float *eff   = k < (int)T.amp3s.size() ? reinterpret_cast<const float *>(sc + (size_t)nc * nst) : nullptr;
                int herr           = 0;
                r = cudaMemsetAsync(e->d_gtc_err, 0, sizeof(int), e->stream);
                // GF_GRAM_TEST_STALL_STAGE (tests of the failure path): the wait for that stage runs out
                const char *stall = std::getenv("GF_GRAM_TEST_STALL_STAGE");
                if(r == cudaSuccess)
                    r = gf_gram_tc_launch(sc, npts, nst, nc, eff, std::max(1, e->sm_count), e->d_gtc_part,
                                          e->d_gtc_out, e->d_gtc_err, e->stream,
                                          e->gram_w >= gf_gram_tc_width(nc) ? e->gram_w : 0, e->gram_ns,
                                          stall && *stall ? std::atoi(stall) : -1);
                if(r == cudaSuccess)
                    r = cudaMemcpyAsync(e->h_gtc.data(), e->d_gtc_out, sizeof(double) * (size_t)m * m,
                                        cudaMemcpyDeviceToHost, e->stream);
                if(r == cudaSuccess)
                    r = cudaMemcpyAsync(&herr, e->d_gtc_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream);
                if(r == cudaSuccess)
                    r = cudaStreamSynchronize(e->stream);
                if(r != cudaSuccess)
                    break;
                if(herr)
                    return gf_fail(e, GF_ERR_CUDA, "tensor-core Gram kernel: a bounded wait ran out");
                const double *G = e->h_gtc.data();
                // X_a conj(X_b) summed: Re = G(re a, re b) + G(im a, im b), Im = G(im a, re b) - G(re a, im b)
                auto ent = [&](int u, int v, double &re, double &im) {
                    re = G[(size_t)(2 * u) * m + 2 * v] + G[(size_t)(2 * u + 1) * m + 2 * v + 1];
                    im = G[(size_t)(2 * u + 1) * m + 2 * v] - G[(size_t)(2 * u) * m + 2 * v + 1];
                };
                std::vector<double> I(2 * (size_t)n * n, 0.0), H(2 * (size_t)std::max(1, nc - n) * n, 0.0);
                for(int i = 0; i < n; ++i)
                    for(int j = i; j < n; ++j) {
                        double re, im;
                        ent(i, j, re, im);
                        if(i == j)
                            im = 0.0;
                        I[2 * (i * n + j)]     = re;
                        I[2 * (i * n + j) + 1] = im;
                        I[2 * (j * n + i)]     = re;
                        I[2 * (j * n + i) + 1] = -im;
                    }
                for(int d = 0; d < nc - n; ++d)
                    for(int b = 0; b < n; ++b)
                        ent(n + d, b, H[2 * (d * n + b)], H[2 * (d * n + b) + 1]);
                ty.amp_I[k] = I;
                ty.amp_H[k] = H;
            }
            if(r != cudaSuccess)
                break;
            ty.amp_params = snap[t];
            ty.norm_valid = true;
            continue;
        }
        if(r == cudaSuccess)
            r = launch(e->amp_recompute ? e->mod.gramr : e->mod.gram, dim3(e->gram_blocks, 1, NTILE), dim3(256), 0,
                       e->stream, a);
        if(r == cudaSuccess)
            r = cudaMemcpyAsync(e->h_gram, e->d_gram, gbytes, cudaMemcpyDeviceToHost, e->stream);
        if(r == cudaSuccess)
            r = cudaStreamSynchronize(e->stream);
        if(r != cudaSuccess)
            break;
        for(int k = 0; k < NAN_; ++k) {
            const int n = T.amp_count(k);
            int nd      = 0;
            for(auto &th : T.amp_theta(k))
                nd += (int)th.amps.size();
            std::vector<double> I(2 * (size_t)n * n, 0.0), H(2 * (size_t)std::max(1, nd) * n, 0.0);
            // entry q of the node: pairs i <= j, then derivative rows d x n (the generator's order)
            std::vector<std::array<int, 3>> ent;
            for(int i = 0; i < n; ++i)
                for(int j = i; j < n; ++j)
                    ent.push_back({0, i, j});
            for(int d = 0; d < nd; ++d)
                for(int b = 0; b < n; ++b)
                    ent.push_back({1, d, b});
            for(int z = 0; z < NTILE; ++z) {
                const auto &tile = e->plan.gram_tiles[z];
                if(tile.amp != k)
                    continue;
                for(int q = tile.p0; q < tile.p1; ++q) {
                    const int l = q - tile.p0;
                    double re = 0, im = 0;
                    for(int b = 0; b < e->gram_blocks; ++b) {
                        const double *g = e->h_gram + ((size_t)z * e->gram_blocks + b) * PM2;
                        re += g[2 * l];
                        im += g[2 * l + 1];
                    }
                    const int i = ent[q][1], j = ent[q][2];
                    if(ent[q][0] == 0) {
                        I[2 * (i * n + j)]     = re;
                        I[2 * (i * n + j) + 1] = im;
                        I[2 * (j * n + i)]     = re;
                        I[2 * (j * n + i) + 1] = i == j ? im : -im;
                    } else {
                        H[2 * (i * n + j)]     = re;
                        H[2 * (i * n + j) + 1] = im;
                    }
                }
            }
            ty.amp_I[k] = I;
            ty.amp_H[k] = H;
        }
        ty.amp_params = snap[t];
        ty.norm_valid = true;
    }
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "amplitude caches");
    return GF_OK;
}

// Host completion of one toy's result o = [nll, status, grad...]: status bits of host-computed factors and
// the extended AddPdf term (AddPdf::calculateNLL, src/PDFs/combine/AddPdf.cu:187-204).
void postToy(gf_engine *e, int t, double *o) {
    const gf::Tree &T = e->tree;
    int st            = (int)o[1] | e->host_flag[t];
    if(e->plan.factor_root && !(st & 3)) {
        // -log(P N) summed: the kernels returned sum -log P (and -dP/P) and the count of events with P > 0
        const double cnt = o[2 + T.NG], N = e->root_N[t];
        o[0] += -cnt * std::log(N);
        for(int s = 0; s < T.NG; ++s)
            o[2 + s] += -cnt * e->root_dN[(size_t)t * std::max(1, T.NG) + s] / N;
        if(o[0] == 0.0)
            st |= 4;
    }
    if(T.extended_root && !(st & 4)) {
        // the yields as the kernels saw them (rounded to R in GF_MIXED)
        const double *P = e->h_P + (size_t)t * T.n_params;
        auto q          = [&](int p) { return e->precision == GF_MIXED ? (double)(float)P[p] : P[p]; };
        double ex       = 0;
        for(int p : T.nodes[0].params)
            ex += q(p);
        const double ne = e->toys[t].total;
        o[0] += (ex - ne * std::log(ex));
        for(int p : T.nodes[0].params)
            if(T.gslot[p] >= 0)
                o[2 + T.gslot[p]] += 1.0 - ne / ex;
    }
    o[1] = (double)st;
}

} // namespace

int gf_fail(gf_engine *e, int code, const std::string &msg) {
    if(e)
        e->err = msg;
    else
        g_create_err = msg;
    return code;
}

int gf_cuda_check(gf_engine *e, cudaError_t r, const char *what) {
    if(r == cudaSuccess)
        return GF_OK;
    return gf_fail(e, r == cudaErrorMemoryAllocation ? GF_ERR_OOM : GF_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(r));
}

// Runs one evaluation of every active toy.  Results land in e->h_out.
// The event-chunking autotuner, keyed by (tree, precision, toys, events): one full evaluation (so that the
// tables, normalisations and caches the event kernel reads are valid), then the gradient event kernel timed
// with CUDA events after an L2 flush (best of 5 after 2 warm-up launches) at chunk sizes base/2, base,
// 2 base, 4 base; the fastest is kept for the engine and remembered for the process.
int autotune(gf_engine *e) {
    static std::mutex mu;
    static std::map<std::string, int> cache;
    int64_t total = 0;
    for(auto &t : e->toys)
        total += t.n;
    const std::string key = std::to_string(std::hash<std::string>{}(e->plan.source)) + ":" +
                            std::to_string(e->precision) + ":" + std::to_string(e->n_toys) + ":" + std::to_string(total);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if(it != cache.end())
            return it->second == e->chunk ? GF_OK : setChunks(e, it->second);
    }
    {
        GfArgs a0    = makeArgs(e);
        cudaError_t r0 = cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
        if(r0 == cudaSuccess)
            r0 = enqueuePrep(e, true, a0);
        if(r0 == cudaSuccess)
            r0 = launch(evtGradKernel(e), dim3(evtGrid(e)), dim3(e->block), evtGradSmem(e), e->stream, a0);
        if(r0 == cudaSuccess)
            r0 = cudaStreamSynchronize(e->stream);
        if(r0 != cudaSuccess)
            return gf_cuda_check(e, r0, "autotune evaluation");
    }
    cudaError_t r = cudaSuccess;
    // each timed launch starts from a cold L2 (a device buffer of twice the L2 size is overwritten before it),
    // as for inputs larger than L2 and as the benchmark measures
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, e->device);
    const size_t flushBytes = (size_t)std::max(l2, 1 << 20) * 2;
    void *flush             = nullptr;
    if(cudaMalloc(&flush, flushBytes) != cudaSuccess) {
        cudaGetLastError();
        flush = nullptr;
    }
    const int base = e->chunk;
    std::vector<int> cands;
    for(int64_t c : {(int64_t)base / 2, (int64_t)base, 2 * (int64_t)base, 4 * (int64_t)base}) {
        c = std::min<int64_t>(std::max<int64_t>((c + 255) / 256 * 256, 256), 1 << 20);
        if(std::find(cands.begin(), cands.end(), (int)c) == cands.end())
            cands.push_back((int)c);
    }
    int best      = base;
    float bestMs  = 1e30f;
    for(int c : cands) {
        int rc = setChunks(e, c);
        if(rc)
            return rc;
        GfArgs a = makeArgs(e);
        float mn = 1e30f;
        for(int it = 0; it < 7 && r == cudaSuccess; ++it) {
            if(flush)
                r = cudaMemsetAsync(flush, it & 0xff, flushBytes, e->stream);
            if(r == cudaSuccess)
                r = cudaEventRecord(e->ev[1], e->stream);
            if(r == cudaSuccess)
                r = launch(evtGradKernel(e), dim3(evtGrid(e)), dim3(e->block), evtGradSmem(e), e->stream, a);
            if(r == cudaSuccess)
                r = cudaEventRecord(e->ev[2], e->stream);
            if(r == cudaSuccess)
                r = cudaStreamSynchronize(e->stream);
            float ms = 0;
            if(r == cudaSuccess && it >= 2 && cudaEventElapsedTime(&ms, e->ev[1], e->ev[2]) == cudaSuccess)
                mn = std::min(mn, ms);
        }
        if(r != cudaSuccess) {
            if(flush)
                cudaFree(flush);
            return gf_cuda_check(e, r, "autotune timing");
        }
        if(mn < bestMs) {
            bestMs = mn;
            best   = c;
        }
    }
    if(flush)
        cudaFree(flush);
    {
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = best;
    }
    e->tuned_chunk = best;
    return best == e->chunk ? GF_OK : setChunks(e, best);
}

// NVTX range for the scope of one FCN phase (visible in Nsight Systems / Nsight Compute; no cost otherwise)
struct NvtxScope {
    explicit NvtxScope(const char *name) { nvtxRangePushA(name); }
    ~NvtxScope() { nvtxRangePop(); }
};

// The host's mark of a one-launch row word not yet written: a signalling-NaN bit pattern, which no arithmetic
// result (quiet NaNs only) and no status or zero the kernel stores can equal.
static constexpr uint64_t kRowUnset = 0x7ff40000dead0001ull;

// A row word written by the device into mapped host memory (one aligned 8-byte store), read as a double.
static inline double wordValue(const uint64_t *p) {
    const uint64_t u = __atomic_load_n(p, __ATOMIC_RELAXED);
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
}

// Device time of the last evaluation (its CUDA events), read when first asked for after the evaluation.
double lastMsTotal(const gf_engine *e) {
    if(e->timing_pending) {
        e->timing_pending = false;
        float ms = 0;
        if(cudaEventSynchronize(e->ev[3]) == cudaSuccess && cudaEventElapsedTime(&ms, e->ev[0], e->ev[3]) == cudaSuccess)
            e->last_ms_total = ms;
        else
            cudaGetLastError();
    }
    return e->last_ms_total;
}

int gf_run(gf_engine *e, bool grad, int, int) {
    NvtxScope fcn(grad ? "gf_fcn_grad" : "gf_fcn");
    int rc = buildLayout(e);
    if(rc)
        return rc;
    {
        NvtxScope s("gf_amplitude_caches");
        if((rc = updateAmpCaches(e)))
            return rc;
    }
    fillRecords(e);
    if(e->tune_pending) {
        NvtxScope s("gf_autotune");
        e->tune_pending = false;
        if((rc = autotune(e)))
            return rc;
    }
    // one-launch evaluation: every word of every chunk row starts as kRowUnset and only the CTA that evaluated
    // the chunk overwrites it, so the host can read each word as soon as it changes, and an evaluation that a
    // barrier wait stopped cannot pass for a result
    const bool fused = fusedPath(e);
    const int frow   = fused ? e->plan.fused_row[grad ? 1 : 0] : 0;
    if(fused) {
        uint64_t *w = reinterpret_cast<uint64_t *>(e->h_fpart);
        for(size_t i = 0, n = (size_t)e->n_chunks * frow; i < n; ++i)
            w[i] = kRowUnset;
    }
    cudaError_t r;
    if(e->use_graph && !(fused && (!e->fused_graph_ok || e->fused_direct))) {
        cudaGraphExec_t &ge = e->graph[grad ? 1 : 0];
        if(!ge) {
            cudaGraph_t g = nullptr;
            r             = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
            if(r != cudaSuccess)
                return gf_cuda_check(e, r, "cudaStreamBeginCapture");
            cudaError_t r1 = enqueueEval(e, grad);
            r              = cudaStreamEndCapture(e->stream, &g);
            if(r1 == cudaSuccess && r == cudaSuccess) {
                r = cudaGraphInstantiate(&ge, g, 0);
                if(r != cudaSuccess)
                    ge = nullptr;
            }
            if(fused && ge) {
                // the graph's one kernel node: its arguments carry the record, replaced before every launch
                size_t nn = 0;
                cudaGraphGetNodes(g, nullptr, &nn);
                std::vector<cudaGraphNode_t> nodes(nn);
                cudaGraphGetNodes(g, nodes.data(), &nn);
                cudaGraphNode_t kn = nullptr;
                for(auto nd : nodes) {
                    cudaGraphNodeType ty;
                    if(cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                        kn = nd;
                }
                if(kn) {
                    cudaKernelNodeParams &kp = e->fused_kp[grad ? 1 : 0];
                    kp                       = cudaKernelNodeParams{};
                    kp.func                  = (void *)(grad ? e->mod.fcn_g : e->mod.fcn_n);
                    kp.gridDim               = dim3(e->fcn_grid);
                    kp.blockDim              = dim3(e->block);
                    kp.sharedMemBytes        = (unsigned)e->plan.fused_smem[grad ? 1 : 0];
                    e->graph_src[grad ? 1 : 0]  = g;
                    e->fused_node[grad ? 1 : 0] = kn;
                    g                           = nullptr;
                } else {
                    cudaGetLastError();
                    cudaGraphExecDestroy(ge);
                    ge = nullptr;
                    r  = cudaErrorNotSupported;
                }
            }
            if(g)
                cudaGraphDestroy(g);
            if(fused && (r1 != cudaSuccess || r != cudaSuccess)) {
                // a cooperative launch this runtime does not capture: launch it directly from now on
                cudaGetLastError();
                e->fused_graph_ok = false;
                ge                = nullptr;
            } else if(r1 != cudaSuccess)
                return gf_cuda_check(e, r1, "capturing the evaluation graph");
            else if(r != cudaSuccess)
                return gf_cuda_check(e, r, "cudaStreamEndCapture / cudaGraphInstantiate");
        }
        if(ge) {
            NvtxScope s("gf_graph_launch");
            if(fused) {
                GfArgs a                = fusedArgs(e, grad);
                void *args[]            = {&a};
                cudaKernelNodeParams kp = e->fused_kp[grad ? 1 : 0];
                kp.kernelParams         = args;
                kp.extra                = nullptr;
                r                       = cudaGraphExecKernelNodeSetParams(ge, e->fused_node[grad ? 1 : 0], &kp);
                if(r != cudaSuccess) {
                    // this runtime does not update the captured cooperative node: launch directly from now on
                    cudaGetLastError();
                    e->fused_graph_ok = false;
                    r                 = enqueueEval(e, grad);
                } else {
                    r = cudaGraphLaunch(ge, e->stream);
                    if(r == cudaSuccess)
                        ++e->bar_epoch;
                }
            } else
                r = cudaGraphLaunch(ge, e->stream);
        } else
            r = enqueueEval(e, grad);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "evaluation launch");
    } else {
        r = enqueueEval(e, grad);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "launch");
    }
    bool stopped = false;
    if(fused) {
        // the chunk rows in chunk order: sums of the components, the OR of the status words. Each word of a row
        // is written once per launch by one aligned 8-byte store, so a word that no longer holds kRowUnset is
        // final: the host adds the rows as they arrive instead of waiting for the launch to end and its stream
        // to report it (5-6 us per FCN), and the kernel needs no fence. A row still holding kRowUnset once the
        // stream reports the launch's end was never written (its CTA stopped at a barrier or on its bulk copy).
        const int nc = frow - 1, NGp = 1 + (grad ? e->tree.NG : 0);
        std::vector<double> &sum = e->fsum;
        sum.assign(std::max(1, nc), 0.0);
        int st = 0;
        bool ended = false;
        if(e->wait_sync) {
            // GF_WAIT_SYNC=1: wait for the launch's end first (the rows are then all final or never written)
            if((r = cudaStreamSynchronize(e->stream)) != cudaSuccess)
                return gf_cuda_check(e, r, "evaluation");
            ended = true;
        }
        unsigned spins = 0;
        for(int c = 0; c < e->n_chunks;) {
            const uint64_t *row = reinterpret_cast<const uint64_t *>(e->h_fpart + (size_t)c * frow);
            bool ready = true;
            for(int k = 0; k < frow && ready; ++k)
                ready = __atomic_load_n(row + k, __ATOMIC_RELAXED) != kRowUnset;
            if(!ready && !ended) {
                if((++spins & 127u) == 0) {
                    r = cudaStreamQuery(e->stream);
                    if(r == cudaSuccess)
                        ended = true; // the launch's writes are all visible: read this row once more
                    else if(r != cudaErrorNotReady)
                        return gf_cuda_check(e, r, "evaluation");
                }
                continue;
            }
            if(!ready)
                stopped = true;
            else {
                st |= (int)wordValue(row + nc);
                for(int k = 0; k < nc; ++k)
                    sum[k] += wordValue(row + k);
            }
            ++c;
        }
        e->timing_pending = true;
        double *o = e->h_out;
        o[0]      = sum[0];
        for(int k = 1; k < NGp; ++k)
            o[1 + k] = sum[k];
        if(e->plan.factor_root)
            o[2 + e->tree.NG] = sum[NGp];
        else if(o[0] == 0.0)
            st |= 4;
        o[1]    = (double)st;
        stopped = stopped || (st & 8);
        if(!stopped && (st & 3)) {
            // a numeric normalisation was NaN or not positive: clear the flag word for the next evaluation
            cudaMemsetAsync(e->d_qflag, 0, sizeof(int) * e->n_toys, e->stream);
            cudaStreamSynchronize(e->stream);
        }
    } else {
        r = cudaStreamSynchronize(e->stream);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "evaluation");
        e->timing_pending = true;
        lastMsTotal(e);
    }
    if(stopped) {
        // a grid barrier wait ran out: clear the barrier words and the completion counters and flags that
        // the stopped CTAs left behind, so that the next evaluation starts clean
        const gf::Tree &T = e->tree;
        cudaMemsetAsync(e->d_gbar, 0, 4 * sizeof(unsigned), e->stream);
        e->bar_epoch = 0;
        cudaMemsetAsync(e->d_counter, 0, sizeof(unsigned) * e->n_toys, e->stream);
        cudaMemsetAsync(e->d_gcounter, 0, sizeof(unsigned) * e->n_toys * std::max<size_t>(1, T.nums.size()), e->stream);
        cudaMemsetAsync(e->d_qflag, 0, sizeof(int) * e->n_toys, e->stream);
        r = cudaStreamSynchronize(e->stream);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "clearing the grid barrier");
        e->h_out[1] = 8.0;
        return gf_fail(e, GF_ERR_TIMEOUT, "a grid barrier wait of the one-launch evaluation ran out");
    }
    return GF_OK;
}

extern "C" {

const char *gf_version(void) {
    static std::string v = "gfengine 0.1 (sm_103a, nvrtc " + gf::rtc_version() + ")";
    return v.c_str();
}

const char *gf_last_error(const gf_engine *eng) { return eng ? eng->err.c_str() : g_create_err.c_str(); }

int gf_engine_create(gf_engine **out, int device, int precision) {
    if(!out)
        return gf_fail(nullptr, GF_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if(precision != GF_FP64 && precision != GF_MIXED)
        return gf_fail(nullptr, GF_ERR_INVALID, "precision must be GF_FP64 or GF_MIXED");
    int count      = 0;
    cudaError_t r  = cudaGetDeviceCount(&count);
    if(r != cudaSuccess || count == 0) {
        cudaGetLastError();
        return gf_fail(nullptr, GF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(r));
    }
    if(device < 0 || device >= count)
        return gf_fail(nullptr, GF_ERR_INVALID, "device index out of range");
    gf_engine *e = new(std::nothrow) gf_engine();
    if(!e)
        return gf_fail(nullptr, GF_ERR_OOM, "out of host memory");
    e->device    = device;
    e->precision = precision;
    if((r = cudaSetDevice(device)) != cudaSuccess || (r = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        g_create_err = std::string("CUDA init: ") + cudaGetErrorString(r);
        delete e;
        return GF_ERR_CUDA;
    }
    for(auto &ev : e->ev)
        cudaEventCreate(&ev);
    cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device);
    if(const char *g = std::getenv("GF_NO_GRAPH"))
        e->use_graph = !(g[0] == '1');
    if(const char *d = std::getenv("GF_FUSED_DIRECT"))
        e->fused_direct = d[0] == '1';
    if(const char *w = std::getenv("GF_WAIT_SYNC"))
        e->wait_sync = w[0] == '1';
    if(const char *c = std::getenv("GF_CHUNK")) {
        e->chunk       = std::max(256, (atoi(c) / 256) * 256);
        e->chunk_fixed = true;
    }
    // programmatic dependent launch chains the mixed engine's kernels (C2 FCN 32.3 -> 30.0 us); in the FP64
    // engine the early-resident event CTAs slowed the chain instead (C2 FCN 193 -> 455 us), so it is off there
    e->use_pdl = precision == GF_MIXED;
    if(const char *p = std::getenv("GF_NO_PDL"))
        e->use_pdl = e->use_pdl && !(p[0] == '1');
    if(const char *f = std::getenv("GF_FUSED"))
        e->use_fused = !(f[0] == '0');
    if(const char *ks = std::getenv("GF_KSORT"))
        e->use_ksort = ks[0] != '0';
    if(const char *st = std::getenv("GF_STAGE"))
        e->use_stage = !(st[0] == '0');
    if(const char *c = std::getenv("GF_EVT_CTAS_PER_SM")) {
        e->evt_ctas_per_sm   = std::max(1, atoi(c));
        e->evt_ctas_fixed    = true;
    }
    e->toys.assign(1, GfToy());
    *out = e;
    return GF_OK;
}

int gf_engine_destroy(gf_engine *e) {
    if(!e)
        return GF_OK;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    freeLayout(e);
    for(auto &t : e->toys)
        freeToy(t);
    freeNormEvents(e);
    dfree(e->d_vals);
    dfree(e->d_stage);
    hfree(e->h_uperr);
    freeModule(e);
    for(auto &ev : e->ev)
        if(ev)
            cudaEventDestroy(ev);
    if(e->stream)
        cudaStreamDestroy(e->stream);
    delete e;
    return GF_OK;
}

static int compileTree(gf_engine *e);

int gf_set_tree(gf_engine *e, const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                const int32_t *grad_mask) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    cudaSetDevice(e->device);
    gf::Tree t;
    // binned metrics: two more columns after the observables, the bin content and the volume / error
    std::vector<gf_observable> ob(obs, obs + std::max(0, n_obs));
    if(e->fit_metric != GF_FIT_UNBINNED_NLL) {
        ob.push_back(gf_observable{-1e300, 1e300, 1, 0});
        ob.push_back(gf_observable{-1e300, 1e300, 1, 0});
    }
    t.fit_metric    = e->fit_metric;
    std::string why = t.build(nodes, n_nodes, ob.data(), (int)ob.size(), n_params, grad_mask);
    if(!why.empty())
        return gf_fail(e, GF_ERR_BAD_TREE, why);
    freeLayout(e);
    for(auto &ty : e->toys)
        freeToy(ty);
    freeNormEvents(e);
    e->tree        = t;
    e->has_tree    = false;
    e->amp_decided = false;
    if(!t.amp4s.empty()) {
        const size_t k = t.amp4s.size();
        e->norm_buf.assign(k, nullptr);
        e->norm_n.assign(k, 0);
        int rc = dalloc(e, e->d_nevt, k);
        if(!rc)
            rc = dalloc(e, e->d_nnorm, k);
        if(rc)
            return rc;
    }
    int rc = compileTree(e);
    if(rc)
        return rc;
    e->layout_ready = false;
    e->has_tree     = true;
    return GF_OK;
}

// Generates and loads the kernels of the engine's tree, shaped for one toy or for a batch of toys, and
// sizes the event chunks from the gradient event kernel's occupancy.
static int compileTree(gf_engine *e) {
    e->batch_kernels = e->n_toys > 1;
    try {
        e->plan = gf::generate_kernels(e->tree, e->precision == GF_MIXED, e->block, e->batch_kernels, e->shapes);
    } catch(std::exception &ex) {
        return gf_fail(e, GF_ERR_BAD_TREE, ex.what());
    }
    int rc = loadModule(e);
    if(rc)
        return rc;
    if(!e->evt_ctas_fixed) {
        // resident CTAs per SM of the gradient event kernel (the one a fit runs), for the chunk layout
        int occ = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)e->mod.evt_g, e->block,
                                                         e->plan.evt_smem_grad) != cudaSuccess) {
            cudaGetLastError();
            occ = 0;
        }
        e->evt_ctas_per_sm = std::min(8, std::max(1, occ));
    }
    // the one-launch kernel's grid: every CTA resident (a cooperative launch), at most as many per SM as the
    // event kernel's chunk layout assumes
    e->fcn_grid = 0;
    if(e->plan.fused && e->mod.fcn_g && e->mod.fcn_n) {
        int o1 = 0, o0 = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, (const void *)e->mod.fcn_g, e->block,
                                                         e->plan.fused_smem[1]) != cudaSuccess ||
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o0, (const void *)e->mod.fcn_n, e->block,
                                                         e->plan.fused_smem[0]) != cudaSuccess) {
            cudaGetLastError();
            o1 = o0 = 0;
        }
        const int per = std::min(std::min(o1, o0), e->evt_ctas_per_sm);
        e->fcn_grid   = per > 0 ? per * e->sm_count : 0;
    }
    return GF_OK;
}

int gf_set_fit_metric(gf_engine *e, int fit_metric) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    if(fit_metric < GF_FIT_UNBINNED_NLL || fit_metric > GF_FIT_BINNED_CHISQ)
        return gf_fail(e, GF_ERR_INVALID, "unknown fit metric");
    if(e->has_tree && fit_metric != e->fit_metric)
        return gf_fail(e, GF_ERR_STATE, "gf_set_fit_metric must come before gf_set_tree");
    e->fit_metric = fit_metric;
    return GF_OK;
}

int gf_set_num_toys(gf_engine *e, int n) {
    if(!e || n < 1)
        return gf_fail(e, GF_ERR_INVALID, "toy count must be >= 1");
    cudaSetDevice(e->device);
    freeLayout(e);
    for(auto &t : e->toys)
        freeToy(t);
    e->n_toys = n;
    e->toys.assign(n, GfToy());
    e->amp_decided = false;
    // one toy and batches of toys use differently shaped table and grid kernels
    if(e->has_tree && (n > 1) != e->batch_kernels)
        return compileTree(e);
    return GF_OK;
}

int gf_upload_events(gf_engine *e, int toy, const double *soa, int64_t n) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    if(!e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "gf_set_tree must come before gf_upload_events");
    if(toy < 0 || toy >= e->n_toys)
        return gf_fail(e, GF_ERR_INVALID, "toy index out of range");
    if(n < 0 || (n > 0 && !soa))
        return gf_fail(e, GF_ERR_INVALID, "bad event array");
    cudaSetDevice(e->device);
    const gf::Tree &T = e->tree;
    const int NO = (int)T.obs.size(), NC = (int)T.convs.size();
    GfToy &ty    = e->toys[toy];
    int64_t npad = std::max<int64_t>(8, (n + 7) / 8 * 8);
    size_t rs    = rsize(e);
    cudaError_t r;
    // a re-upload of the same size keeps the buffers, the chunk layout and the captured graphs
    const bool reuse = ty.loaded && ty.n == n && ty.npad == npad;
    if(!reuse) {
        freeToy(ty);
        e->layout_ready = false;
        dropGraphs(e);
        size_t colBytes = (size_t)npad * rs, kBytes = (size_t)npad * sizeof(int);
        void *base      = nullptr;
        r = cudaMalloc(&base, colBytes * NO + kBytes * std::max(NC, 0) + 256);
        if(r != cudaSuccess)
            return gf_cuda_check(e, r, "cudaMalloc events");
        for(int o = 0; o < NO; ++o)
            ty.cols[o] = (char *)base + colBytes * o;
        for(int c = 0; c < NC; ++c)
            ty.kcols[c] = (int *)((char *)base + colBytes * NO + kBytes * c);
        // Amp3Body: cached amplitudes (R2 per event and resonance) and, in mixed precision, FP64 copies of
        // the Dalitz variables for the amplitude kernel
        const int NA = T.n_amp_cols;
        if(NA > 0) {
            decideAmpMode(e, npad);
            // recompute mode: no derivative columns (their pointers stay null)
            std::vector<char> keep(NA, 1);
            if(e->amp_recompute)
                for(int k = 0; k < T.n_amp_nodes(); ++k)
                    for(auto &th : T.amp_theta(k))
                        for(size_t j = 0; j < th.amps.size(); ++j)
                            keep[th.col0 + (int)j] = 0;
            int nkeep = 0;
            for(int c = 0; c < NA; ++c)
                nkeep += keep[c];
            std::vector<int> dob;
            for(auto &A : T.amp3s)
                for(int o : {A.o12, A.o13})
                    if(std::find(dob.begin(), dob.end(), o) == dob.end())
                        dob.push_back(o);
            for(auto &A : T.amp4s)
                for(int o : A.obs)
                    if(std::find(dob.begin(), dob.end(), o) == dob.end())
                        dob.push_back(o);
            const bool mixed = e->precision == GF_MIXED;
            size_t aBytes    = (size_t)npad * 2 * rs;
            size_t bytes     = aBytes * nkeep + (mixed ? (size_t)npad * 8 * dob.size() : 0) + 256;
            r                = cudaMalloc(&ty.abase, bytes);
            if(r != cudaSuccess) {
                freeToy(ty);
                return gf_cuda_check(e, r, "cudaMalloc amplitude cache");
            }
            for(int c = 0, q = 0; c < NA; ++c)
                ty.acols[c] = keep[c] ? (char *)ty.abase + aBytes * q++ : nullptr;
            for(size_t k = 0; k < dob.size(); ++k)
                ty.dcols[dob[k]] = mixed ? (double *)((char *)ty.abase + aBytes * nkeep + (size_t)npad * 8 * k)
                                         : (double *)ty.cols[dob[k]];
        }
    }
    ty.amp_valid = false;
    const int64_t need = std::max<int64_t>(1, n) * NO;
    if(e->stage_cap < need) {
        dfree(e->d_stage);
        r = cudaMalloc((void **)&e->d_stage, sizeof(double) * need);
        if(r != cudaSuccess) {
            e->stage_cap = 0;
            return gf_cuda_check(e, r, "cudaMalloc staging");
        }
        e->stage_cap = need;
    }
    if(!e->h_uperr) {
        if((r = cudaHostAlloc((void **)&e->h_uperr, sizeof(int), cudaHostAllocMapped)) != cudaSuccess)
            return gf_cuda_check(e, r, "cudaHostAlloc flag");
    }
    double *stage = e->d_stage;
    // the conversion kernel raises the range error in page-locked host memory, read after the synchronise
    // below (no memset, no copy back)
    int *derr = nullptr;
    if((r = cudaHostGetDevicePointer((void **)&derr, e->h_uperr, 0)) != cudaSuccess)
        return gf_cuda_check(e, r, "mapped flag");
    *(volatile int *)e->h_uperr = 0;
    // page-locked host events are read by the conversion kernel in place (no staging copy); other host
    // memory goes through the device staging buffer
    const double *src = stage;
    bool direct       = false;
    {
        cudaPointerAttributes pa{};
        const char *st = std::getenv("GF_UPLOAD_STAGE");
        if(n > 0 && !(st && st[0] == '1') && cudaPointerGetAttributes(&pa, soa) == cudaSuccess &&
           pa.type == cudaMemoryTypeHost && pa.devicePointer) {
            src    = static_cast<const double *>(pa.devicePointer);
            direct = true;
        }
        cudaGetLastError();
    }
    if(n > 0 && !direct)
        cudaMemcpyAsync(stage, soa, sizeof(double) * n * NO, cudaMemcpyHostToDevice, e->stream);
    ConvertArgs a{};
    a.soa    = src;
    a.n      = n;
    a.npad   = npad;
    a.n_obs  = NO;
    a.n_conv = NC;
    for(int o = 0; o < NO; ++o) {
        a.cols[o]    = ty.cols[o];
        a.pad_val[o] = 0.5 * (T.obs[o].lo + T.obs[o].hi);
    }
    for(int c = 0; c < NC; ++c) {
        a.kcols[c]     = ty.kcols[c];
        a.conv_obs[c]  = T.convs[c].obs;
        a.conv_lo[c]   = T.convs[c].lo;
        a.conv_step[c] = T.convs[c].step;
        {
            double lbo = T.convs[c].lo / T.convs[c].step;
            lbo -= std::floor(lbo);
            a.conv_lbo[c]      = lbo;
            a.conv_lbo_f[c]    = (float)lbo;
            a.conv_inv_step[c] = (float)(1.0 / T.convs[c].step);
        }
        a.conv_kmin[c] = T.convs[c].kmin;
        a.conv_kmax[c] = T.convs[c].kmax;
    }
    a.err = derr;
    unsigned blocks = (unsigned)((npad + 255) / 256);
    // the one-launch tabulated path sorts toy 0's events by bin offset
    const bool sorted = toy == 0 && e->n_toys == 1 && e->plan.fused_tab && e->use_ksort && NC > 0;
    if(e->precision == GF_MIXED)
        gf_convert_events<float><<<blocks, 256, 0, e->stream>>>(a);
    else
        gf_convert_events<double><<<blocks, 256, 0, e->stream>>>(a);
    if(e->precision == GF_MIXED && n > 0)
        for(int o = 0; o < NO; ++o)
            if(ty.dcols[o])
                cudaMemcpyAsync(ty.dcols[o], src + (size_t)o * n, sizeof(double) * n, cudaMemcpyDefault, e->stream);
    r        = cudaStreamSynchronize(e->stream);
    int herr = *(volatile int *)e->h_uperr;
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "event conversion");
    ty.n      = n;
    ty.npad   = npad;
    ty.loaded = true;
    ty.total  = (double)n;
    if(e->fit_metric != GF_FIT_UNBINNED_NLL) {
        ty.total = 0;
        for(int64_t i = 0; i < n; ++i)
            ty.total += soa[(int64_t)(NO - 2) * n + i];
    }
    if(herr)
        return gf_fail(e, GF_ERR_INVALID, "event outside the observable range of a ConvolutionPdf");
    ty.ksort_valid = false;
    if(sorted)
        return buildKSort(e);
    return GF_OK;
}

int gf_set_params(gf_engine *e, int toy, const double *p, int n) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(toy < 0 || toy >= e->n_toys || n != e->tree.n_params || (n > 0 && !p))
        return gf_fail(e, GF_ERR_INVALID, "bad toy index or parameter count");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    std::memcpy(e->h_P + (size_t)toy * n, p, sizeof(double) * n);
    return GF_OK;
}

static int evalOne(gf_engine *e, int toy, bool grad, double *nll, double *g) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(toy < 0 || toy >= e->n_toys)
        return gf_fail(e, GF_ERR_INVALID, "toy index out of range");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    for(int t = 0; t < e->n_toys; ++t)
        e->h_active[t] = (t == toy);
    rc = gf_run(e, grad, -1, 1);
    if(rc)
        return rc;
    const int NGp = 1 + e->tree.NG;
    double *o     = e->h_out + (size_t)toy * (NGp + 2);
    postToy(e, toy, o);
    if(nll)
        *nll = o[0];
    if(grad && g)
        for(int s = 0; s < e->tree.NG; ++s)
            g[s] = o[2 + s];
    int st = statusOf(o[1]);
    if(st == GF_ERR_NAN_NORM)
        return gf_fail(e, st, "NaN in normalization");
    if(st == GF_ERR_NONPOS_NORM)
        return gf_fail(e, st, "non-positive normalization");
    if(st == GF_ERR_ZERO_NLL)
        return gf_fail(e, st, "zero NLL");
    return GF_OK;
}

int gf_nll(gf_engine *e, int toy, double *nll) { return evalOne(e, toy, false, nll, nullptr); }

int gf_nll_grad(gf_engine *e, int toy, double *nll, double *grad) { return evalOne(e, toy, true, nll, grad); }

int gf_num_grad(const gf_engine *e) { return e && e->has_tree ? e->tree.NG : 0; }
int gf_num_params(const gf_engine *e) { return e && e->has_tree ? e->tree.n_params : 0; }
int gf_num_toys(const gf_engine *e) { return e ? e->n_toys : 0; }
int gf_grad_params(const gf_engine *e, int32_t *out, int cap) {
    if(!e || !e->has_tree)
        return 0;
    int n = (int)e->tree.gparam.size();
    for(int s = 0; s < n && s < cap; ++s)
        out[s] = e->tree.gparam[s];
    return n;
}

int gf_nll_batch(gf_engine *e, int n_toys, const double *P, const int32_t *active, double *nll, double *grad) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(n_toys != e->n_toys || !P || !nll)
        return gf_fail(e, GF_ERR_INVALID, "n_toys must equal the engine's toy count");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    const int np = e->tree.n_params, NGp = 1 + e->tree.NG;
    std::memcpy(e->h_P, P, sizeof(double) * (size_t)n_toys * np);
    for(int t = 0; t < n_toys; ++t)
        e->h_active[t] = active ? (active[t] != 0) : 1;
    rc = gf_run(e, grad != nullptr, -1, 1);
    if(rc)
        return rc;
    int worst = GF_OK;
    for(int t = 0; t < n_toys; ++t) {
        if(!e->h_active[t])
            continue;
        double *o = e->h_out + (size_t)t * (NGp + 2);
        postToy(e, t, o);
        nll[t] = o[0];
        if(grad)
            for(int s = 0; s < e->tree.NG; ++s)
                grad[(size_t)t * e->tree.NG + s] = o[2 + s];
        int st = statusOf(o[1]);
        if(st != GF_OK) {
            nll[t] = NAN;
            if(worst == GF_OK)
                worst = st;
        }
    }
    if(worst != GF_OK)
        return gf_fail(e, worst, "a toy had an invalid normalisation or zero NLL (its nll is NaN)");
    return GF_OK;
}

int gf_normalize(gf_engine *e, int toy, double *integral, double *norm) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(toy < 0 || toy >= e->n_toys)
        return gf_fail(e, GF_ERR_INVALID, "toy index out of range");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    const gf::Tree &T = e->tree;
    const int NT = e->n_toys, NQ = (int)T.nums.size(), np = T.n_params;
    for(int t = 0; t < NT; ++t)
        e->h_active[t] = (t == toy);
    if((rc = updateAmpCaches(e)))
        return rc;
    fillRecords(e);
    GfArgs a = makeArgs(e);
    cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
    cudaError_t r = enqueuePrep(e, false, a);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "normalisation kernels");
    std::vector<double> gsum((size_t)NT * std::max(1, NQ));
    if(NQ > 0)
        cudaMemcpyAsync(gsum.data(), e->d_gsum, sizeof(double) * (size_t)NT * NQ, cudaMemcpyDeviceToHost, e->stream);
    cudaMemsetAsync(e->d_qflag, 0, sizeof(int) * NT, e->stream); // zero between evaluations
    r = cudaStreamSynchronize(e->stream);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "normalisation");
    const double *P = e->h_P + (size_t)toy * np;
    const int n     = (int)T.nodes.size();
    std::vector<double> I(n, 1.0), N(n, 1.0);
    // forced nodes keep 1; evaluate children before parents
    std::vector<char> forced(n, 0);
    for(int i = 0; i < n; ++i) {
        const gf::TNode &nd = T.nodes[i];
        bool f = forced[i] || (nd.op == GF_OP_CONVOLUTION) || (nd.op == GF_OP_AMP3BODY) || (nd.op == GF_OP_AMP4BODY) ||
                 (nd.op == GF_OP_PROD && T.nk[i] == gf::NK_NUMERIC);
        for(int c : nd.children)
            forced[c] = forced[c] || f;
    }
    for(int i = n - 1; i >= 0; --i) {
        const gf::TNode &nd = T.nodes[i];
        switch(T.nk[i]) {
        case gf::NK_EXP: {
            const gf_observable &o = T.obs[nd.obs[0]];
            double al = P[nd.params[0]];
            I[i]      = al == 0 ? o.hi - o.lo : (std::exp(al * o.hi) - std::exp(al * o.lo)) / al;
            N[i]      = 1.0 / I[i];
            break;
        }
        case gf::NK_GAUSS: {
            double s = P[nd.params[1]];
            s *= std::sqrt(2.0) * std::sqrt(std::atan2(0.0, -1.0));
            I[i] = s;
            N[i] = 1.0 / s;
            break;
        }
        case gf::NK_AMP3:
        case gf::NK_AMP4: {
            gf::NormLayout::Analytic none;
            none.node = i;
            I[i]      = ampIntegral(e, toy, i, P, none, nullptr);
            N[i]      = 1.0 / I[i];
            break;
        }
        case gf::NK_NUMERIC: {
            const gf::NumInfo &g = T.nums[T.num_of[i]];
            double v = 1;
            v *= g.volume;
            v /= (double)g.total;
            v *= gsum[(size_t)toy * NQ + T.num_of[i]];
            I[i] = v;
            N[i] = 1.0 / v;
            break;
        }
        default:
            N[i] = 1.0;
            if(forced[i])
                I[i] = 1.0;
            else if(nd.op == GF_OP_ADD || nd.op == GF_OP_ADD_EXT) {
                double ret = 0, tw = 0;
                size_t nc  = nd.children.size();
                for(size_t c = 0; c + 1 < nc; ++c) {
                    double w = P[nd.params[c]];
                    tw += w;
                    ret += I[nd.children[c]] * w;
                }
                double last = I[nd.children[nc - 1]];
                if(nd.op == GF_OP_ADD_EXT) {
                    double lw = P[nd.params[nc - 1]];
                    tw += lw;
                    ret += last * lw;
                    ret /= tw;
                } else
                    ret += (1 - tw) * last;
                I[i] = ret;
            } else
                I[i] = 1.0;
        }
    }
    for(int i = 0; i < n; ++i) {
        if(integral)
            integral[i] = I[i];
        if(norm)
            norm[i] = N[i];
    }
    return GF_OK;
}

int gf_eval_events(gf_engine *e, int toy, int node, int metric, double *out, int64_t n_out) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(node != 0)
        return gf_fail(e, GF_ERR_INVALID, "per-event evaluation is defined for the root node; build a tree for a component");
    if(toy < 0 || toy >= e->n_toys || !out)
        return gf_fail(e, GF_ERR_INVALID, "bad arguments");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    GfToy &ty = e->toys[toy];
    if(n_out < ty.n)
        return gf_fail(e, GF_ERR_INVALID, "output array too small");
    if(e->vals_cap < ty.npad) {
        dfree(e->d_vals);
        if(dalloc(e, e->d_vals, (size_t)ty.npad, false))
            return GF_ERR_OOM;
        e->vals_cap = ty.npad;
    }
    const int NT = e->n_toys;
    for(int t = 0; t < NT; ++t)
        e->h_active[t] = (t == toy);
    if((rc = updateAmpCaches(e)))
        return rc;
    fillRecords(e);
    GfArgs a  = makeArgs(e);
    a.metric  = metric;
    cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
    cudaError_t r = enqueuePrep(e, false, a);
    if(r == cudaSuccess)
        r = launch(e->mod.val_n, dim3(evtGrid(e)), dim3(e->block), e->plan.evt_smem_nograd, e->stream, a);
    if(r == cudaSuccess && ty.n > 0)
        r = cudaMemcpyAsync(out, e->d_vals, sizeof(double) * ty.n, cudaMemcpyDeviceToHost, e->stream);
    if(r == cudaSuccess)
        r = cudaMemsetAsync(e->d_qflag, 0, sizeof(int) * NT, e->stream); // zero between evaluations
    if(r == cudaSuccess)
        r = cudaStreamSynchronize(e->stream);
    return gf_cuda_check(e, r, "per-event evaluation");
}

int gf_last_timing(const gf_engine *e, double *ms_total, double *ms_evt) {
    if(!e)
        return GF_ERR_INVALID;
    if(ms_total)
        *ms_total = lastMsTotal(e);
    if(ms_evt)
        *ms_evt = e->last_ms_evt;
    return GF_OK;
}

int gf_time_kernels(gf_engine *e, int toy, int with_grad, double *ms_conv, double *ms_grid, double *ms_event) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(toy < -1 || toy >= e->n_toys)
        return gf_fail(e, GF_ERR_INVALID, "toy index out of range");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    const bool grad = with_grad != 0;
    const gf::Tree &T = e->tree;
    for(int t = 0; t < e->n_toys; ++t)
        e->h_active[t] = (toy < 0 || t == toy);
    if((rc = updateAmpCaches(e)))
        return rc;
    fillRecords(e);
    GfArgs a = makeArgs(e);
    cudaError_t r = cudaMemsetAsync(e->d_qflag, 0, sizeof(int) * e->n_toys, e->stream);
    if(r == cudaSuccess)
        r = cudaMemcpyAsync(e->d_P, e->h_P, e->pblock_bytes, cudaMemcpyHostToDevice, e->stream);
    cudaEvent_t t0 = e->ev[0], t1 = e->ev[1], t2 = e->ev[2], t3 = e->ev[3];
    if(r == cudaSuccess)
        r = cudaEventRecord(t0, e->stream);
    if(r == cudaSuccess && !T.convs.empty())
        r = launch(grad ? e->mod.conv_g : e->mod.conv_n, dim3(e->plan.conv_blocks, e->n_toys, (unsigned)T.convs.size()),
                   dim3(e->block), grad ? e->plan.conv_smem_grad : e->plan.conv_smem_nograd, e->stream, a);
    if(r == cudaSuccess)
        r = cudaEventRecord(t1, e->stream);
    if(r == cudaSuccess && !T.nums.empty() && gridWork(e))
        r = launch(grad ? e->mod.grid_g : e->mod.grid_n, dim3(e->plan.max_grid_blocks, e->n_toys, (unsigned)T.nums.size()),
                   dim3(e->block), 0, e->stream, a);
    if(r == cudaSuccess)
        r = cudaEventRecord(t2, e->stream);
    if(r == cudaSuccess)
        r = launch(grad ? evtGradKernel(e) : e->mod.evt_n, dim3(evtGrid(e)), dim3(e->block),
                   grad ? evtGradSmem(e) : e->plan.evt_smem_nograd, e->stream, a);
    if(r == cudaSuccess)
        r = cudaEventRecord(t3, e->stream);
    if(r == cudaSuccess)
        r = cudaStreamSynchronize(e->stream);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "kernel timing");
    float f = 0;
    if(ms_conv)
        *ms_conv = cudaEventElapsedTime(&f, t0, t1) == cudaSuccess ? f : 0.0;
    if(ms_grid)
        *ms_grid = cudaEventElapsedTime(&f, t1, t2) == cudaSuccess ? f : 0.0;
    if(ms_event)
        *ms_event = cudaEventElapsedTime(&f, t2, t3) == cudaSuccess ? f : 0.0;
    return GF_OK;
}

int64_t gf_event_chunk(const gf_engine *e) { return e && e->layout_ready ? e->chunk : 0; }

int gf_set_wait_limit(gf_engine *e, uint64_t ns) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    e->bar_ns = ns ? ns : 1000000000ull;
    return GF_OK;
}

int gf_set_gram_wait_limit(gf_engine *e, uint64_t ns) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    e->gram_ns = ns;
    return GF_OK;
}

// ---- launch-shape autotuner ----
namespace {

// Device time of one gradient evaluation of every toy (the engine's CUDA events around it), after a write of
// twice the L2 size; the best of `reps` after one untimed evaluation.
int timeEval(gf_engine *e, void *flush, size_t flushBytes, int reps, double *best) {
    *best = 1e30;
    for(int it = 0; it <= reps; ++it) {
        if(flush && cudaMemsetAsync(flush, it & 0xff, flushBytes, e->stream) != cudaSuccess)
            return gf_cuda_check(e, cudaGetLastError(), "autotune flush");
        for(int t = 0; t < e->n_toys; ++t)
            e->h_active[t] = 1;
        if(int rc = gf_run(e, true, -1, 1))
            return rc;
        if(it > 0)
            *best = std::min(*best, lastMsTotal(e));
    }
    return GF_OK;
}

// Recompiles the tree with the given shapes and rebuilds the layout, keeping the parameters, the active flags
// and the event chunk.
int applyShapes(gf_engine *e, const gf::Shapes &sh, const std::vector<double> &P, const std::vector<int> &act) {
    const int chunk = e->chunk;
    const bool fixed = e->chunk_fixed;
    e->shapes = sh;
    if(int rc = compileTree(e))
        return rc;
    e->layout_ready = false;
    e->chunk_fixed  = true;
    e->chunk        = chunk;
    int rc          = buildLayout(e);
    e->chunk_fixed  = fixed;
    if(rc)
        return rc;
    std::memcpy(e->h_P, P.data(), sizeof(double) * P.size());
    for(int t = 0; t < e->n_toys; ++t)
        e->h_active[t] = act[t];
    return GF_OK;
}

struct TunedShapes {
    gf::Shapes sh;
    int gram_w = 0;
};

} // namespace

int gf_tune_shapes(gf_engine *e) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    static std::mutex mu;
    static std::map<std::string, TunedShapes> cache;
    int64_t total = 0;
    for(auto &t : e->toys)
        total += t.n;
    const gf::Tree &T = e->tree;
    const int np      = std::max(1, T.n_params);
    std::vector<double> P(e->h_P, e->h_P + (size_t)e->n_toys * np);
    std::vector<int> act(e->h_active, e->h_active + e->n_toys);
    const std::string key = std::to_string(std::hash<std::string>{}(
                                gf::generate_kernels(T, e->precision == GF_MIXED, e->block, e->batch_kernels).source)) +
                            ":" + std::to_string(e->precision) + ":" + std::to_string(e->n_toys) + ":" +
                            std::to_string(total) + ":" + std::to_string(e->amp_recompute ? 1 : 0);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if(it != cache.end()) {
            e->gram_w = it->second.gram_w;
            if(it->second.sh.conv_kp == e->plan.conv_kp && it->second.sh.grid_bpb == e->plan.grid_bins_per_block)
                return GF_OK;
            return applyShapes(e, it->second.sh, P, act);
        }
    }
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, e->device);
    const size_t flushBytes = (size_t)std::max(l2, 1 << 20) * 2;
    void *flush             = nullptr;
    if(cudaMalloc(&flush, flushBytes) != cudaSuccess) {
        cudaGetLastError();
        flush = nullptr;
    }
    struct Free {
        void *p;
        ~Free() {
            if(p)
                cudaFree(p);
        }
    } guard{flush};
    // candidates: table k-tiles (batches with convolutions), then grid bins per CTA (grids not folded into a
    // table), each with the best of the other; the chunk stays as it is while they are compared
    gf::Shapes best{e->plan.conv_kp, e->plan.grid_bins_per_block};
    double bestMs = 1e30;
    if((rc = timeEval(e, flush, flushBytes, 5, &bestMs)))
        return rc;
    auto tryShape = [&](gf::Shapes sh) -> int {
        if(sh.conv_kp == best.conv_kp && sh.grid_bpb == best.grid_bpb)
            return GF_OK;
        if(int r2 = applyShapes(e, sh, P, act))
            return r2;
        double ms = 0;
        if(int r2 = timeEval(e, flush, flushBytes, 5, &ms))
            return r2;
        if(ms < bestMs) {
            bestMs = ms;
            best   = sh;
        }
        return GF_OK;
    };
    if(e->batch_kernels && !T.convs.empty())
        for(int kp : {1, 2, 4, 8})
            if((rc = tryShape(gf::Shapes{kp, best.grid_bpb})))
                return rc;
    bool unfolded = false;
    for(size_t q = 0; q < T.nums.size(); ++q)
        unfolded = unfolded || !e->plan.num_folded[q];
    if(unfolded)
        for(int bpb : {128, 256, 512, 1024, 2048})
            if((rc = tryShape(gf::Shapes{best.conv_kp, bpb})))
                return rc;
    if(e->shapes.conv_kp != best.conv_kp || e->shapes.grid_bpb != best.grid_bpb ||
       e->plan.conv_kp != best.conv_kp || e->plan.grid_bins_per_block != best.grid_bpb)
        if((rc = applyShapes(e, best, P, act)))
            return rc;
    // tensor-core Gram slice width: the integral rebuild timed at every width the widest node allows
    int bestW = 0;
    if(e->gram_tc && !e->amp_recompute && T.n_amp_nodes() > 0) {
        int wmin = 16;
        for(int k = 0; k < T.n_amp_nodes(); ++k)
            wmin = std::max(wmin, gf_gram_tc_width(ampColumns(T, k)));
        double bestG = 1e30;
        for(int w : {16, 32, 64}) {
            if(w < wmin)
                continue;
            e->gram_w = w;
            double mn = 1e30;
            for(int it = 0; it < 4; ++it) {
                for(auto &ty : e->toys)
                    ty.norm_valid = false;
                if(flush)
                    cudaMemsetAsync(flush, it & 0xff, flushBytes, e->stream);
                cudaStreamSynchronize(e->stream);
                const auto t0 = std::chrono::steady_clock::now();
                if((rc = updateAmpCaches(e)))
                    return rc;
                const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                if(it > 0)
                    mn = std::min(mn, ms);
            }
            if(mn < bestG) {
                bestG = mn;
                bestW = w;
            }
        }
        e->gram_w = bestW;
        for(auto &ty : e->toys)
            ty.norm_valid = false;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = TunedShapes{best, bestW};
    }
    return GF_OK;
}

int gf_get_shapes(const gf_engine *e, int32_t *conv_kp, int32_t *grid_bpb, int32_t *gram_w) {
    if(!e || !e->has_tree)
        return gf_fail(nullptr, GF_ERR_STATE, "no tree");
    if(conv_kp)
        *conv_kp = e->plan.conv_kp;
    if(grid_bpb)
        *grid_bpb = e->plan.grid_bins_per_block;
    if(gram_w) {
        int w = 0;
        for(int k = 0; k < e->tree.n_amp_nodes(); ++k)
            w = std::max(w, gf_gram_tc_width(ampColumns(e->tree, k)));
        *gram_w = e->gram_tc ? std::max(e->gram_w, w) : 0;
    }
    return GF_OK;
}

int gf_set_amp_mode(gf_engine *e, int mode, int64_t budget_bytes) {
    if(!e)
        return gf_fail(nullptr, GF_ERR_INVALID, "null engine");
    if(mode < GF_AMP_AUTO || mode > GF_AMP_RECOMPUTE || budget_bytes < 0)
        return gf_fail(e, GF_ERR_INVALID, "amplitude mode: GF_AMP_AUTO, GF_AMP_STORE or GF_AMP_RECOMPUTE, budget >= 0");
    for(auto &t : e->toys)
        if(t.loaded)
            return gf_fail(e, GF_ERR_STATE, "gf_set_amp_mode must come before gf_upload_events");
    e->amp_mode    = mode;
    e->amp_budget  = budget_bytes;
    e->amp_decided = false;
    return GF_OK;
}

int64_t gf_amp_store_bytes(const gf_engine *e) {
    if(!e || !e->has_tree || e->tree.n_amp_nodes() == 0 || e->toys.empty() || !e->toys[0].loaded)
        return 0;
    return (int64_t)ampStoreBytes(e, e->toys[0].npad);
}

int gf_amp_recomputing(const gf_engine *e) {
    if(!e)
        return -1;
    return e->amp_decided ? (e->amp_recompute ? 1 : 0) : -1;
}

int gf_launches_per_eval(const gf_engine *e, int) {
    if(!e || !e->has_tree)
        return 0;
    if(fusedPath(e))
        return 1;
    return 1 + (e->tree.convs.empty() ? 0 : 1) + (e->tree.nums.empty() || !gridWork(e) ? 0 : 1);
}

int gf_set_norm_events(gf_engine *e, int node, const double *soa5, int64_t n) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(node < 0 || node >= (int)e->tree.nodes.size() || e->tree.amp4_of[node] < 0)
        return gf_fail(e, GF_ERR_INVALID, "not an Amp4Body node");
    if(n <= 0 || !soa5)
        return gf_fail(e, GF_ERR_INVALID, "normalisation events: n must be positive");
    cudaSetDevice(e->device);
    const int k = e->tree.amp4_of[node];
    dfree(e->norm_buf[k]);
    e->norm_n[k] = 0;
    int rc = dalloc(e, e->norm_buf[k], (size_t)5 * n, false);
    if(rc)
        return rc;
    cudaError_t r = cudaMemcpy(e->norm_buf[k], soa5, sizeof(double) * 5 * (size_t)n, cudaMemcpyHostToDevice);
    const long long nn = n;
    if(r == cudaSuccess)
        r = cudaMemcpy(e->d_nevt + k, &e->norm_buf[k], sizeof(double *), cudaMemcpyHostToDevice);
    if(r == cudaSuccess)
        r = cudaMemcpy(e->d_nnorm + k, &nn, sizeof(long long), cudaMemcpyHostToDevice);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "normalisation events");
    e->norm_n[k] = n;
    for(auto &ty : e->toys)
        ty.norm_valid = false;
    return GF_OK;
}

static int ampNode(gf_engine *e, int toy, int node, int *ai) {
    if(!e || !e->has_tree)
        return gf_fail(e, GF_ERR_STATE, "no tree");
    if(toy < 0 || toy >= e->n_toys || node < 0 || node >= (int)e->tree.nodes.size() || e->tree.amp_index(node) < 0)
        return gf_fail(e, GF_ERR_INVALID, "not an Amp3Body or Amp4Body node, or toy index out of range");
    cudaSetDevice(e->device);
    int rc = buildLayout(e);
    if(rc)
        return rc;
    for(int t = 0; t < e->n_toys; ++t)
        e->h_active[t] = (t == toy);
    *ai = e->tree.amp_index(node);
    return updateAmpCaches(e);
}

int gf_amp3_integrals(gf_engine *e, int toy, int node, double *out, int cap) {
    int ai = -1, rc = ampNode(e, toy, node, &ai);
    if(rc)
        return rc;
    const std::vector<double> &I = e->toys[toy].amp_I[ai];
    if(!out || cap < (int)I.size())
        return gf_fail(e, GF_ERR_INVALID, "output holds fewer than 2 n^2 values");
    std::memcpy(out, I.data(), sizeof(double) * I.size());
    return GF_OK;
}

int gf_amp3_cached_wave(gf_engine *e, int toy, int node, int res, double *out, int64_t n_out) {
    int ai = -1, rc = ampNode(e, toy, node, &ai);
    if(rc)
        return rc;
    GfToy &ty = e->toys[toy];
    if(res < 0 || res >= e->tree.amp_count(ai) || !out || n_out < ty.n)
        return gf_fail(e, GF_ERR_INVALID, "bad resonance index or output size");
    const size_t rs = rsize(e);
    std::vector<char> buf((size_t)std::max<int64_t>(1, ty.n) * 2 * rs);
    cudaError_t r = cudaSuccess;
    if(ty.n > 0)
        r = cudaMemcpyAsync(buf.data(), ty.acols[e->tree.amp_col0(ai) + res], (size_t)ty.n * 2 * rs,
                            cudaMemcpyDeviceToHost, e->stream);
    if(r == cudaSuccess)
        r = cudaStreamSynchronize(e->stream);
    if(r != cudaSuccess)
        return gf_cuda_check(e, r, "reading the amplitude cache");
    for(int64_t i = 0; i < 2 * ty.n; ++i)
        out[i] = rs == 4 ? (double)reinterpret_cast<const float *>(buf.data())[i]
                         : reinterpret_cast<const double *>(buf.data())[i];
    return GF_OK;
}

int gf_generated_source(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                        const int32_t *grad_mask, int precision, char *buf, int64_t cap, int64_t *len) {
    gf::Tree t;
    std::string why = t.build(nodes, n_nodes, obs, n_obs, n_params, grad_mask);
    if(!why.empty())
        return gf_fail(nullptr, GF_ERR_BAD_TREE, why);
    gf::KernelPlan p;
    try {
        p = gf::generate_kernels(t, precision == GF_MIXED, 256, false);
    } catch(std::exception &ex) {
        return gf_fail(nullptr, GF_ERR_BAD_TREE, ex.what());
    }
    if(len)
        *len = (int64_t)p.source.size();
    if(buf && cap > 0) {
        int64_t m = std::min<int64_t>(cap - 1, (int64_t)p.source.size());
        std::memcpy(buf, p.source.data(), (size_t)m);
        buf[m] = 0;
    }
    return GF_OK;
}

static int compileTreeShaped(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                             const int32_t *grad_mask, int precision, bool batch, int64_t *cubin_bytes) {
    gf::Tree t;
    std::string why = t.build(nodes, n_nodes, obs, n_obs, n_params, grad_mask);
    if(!why.empty())
        return gf_fail(nullptr, GF_ERR_BAD_TREE, why);
    gf::KernelPlan p;
    try {
        p = gf::generate_kernels(t, precision == GF_MIXED, 256, batch);
    } catch(std::exception &ex) {
        return gf_fail(nullptr, GF_ERR_BAD_TREE, ex.what());
    }
    std::vector<char> cubin;
    std::string log;
    if(!gf::rtc_compile(p.source, "sm_103a", cubin, log))
        return gf_fail(nullptr, GF_ERR_COMPILE, log);
    if(cubin_bytes)
        *cubin_bytes = (int64_t)cubin.size();
    return GF_OK;
}

int gf_compile_tree(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                    const int32_t *grad_mask, int precision, int64_t *cubin_bytes) {
    return compileTreeShaped(nodes, n_nodes, obs, n_obs, n_params, grad_mask, precision, false, cubin_bytes);
}

int gf_compile_tree_batch(const gf_node *nodes, int n_nodes, const gf_observable *obs, int n_obs, int n_params,
                          const int32_t *grad_mask, int precision, int64_t *cubin_bytes) {
    return compileTreeShaped(nodes, n_nodes, obs, n_obs, n_params, grad_mask, precision, true, cubin_bytes);
}

} // extern "C"
