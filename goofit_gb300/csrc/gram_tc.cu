// Normalisation-integral Gram matrix on the 5th-generation tensor cores (tcgen05.mma, kind::tf32).
//
// Replaces the per-entry reductions of the reference's normalisation integrals
// (src/PDFs/physics/detail/SpecialResonanceIntegrator.cu:52-121 for Amp3Body, one launch per resonance pair;
// src/PDFs/physics/detail/NormIntegrator.cu:15-68 for Amp4Body, every FCN) by one contraction over the
// normalisation points.  The amplitudes of the points are complex FP32 columns X_c (c < C) in HBM, written
// by the generated gf_ampn kernel, optionally with an efficiency column e.  With x_r the 2C real columns
// (Re X_0, Im X_0, Re X_1, ...) the kernel computes the real Gram matrix
//     G_rs = sum_p x_r(p) e(p) x_s(p),
// from which the host forms I_ab = sum_p X_a conj(X_b) e and the derivative rows H.
//
// Tensor-core mapping.  One MMA is D[128 x 128] += A[128 x 8] B[128 x 8]^T with both operands K-major in
// shared memory and the point index as K.  The 128 rows are S = 128 / W slices of W >= 2C real columns,
// each slice a different range of points, so the W x W diagonal blocks of D are the slices' Gram matrices
// (the off-diagonal blocks are products of unrelated points and are never read).  FP32 operands are split
// into TF32 pairs, x = hi + lo, and each product takes three MMAs (hi.hi + hi.lo + lo.hi): about 22
// significant bits per product.  The tensor core's FP32 accumulation rounds towards zero, so the large
// hi.hi products never accumulate over more than one stage (32 points per slice): they go into one of two
// tensor-memory accumulators by stage parity, and the threads read the previous stage's accumulator back
// (tcgen05.ld) into compensated FP32 registers while the tensor core works on the current stage.  The
// cross terms hi.lo + lo.hi, 2^-11 smaller, accumulate in a third accumulator over the CTA's points.  The
// CTAs' partials are summed in FP64 by gf_gram_tc_sum.
//
// Pipeline per CTA (512 threads for 16-column slices, else 256; one elected thread issues the MMAs): cp.async
// 16-byte copies fill a three-slot ring of raw (unsplit) stages two stages ahead; the threads split the oldest raw
// stage and store it into one of two operand stages in the canonical no-swizzle K-major layout while the tensor
// core works on the other; tcgen05.commit arrives on the operand stage's mbarrier when its MMAs have read it.  Every wait is bounded: a wait that runs out sets *err and the CTA stops issuing work,
// waits (bounded) for what it issued, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"

namespace {

// Threads per CTA: warps 0-3 read tensor-memory lanes 32w .. 32w + 31 (the D rows); all warps copy and split the
// stages.  W = 16 (2 W compensated registers per drain thread) takes 16 warps, which halves each stage's copy and
// split work per warp and gives the single CTA per SM more warps to cover latencies; wider slices keep 8 warps
// (their drain registers do not fit the 128 per thread of a 512-thread CTA).
template <int W>
__host__ __device__ constexpr int threadsFor() { return W == 16 ? 512 : 256; }
constexpr int kRows    = 128; // MMA M = N = 128 rows: S slices x W real columns
constexpr int kKS      = 32;  // points of one slice per stage: four MMA K-steps of 8 (kind::tf32)
constexpr int kOpBytes = kRows * kKS * 4;   // one operand split of one stage: 16 KB
constexpr uint32_t kLBO = 128;              // byte stride between 16-byte K chunks (core matrices along K)
constexpr uint32_t kSBO = (kKS / 4) * 128;  // byte stride between 8-row groups
constexpr uint32_t kColBig   = 128;         // tensor-memory columns: two 128-column accumulators of the
constexpr uint32_t kColSmall = 256;         // hi.hi products (one per stage parity), one of the cross terms
constexpr uint32_t kTmemCols = 512;         // allocation (a power of two): one CTA per SM
constexpr int kOperandBytes  = 2 * 4 * kOpBytes;  // two stages of A_hi, A_lo, B_hi, B_lo: 128 KB
constexpr int kRawSlots      = 3;                 // raw stages: two in flight while one is transformed
constexpr int kRawRow        = kKS * 8 + 16;      // one (slice, column) row of a raw stage: 32 float2 + pad
constexpr int kRawCplx       = 64 * kRawRow;      // at most S x C = 64 rows
constexpr int kRawSlot       = kRawCplx + 8 * kKS * 4; // + the efficiency of S <= 8 slices
constexpr int kSmemBytes     = kOperandBytes + kRawSlots * kRawSlot;
// 2 s: the default limit of a per-stage mbarrier wait, and always the limit of the wait for the last committed
// MMAs before the tensor memory is freed (that wait must not give up while MMAs may still write it)
constexpr unsigned long long kWaitNs = 2000000000ull;

// Instruction descriptor of tcgen05.mma kind::tf32: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kRows >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 (bits 0-13), leading byte offset >> 4
// (bits 16-29), stride byte offset >> 4 (bits 32-45), descriptor version 1 (bits 46-47), base offset 0,
// no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Byte offset of element (row r, point k) of one operand split in the canonical no-swizzle K-major layout:
// 8-row x 16-byte core matrices of 128 contiguous bytes, K chunks kLBO apart, row groups kSBO apart.
__device__ __forceinline__ uint32_t op_off(int r, int k) {
    return (uint32_t)(r >> 3) * kSBO + (uint32_t)(k >> 2) * kLBO + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

// x rounded to TF32 (11 significant bits, ties away from zero) by integer operations; x - tf32_hi(x) is
// exact in FP32 and at most half a TF32 unit, and the tensor core reads it truncated to TF32 (~22 bits in all)
__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u); }

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

// Waits until phase `parity` of the mbarrier has completed; false after `limit` ns of the global timer.  Each
// try_wait suspends the thread for at most min(limit, 1 ms) (its suspend-time hint), so that a short limit is
// checked within about that time instead of the hardware's own suspension limit.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, unsigned long long limit) {
    const unsigned long long t0 = globaltimer();
    const uint32_t hint         = limit < 1000000ull ? (uint32_t)limit : 1000000u;
    while(true) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(addr), "r"(parity), "r"(hint)
                     : "memory");
        if(done)
            return true;
        if(globaltimer() - t0 > limit)
            return false;
    }
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
                 "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// asynchronous global -> shared copies (cp.async); a source size of 0 writes zeros
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// h + l += v, the rounding error of the sum kept in l
__device__ __forceinline__ void two_sum_add(float &h, float &l, float v) {
    const float s  = h + v;
    const float bp = s - h;
    l += (h - (s - bp)) + (v - bp);
    h = s;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for(int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}

// W real columns per slice (2C <= W), S = 128 / W slices.  eff != nullptr: the efficiency multiplies B.
// Columns sc[c * nst + p], nst a multiple of 4; sc and eff 16-byte aligned.
template <int W>
__global__ void __launch_bounds__(threadsFor<W>(), 1)
    gf_gram_tc(const float2 *__restrict__ sc, long long npts, long long nst, int ncol, const float *__restrict__ eff,
               long long per_cta, double *__restrict__ part, int *__restrict__ err, unsigned long long wait_ns,
               int stall) {
    constexpr int S  = kRows / W;
    constexpr int kThreads = threadsFor<W>();
    constexpr int KC = kKS / 4; // 16-byte chunks of 4 points per row and stage
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ __align__(8) unsigned long long mbar_never; // no thread or copy ever arrives on it
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool weighted = eff != nullptr;
    const int nops      = weighted ? 4 : 2; // A_hi, A_lo [, B_hi, B_lo]
    const long long b0  = (long long)blockIdx.x * per_cta;
    const long long L   = per_cta / S;      // points per slice
    const int T         = (int)(L / kKS);   // stages

    // zero both operand stages once: rows beyond 2C of every slice stay zero
    for(int i = tid; i < kOperandBytes / 16; i += kThreads)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    if(tid == 0) {
        mbar_init(smem_u32(&mbar[0]), 1);
        mbar_init(smem_u32(&mbar[1]), 1);
        mbar_init(smem_u32(&mbar_never), 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    // warps 0-3: this thread's D row and its slice; compensated FP32 sums of the drained stage blocks
    const int row = 32 * (warp & 3) + lane, slice = row / W;
    float acc_h[W], acc_l[W];
#pragma unroll
    for(int j = 0; j < W; ++j)
        acc_h[j] = acc_l[j] = 0.f;
    const uint32_t lanebase = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    int issued_last         = -1; // last stage whose MMAs were committed

    // adds the W x W block of this thread's slice from tensor-memory columns col0 .. col0 + 127 (warps 0-3)
    auto drain = [&](uint32_t col0) {
        if(warp >= 4)
            return;
        float v[16];
        if(W == 16) {
            // warp w holds slices 2w (lanes 0-15) and 2w + 1 (lanes 16-31)
            float v2[16];
            tmem_ld16(lanebase + col0 + (uint32_t)(32 * warp), v);
            tmem_ld16(lanebase + col0 + (uint32_t)(32 * warp + 16), v2);
#pragma unroll
            for(int j = 0; j < 16; ++j)
                two_sum_add(acc_h[j], acc_l[j], lane < 16 ? v[j] : v2[j]);
        } else {
#pragma unroll
            for(int q = 0; q < W / 16; ++q) {
                tmem_ld16(lanebase + col0 + (uint32_t)(slice * W + 16 * q), v);
#pragma unroll
                for(int j = 0; j < 16; ++j)
                    two_sum_add(acc_h[16 * q + j], acc_l[16 * q + j], v[j]);
            }
        }
    };
    // waits for stage u's MMAs (and so for every earlier one); false on every thread if any wait ran out
    // stall = u (a test of the failure path, -1 otherwise): stage u's wait also waits for a barrier that never
    // completes, so that it runs out after wait_ns while the stage's MMAs complete normally
    auto stage_done = [&](int u) -> bool {
        bool ok = mbar_wait(smem_u32(&mbar[u & 1]), (uint32_t)((u >> 1) & 1), wait_ns);
        if(u == stall)
            ok = ok && mbar_wait(smem_u32(&mbar_never), 0u, wait_ns);
        return !__syncthreads_or(!ok);
    };

    // raw stage ring after the operand stages: per (slice, column) a row of 32 points (float2), padded so
    // that rows of consecutive columns fall in different banks, then the efficiency of each slice
    unsigned char *rawbase = smem + kOperandBytes;
    const int nrow         = S * ncol;
    auto copy_stage = [&](int t) {
        unsigned char *slot = rawbase + (size_t)(t % kRawSlots) * kRawSlot;
        // 16-byte copies of 2 points; consecutive threads take consecutive chunks of one column
        for(int j = tid; j < nrow * (kKS / 2); j += kThreads) {
            const int rr = j / (kKS / 2), h = j % (kKS / 2);
            const int s = rr / ncol, c = rr % ncol;
            const long long p = b0 + (long long)s * L + (long long)t * kKS + 2 * h;
            const long long n = p < npts ? (npts - p < 2 ? npts - p : 2) : 0;
            cp_async16(smem_u32(slot + rr * kRawRow + h * 16), n > 0 ? (const void *)(sc + (long long)c * nst + p) : (const void *)sc,
                       (uint32_t)(8 * n));
        }
        if(weighted)
            for(int j = tid; j < S * KC; j += kThreads) {
                const int s = j / KC, h = j % KC;
                const long long p = b0 + (long long)s * L + (long long)t * kKS + 4 * h;
                const long long n = p < npts ? (npts - p < 4 ? npts - p : 4) : 0;
                cp_async16(smem_u32(slot + kRawCplx + (s * kKS + 4 * h) * 4), n > 0 ? (const void *)(eff + p) : (const void *)eff,
                           (uint32_t)(4 * n));
            }
        cp_async_commit();
    };
    for(int t = 0; t < kRawSlots - 1; ++t) {
        if(t < T)
            copy_stage(t);
        else
            cp_async_commit();
    }

    for(int t = 0; t < T; ++t) {
        const int buf     = t & 1;
        unsigned char *st = smem + (size_t)buf * nops * kOpBytes;
        // keep kRawSlots - 1 stages of loads in flight (the slot written now was last read in stage t - 1,
        // before that stage's barrier); after the wait and the barrier stage t's raw data is complete
        if(t + kRawSlots - 1 < T)
            copy_stage(t + kRawSlots - 1);
        else
            cp_async_commit();
        cp_async_wait<kRawSlots - 1>();
        // the MMAs of stage t - 2 have read this operand buffer (waited for already by the drain of t - 1)
        if(t >= 2 && !mbar_wait(smem_u32(&mbar[buf]), (uint32_t)(((t - 2) >> 1) & 1), wait_ns))
            s_fail = 1;
        __syncthreads();
        // one task = one real row x 4 points: 8 consecutive lanes write the 8 rows of one core matrix
        const unsigned char *slot = rawbase + (size_t)(t % kRawSlots) * kRawSlot;
        for(int u = warp; u < 2 * (kRows / 8); u += kThreads / 32) {
            const int r = 8 * (u >> 1) + (lane & 7), kc = 4 * (u & 1) + (lane >> 3);
            const int s = r / W, i = r % W, c = i >> 1;
            if(c >= ncol)
                continue;
            const float4 *src = reinterpret_cast<const float4 *>(slot + (s * ncol + c) * kRawRow + kc * 32);
            const float4 q0 = src[0], q1 = src[1]; // (x0, y0, x1, y1), (x2, y2, x3, y3)
            const float4 v  = (i & 1) ? make_float4(q0.y, q0.w, q1.y, q1.w) : make_float4(q0.x, q0.z, q1.x, q1.z);
            float4 h, l;
            h.x = tf32_hi(v.x); h.y = tf32_hi(v.y); h.z = tf32_hi(v.z); h.w = tf32_hi(v.w);
            l.x = v.x - h.x; l.y = v.y - h.y; l.z = v.z - h.z; l.w = v.w - h.w;
            const uint32_t o = op_off(r, 4 * kc);
            *reinterpret_cast<float4 *>(st + o)            = h;
            *reinterpret_cast<float4 *>(st + kOpBytes + o) = l;
            if(weighted) {
                const float4 e = *reinterpret_cast<const float4 *>(slot + kRawCplx + (s * kKS + 4 * kc) * 4);
                const float4 b = make_float4(v.x * e.x, v.y * e.y, v.z * e.z, v.w * e.w);
                h.x = tf32_hi(b.x); h.y = tf32_hi(b.y); h.z = tf32_hi(b.z); h.w = tf32_hi(b.w);
                l.x = b.x - h.x; l.y = b.y - h.y; l.z = b.z - h.z; l.w = b.w - h.w;
                *reinterpret_cast<float4 *>(st + 2 * kOpBytes + o) = h;
                *reinterpret_cast<float4 *>(st + 3 * kOpBytes + o) = l;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        if(s_fail)
            break;
        tc_fence_after();
        if(tid == 0) {
            // hi.hi into this stage's accumulator (fresh each stage: at most 4 FP32 accumulations of the
            // large products), hi.lo + lo.hi into the small-term accumulator for the whole CTA
            const uint32_t ah = smem_u32(st), al = ah + kOpBytes;
            const uint32_t bh = weighted ? ah + 2 * kOpBytes : ah, bl = weighted ? ah + 3 * kOpBytes : al;
            const uint32_t dbig = tmem + kColBig * (uint32_t)buf, dsmall = tmem + kColSmall;
#pragma unroll
            for(int ks = 0; ks < kKS / 8; ++ks) {
                const uint32_t o = (uint32_t)ks * 2 * kLBO; // 8 points = two 16-byte K chunks
                mma_tf32(dbig, smem_desc(ah + o), smem_desc(bh + o), ks > 0 ? 1u : 0u);
            }
#pragma unroll
            for(int ks = 0; ks < kKS / 8; ++ks) {
                const uint32_t o = (uint32_t)ks * 2 * kLBO;
                mma_tf32(dsmall, smem_desc(ah + o), smem_desc(bl + o), (t > 0 || ks > 0) ? 1u : 0u);
                mma_tf32(dsmall, smem_desc(al + o), smem_desc(bh + o), 1u);
            }
            mma_commit(smem_u32(&mbar[buf]));
        }
        issued_last = t;
        // drain the previous stage's accumulator while the tensor core works on this one
        if(t >= 1) {
            if(!stage_done(t - 1)) {
                if(tid == 0)
                    s_fail = 1;
                break;
            }
            tc_fence_after();
            drain(kColBig * (uint32_t)((t - 1) & 1));
            tc_fence_before();
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    if(!s_fail && T > 0) {
        if(stage_done(T - 1)) {
            tc_fence_after();
            drain(kColBig * (uint32_t)((T - 1) & 1));
            drain(kColSmall);
        } else if(tid == 0)
            s_fail = 1;
    }
    __syncthreads();
    const bool failed = s_fail != 0;
    if(failed) {
        if(tid == 0)
            atomicOr(err, 1);
        // wait (bounded) for the last committed stage before the tensor memory goes away
        if(issued_last >= 0)
            mbar_wait(smem_u32(&mbar[issued_last & 1]), (uint32_t)((issued_last >> 1) & 1), kWaitNs);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if(warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    if(failed)
        return;

    // sum the S slices' blocks in shared memory (the operand stages are free now), FP64
    double *red = reinterpret_cast<double *>(smem);
    if(warp < 4) {
#pragma unroll
        for(int j = 0; j < W; ++j)
            red[(size_t)row * W + j] = (double)acc_h[j] + (double)acc_l[j];
    }
    __syncthreads();
    const int m = 2 * ncol;
    double *out = part + (long long)blockIdx.x * m * m;
    for(int q = tid; q < m * m; q += kThreads) {
        const int i = q / m, j = q % m;
        double s = 0.0;
        for(int sl = 0; sl < S; ++sl)
            s += red[(size_t)(sl * W + i) * W + j];
        out[q] = s;
    }
}

// out[q] = sum over the CTAs' partials of entry q: one 128-thread CTA per entry, FP64
__global__ void __launch_bounds__(128) gf_gram_tc_sum(const double *__restrict__ part, int nblk, int nent,
                                                      double *__restrict__ out) {
    __shared__ double red[4];
    const int q = blockIdx.x, tid = threadIdx.x;
    double s = 0.0;
    for(int b = tid; b < nblk; b += 128)
        s += part[(long long)b * nent + q];
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if((tid & 31) == 0)
        red[tid >> 5] = s;
    __syncthreads();
    if(tid == 0)
        out[q] = (red[0] + red[1]) + (red[2] + red[3]);
}

template <int W>
cudaError_t launchW(const float2 *sc, long long npts, long long nst, int ncol, const float *eff, int grid,
                    long long per_cta, double *part, int *err, unsigned long long wait_ns, int stall, cudaStream_t s) {
    // per launch: the attribute belongs to the current device, and the kernel runs once per cache rebuild
    cudaError_t r = cudaFuncSetAttribute(gf_gram_tc<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if(r != cudaSuccess)
        return r;
    // every launch requests the full size: one CTA per SM, so the 512-column allocation never waits
    gf_gram_tc<W><<<grid, threadsFor<W>(), kSmemBytes, s>>>(sc, npts, nst, ncol, eff, per_cta, part, err, wait_ns, stall);
    return cudaGetLastError();
}

} // namespace

int gf_gram_tc_width(int ncol) {
    const int r = 2 * ncol;
    return r <= 16 ? 16 : r <= 32 ? 32 : r <= 64 ? 64 : 0;
}

size_t gf_gram_tc_part_doubles(int ncol, int grid) { return (size_t)grid * 4 * ncol * ncol; }

cudaError_t gf_gram_tc_launch(const float2 *sc, long long npts, long long nst, int ncol, const float *eff,
                              int sm_count, double *part, double *out, int *err, cudaStream_t s, int width,
                              unsigned long long wait_ns, int stall) {
    if(wait_ns == 0)
        wait_ns = kWaitNs;
    const int Wmin = gf_gram_tc_width(ncol);
    const int W    = width == 0 ? Wmin : width;
    if(Wmin == 0 || W < Wmin || (W != 16 && W != 32 && W != 64) || ncol < 1 || npts <= 0 || nst < npts ||
       nst % 4 != 0 || ((uintptr_t)sc & 15) != 0 ||
       (eff && ((uintptr_t)eff & 15) != 0))
        return cudaErrorInvalidValue;
    const long long unit = (long long)(kRows / W) * kKS; // points per stage
    long long per_cta    = (npts + sm_count - 1) / sm_count;
    per_cta              = (per_cta + unit - 1) / unit * unit;
    const int grid       = (int)((npts + per_cta - 1) / per_cta);
    static_assert((size_t)kRows * 64 * 8 <= (size_t)kOperandBytes, "slice reduction does not fit");
    static_assert(kSmemBytes <= 227 * 1024, "shared memory");
    cudaError_t r = W == 16   ? launchW<16>(sc, npts, nst, ncol, eff, grid, per_cta, part, err, wait_ns, stall, s)
                    : W == 32 ? launchW<32>(sc, npts, nst, ncol, eff, grid, per_cta, part, err, wait_ns, stall, s)
                              : launchW<64>(sc, npts, nst, ncol, eff, grid, per_cta, part, err, wait_ns, stall, s);
    if(r != cudaSuccess)
        return r;
    const int nent = 4 * ncol * ncol;
    gf_gram_tc_sum<<<nent, 128, 0, s>>>(part, grid, nent, out);
    return cudaGetLastError();
}
