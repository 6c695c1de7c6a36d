// Generic BF16 tensor-core GEMM on tcgen05:  C[m, n] = sum_k A(m, k) B(n, k)
// with FP32 accumulation in TMEM.
//
// A CTA of 128 threads owns a 128 x BN output tile.  K is consumed in chunks
// of 64: all threads stage the chunk's A (128 x 64) and B (BN x 64) tiles into
// shared memory through the loader functors (which implement implicit
// im2col, transposes and zero padding; each returns 8 bf16 of one row), one
// thread issues four K = 16 MMAs and commits them to the stage's mbarrier,
// and the next chunk is staged into the other buffer while they run.  The
// epilogue reads the accumulator from TMEM (warp w: rows 32 w .. 32 w + 31)
// and hands 8 consecutive columns of a row at a time to the epilogue functor.
// gridDim.z > 1 splits K (the epilogue then accumulates, e.g. atomically).
//
// Loader (index work split so that it is paid once per row and once per K
// group, not per load):
//   typename Row; __device__ Row row(int r) const;     once per CTA and row
//   typename Col; __device__ Col col(int k8) const;    once per K chunk (k = 8 k8 .. 8 k8 + 7)
//   __device__ uint4 load(const Row &, const Col &) const;   8 16-bit values
// Every thread stages a fixed K group of 8 A rows (and BN / 16 B rows).
// Epilogue: __device__ void operator()(int m, int n0, const float (&v)[8]) const
#pragma once
#include <cuda.h>

#include <cstdint>

#include "umma.cuh"

namespace slamgb {

constexpr int kGemmThreads = 128;
constexpr int kGemmKChunk = 64;
constexpr uint32_t kGemmWaitPolls = 1u << 22;
// polls of the failure-detection test's wait on a barrier nothing arrives at
constexpr uint32_t kGemmStallTestPolls = 256;

template <int BN>
constexpr int gemm_smem_bytes() {
    return 2 * (128 * kGemmKChunk * 2 + BN * kGemmKChunk * 2) + 1024;
}

// `layout` bits 0-1 select the operand core-matrix offsets (0: K-direction
// 128 B, row-direction 1024 B; 1: the two exchanged) for the layout
// self-check; bit 2 (failure-detection test) makes the first pipeline wait
// wait on an mbarrier that nothing arrives at, so that it runs out, the MMAs
// already issued are drained and the kernel reports a time-out.
// F16: the loaders return FP16 instead of BF16 values.
template <int BN, bool F16, class LA, class LB, class EP>
__global__ void __launch_bounds__(kGemmThreads) k_umma_gemm(LA la, LB lb, EP ep, int M, int N, int kchunks,
                                                            int chunks_per_split, int layout, int *err) {
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "BN");
    constexpr int A_BYTES = 128 * kGemmKChunk * 2, B_BYTES = BN * kGemmKChunk * 2, STAGE = A_BYTES + B_BYTES;
    constexpr uint32_t IDESC = F16 ? umma::idesc_f16_f32(128, BN) : umma::idesc_bf16_f32(128, BN);
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t mbar[3];
    __shared__ uint32_t tmem_base;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
    const int c_begin = blockIdx.z * chunks_per_split;
    const int c_end = min(kchunks, c_begin + chunks_per_split);
    const int nch = c_end - c_begin;
    if (nch <= 0) return;
    const bool stall_test = (layout & 4) != 0;
    layout &= 3;
    if (warp == 0) {
        umma::tmem_alloc(&tmem_base, BN < 32 ? 32 : BN);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        umma::mbar_init(&mbar[0], 1);
        umma::mbar_init(&mbar[1], 1);
        umma::mbar_init(&mbar[2], 1);  // never arrived at (stall test)
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lbo = layout ? 1024u : 128u, sbo = layout ? 128u : 1024u;
    // thread t writes the 16-byte slots t + 128 j: row group (t >> 6) + 2 j,
    // K group (t >> 3) & 7, row (t & 7) -- conflict-free 16-byte stores
    constexpr int AR = 8, BR = BN / 16;
    const int kg = (tid >> 3) & 7;
    typename LA::Row ra[AR];
    typename LB::Row rb[BR];
#pragma unroll
    for (int j = 0; j < AR; ++j) ra[j] = la.row(m0 + (((tid >> 6) + 2 * j) << 3) + (tid & 7));
#pragma unroll
    for (int j = 0; j < BR; ++j) rb[j] = lb.row(n0 + (((tid >> 6) + 2 * j) << 3) + (tid & 7));
    bool ok = true;
    int c = 0;
    for (; c < nch; ++c) {
        const int s = c & 1;
        uint8_t *sa = smem + s * STAGE;
        uint8_t *sb = sa + A_BYTES;
        // the MMAs of chunk c - 2 read this stage; the decision to go on is
        // block-uniform so every thread leaves the loop at the same chunk
        if (c >= 2) {
            ok = stall_test ? umma::mbar_wait(&mbar[2], 0, kGemmStallTestPolls)
                            : umma::mbar_wait(&mbar[s], ((c - 2) >> 1) & 1, kGemmWaitPolls);
            if (!__syncthreads_and(ok)) break;
        }
        const int k8 = (c_begin + c) * (kGemmKChunk / 8) + kg;
        {
            const typename LA::Col ca = la.col(k8);
#pragma unroll
            for (int j = 0; j < AR; ++j) *reinterpret_cast<uint4 *>(sa + (tid + 128 * j) * 16) = la.load(ra[j], ca);
        }
        {
            const typename LB::Col cb = lb.col(k8);
#pragma unroll
            for (int j = 0; j < BR; ++j) *reinterpret_cast<uint4 *>(sb + (tid + 128 * j) * 16) = lb.load(rb[j], cb);
        }
        umma::fence_smem_to_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            const uint32_t a0 = umma::smem_u32(sa), b0 = umma::smem_u32(sb);
#pragma unroll
            for (int k = 0; k < kGemmKChunk / 16; ++k)
                umma::mma_bf16(tmem, umma::smem_desc(a0 + k * 256, lbo, sbo), umma::smem_desc(b0 + k * 256, lbo, sbo),
                               IDESC, (c > 0 || k > 0) ? 1u : 0u);
            umma::mma_commit(&mbar[s]);
        }
    }
    // all MMAs issued so far are done when the last commit's phase
    // completes; waited for (bounded) whatever stopped the loop, so that no
    // MMA still writes the accumulator when TMEM is released
    const int last = c - 1;
    const bool drained = umma::mbar_wait(&mbar[last & 1], (last >> 1) & 1, kGemmWaitPolls);
    ok = __syncthreads_and(ok && drained) && c == nch;
    umma::fence_after_sync();
    if (ok) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int j = 0; j < BN; j += 8) {
            float v[8];
            umma::tmem_ld8(trow + j, v);
            if (row < M && n0 + j < N) ep(row, n0 + j, v);
        }
    } else if (tid == 0 && err) {
        atomicExch(err, 1);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, BN < 32 ? 32 : BN);
}

// ---------------------------------------------------------------------------
// Asynchronously fed variant.  The operand slots go from global memory
// straight into the stage buffers by cp.async (no register staging): the
// loaders name the source of each 16-byte slot,
//   __device__ const void *src(const Row &, const Col &, int &bytes) const;
// (bytes < 16 zero-fills the rest of the slot; bytes = 0 reads nothing and
// the returned address only has to be a valid one), and S stages of K chunks
// are in flight while the MMAs of the oldest run.  Stage s of chunk c is
// refilled with chunk c + S once the MMAs of chunk c have completed (their
// commit on mbar[s]).  Every wait is bounded like the register-staged
// kernel's; whatever stops the loop, the kernel waits (bounded) for its own
// copies and MMAs before it releases TMEM.
template <int BN, int S>
constexpr int gemm_async_smem_bytes() {
    return S * (128 * kGemmKChunk * 2 + BN * kGemmKChunk * 2) + 1024;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(umma::smem_u32(smem)), "l"(gmem), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_group() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_groups() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// TMA (cp.async.bulk.tensor) load of one 2D box into shared memory,
// completing `bytes` on the mbarrier's transaction count.
__device__ __forceinline__ void tma_load_2d(void *smem, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            umma::smem_u32(smem)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(umma::smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// TMAB: the B operand (the weights, a dense [N][K] matrix) comes by TMA
// instead: per stage one thread issues eight boxes of BN rows x 8 K values
// (16 bytes), K group j landing at j * BN * 16 bytes, so the core matrices
// of B are 128 bytes apart along N and BN * 16 bytes apart along K; the
// stage's "full" mbarrier counts the bytes in and the MMA issuer waits on
// it.  A (the implicit im2col rows) stays on cp.async.
template <int BN, bool F16, int S, bool TMAB, class LA, class LB, class EP>
__global__ void __launch_bounds__(kGemmThreads) k_umma_gemm_async(LA la, LB lb, EP ep, int M, int N, int kchunks,
                                                                  int chunks_per_split, int *err,
                                                                  const __grid_constant__ CUtensorMap tmb) {
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "BN");
    static_assert(S >= 2 && S <= 6, "stages");
    constexpr int A_BYTES = 128 * kGemmKChunk * 2, B_BYTES = BN * kGemmKChunk * 2, STAGE = A_BYTES + B_BYTES;
    constexpr uint32_t IDESC = F16 ? umma::idesc_f16_f32(128, BN) : umma::idesc_bf16_f32(128, BN);
    // B's core-matrix offsets: along K, along N
    constexpr uint32_t B_LBO = TMAB ? BN * 16u : 128u, B_SBO = TMAB ? 128u : 1024u;
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t mbar[S];
    __shared__ __align__(8) uint64_t full[S];
    __shared__ uint32_t tmem_base;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
    const int c_begin = blockIdx.z * chunks_per_split;
    const int c_end = min(kchunks, c_begin + chunks_per_split);
    const int nch = c_end - c_begin;
    if (nch <= 0) return;
    if (warp == 0) {
        umma::tmem_alloc(&tmem_base, BN < 32 ? 32 : BN);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) {
            umma::mbar_init(&mbar[s], 1);
            umma::mbar_init(&full[s], 1);
        }
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    // slots as in k_umma_gemm: thread t fills the 16-byte slots t + 128 j
    constexpr int AR = 8, BR = BN / 16;
    const int kg = (tid >> 3) & 7;
    typename LA::Row ra[AR];
#pragma unroll
    for (int j = 0; j < AR; ++j) ra[j] = la.row(m0 + (((tid >> 6) + 2 * j) << 3) + (tid & 7));
    typename LB::Row rb[TMAB ? 1 : BR];
    if constexpr (!TMAB) {
#pragma unroll
        for (int j = 0; j < BR; ++j) rb[j] = lb.row(n0 + (((tid >> 6) + 2 * j) << 3) + (tid & 7));
    }
    auto issue = [&](int c) {
        uint8_t *sa = smem + (c % S) * STAGE;
        uint8_t *sb = sa + A_BYTES;
        const int k8 = (c_begin + c) * (kGemmKChunk / 8) + kg;
        const typename LA::Col ca = la.col(k8);
#pragma unroll
        for (int j = 0; j < AR; ++j) {
            int bytes;
            const void *g = la.src(ra[j], ca, bytes);
            cp_async16(sa + (tid + 128 * j) * 16, g, bytes);
        }
        if constexpr (TMAB) {
            if (tid == 0) {
                uint64_t *bar = &full[c % S];
                mbar_expect_tx(bar, (uint32_t)B_BYTES);
                const int kx = (c_begin + c) * kGemmKChunk;
#pragma unroll
                for (int j = 0; j < kGemmKChunk / 8; ++j) tma_load_2d(sb + j * BN * 16, &tmb, kx + 8 * j, n0, bar);
            }
        } else {
            const typename LB::Col cb = lb.col(k8);
#pragma unroll
            for (int j = 0; j < BR; ++j) {
                int bytes;
                const void *g = lb.src(rb[j], cb, bytes);
                cp_async16(sb + (tid + 128 * j) * 16, g, bytes);
            }
        }
    };
    int issued = 0;  // chunks whose loads were issued
#pragma unroll
    for (int p = 0; p < S - 1; ++p) {
        if (p < nch) {
            issue(p);
            issued = p + 1;
        }
        cp_async_group();
    }
    bool ok = true;
    int c = 0;
    for (; c < nch; ++c) {
        const int s = c % S;
        // refill the stage the MMAs of chunk c - 1 read, with chunk c + S - 1
        const int pf = c + S - 1;
        if (pf < nch) {
            if (c >= 1) {
                ok = umma::mbar_wait(&mbar[(c - 1) % S], ((c - 1) / S) & 1, kGemmWaitPolls);
                if (!__syncthreads_and(ok)) break;
            }
            issue(pf);
            issued = pf + 1;
        }
        cp_async_group();
        cp_async_wait_groups<S - 1>();  // this thread's copies of chunk c have landed
        umma::fence_smem_to_async();
        bool bok = true;
        if (TMAB && tid == 0) bok = umma::mbar_wait(&full[s], (c / S) & 1, kGemmWaitPolls);
        if (!__syncthreads_and(bok)) {
            ok = false;
            break;
        }
        if (tid == 0) {
            umma::fence_after_sync();
            const uint32_t a0 = umma::smem_u32(smem + s * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
            for (int k = 0; k < kGemmKChunk / 16; ++k)
                umma::mma_bf16(tmem, umma::smem_desc(a0 + k * 256, 128u, 1024u),
                               umma::smem_desc(b0 + k * 2 * B_LBO, B_LBO, B_SBO), IDESC, (c > 0 || k > 0) ? 1u : 0u);
            umma::mma_commit(&mbar[s]);
        }
    }
    cp_async_wait_groups<0>();
    // TMA boxes still in flight (a loop left early): wait for them (bounded)
    // before the CTA's shared memory can go away
    if (TMAB && tid == 0)
        for (int q = c; q < issued; ++q) umma::mbar_wait(&full[q % S], (q / S) & 1, kGemmWaitPolls);
    bool drained = true;
    if (c > 0) {
        const int last = c - 1;
        drained = umma::mbar_wait(&mbar[last % S], (last / S) & 1, kGemmWaitPolls);
    }
    ok = __syncthreads_and(ok && drained) && c == nch;
    umma::fence_after_sync();
    if (ok) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int j = 0; j < BN; j += 8) {
            float v[8];
            umma::tmem_ld8(trow + j, v);
            if (row < M && n0 + j < N) ep(row, n0 + j, v);
        }
    } else if (tid == 0 && err) {
        atomicExch(err, 1);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, BN < 32 ? 32 : BN);
}

// Stages of K chunks per CTA (compile-time override SLAMGB_GEMM_STAGES): the
// network's products have 2-12 chunks per output tile, so fewer stages and
// more resident CTAs per SM hide the load latency better than deep per-CTA
// pipelines.
#ifndef SLAMGB_GEMM_STAGES
#define SLAMGB_GEMM_STAGES 3
#endif
template <int BN, class LA, class LB, class EP, bool F16 = false, int S = SLAMGB_GEMM_STAGES>
cudaError_t launch_umma_gemm_async(const LA &la, const LB &lb, const EP &ep, int M, int N, int K, int *err,
                                   cudaStream_t s, const CUtensorMap *tmb = nullptr) {
    if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
    const int kchunks = (K + kGemmKChunk - 1) / kGemmKChunk;
    constexpr int smem = gemm_async_smem_bytes<BN, S>();
    dim3 grid((M + 127) / 128, (N + BN - 1) / BN, 1);
    if (tmb) {
        static bool attr_set = false;  // per instantiation
        if (!attr_set) {
            cudaError_t e = cudaFuncSetAttribute(k_umma_gemm_async<BN, F16, S, true, LA, LB, EP>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            attr_set = true;
        }
        k_umma_gemm_async<BN, F16, S, true, LA, LB, EP><<<grid, kGemmThreads, smem, s>>>(la, lb, ep, M, N, kchunks,
                                                                                        kchunks, err, *tmb);
    } else {
        static bool attr_set = false;
        if (!attr_set) {
            cudaError_t e = cudaFuncSetAttribute(k_umma_gemm_async<BN, F16, S, false, LA, LB, EP>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            attr_set = true;
        }
        CUtensorMap none{};
        k_umma_gemm_async<BN, F16, S, false, LA, LB, EP><<<grid, kGemmThreads, smem, s>>>(la, lb, ep, M, N, kchunks,
                                                                                         kchunks, err, none);
    }
    return cudaGetLastError();
}

// Host-side launch helper (in a .cu translation unit).
template <int BN, class LA, class LB, class EP, bool F16 = false>
cudaError_t launch_umma_gemm(const LA &la, const LB &lb, const EP &ep, int M, int N, int K, int splits, int layout,
                             int *err, cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
    const int kchunks = (K + kGemmKChunk - 1) / kGemmKChunk;
    if (splits < 1) splits = 1;
    if (splits > kchunks) splits = kchunks;
    const int per = (kchunks + splits - 1) / splits;
    splits = (kchunks + per - 1) / per;
    constexpr int smem = gemm_smem_bytes<BN>();
    static bool attr_set = false;  // per instantiation
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_umma_gemm<BN, F16, LA, LB, EP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    dim3 grid((M + 127) / 128, (N + BN - 1) / BN, splits);
    k_umma_gemm<BN, F16, LA, LB, EP><<<grid, kGemmThreads, smem, s>>>(la, lb, ep, M, N, kchunks, per, layout, err);
    return cudaGetLastError();
}

}  // namespace slamgb
