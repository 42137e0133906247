// Dense FP32 product on the 5th-generation tensor cores (sm_103a): C = beta C + alpha A B^T with A
// (M x K) and B (N x K) row-major, K contiguous, the operation the strip factorisation
// (ocmp_strip.cu) spends its flops in. FP32 accuracy from TF32 tensor-core products by the
// split-operand scheme: with a = a_h + a_l (a_h = a truncated to TF32, which is what the tensor core
// reads from an FP32 operand), A B^T ~ A_h B_h + A_h B_l + A_l B_h, three MMAs per K step into one
// FP32 accumulator in tensor memory. The dropped term A_l B_l and the truncation of the low parts
// leave about 2^-21 relative error per product, against 2^-24 for FP32 FMAs.
//
// One CTA computes one 128 x 128 tile of C with 6 warps:
//   warp 0     TMA producer: 128 x 32 FP32 boxes of A and B (128-byte rows, 128B swizzle) into a
//              3-stage shared-memory ring (cp.async.bulk.tensor, mbarrier completion);
//   warps 2-5  split the staged boxes into their low parts (x - trunc_tf32(x), same swizzled layout,
//              elementwise), then run the epilogue: tcgen05.ld of the accumulator (each warp its 32
//              TMEM lanes = rows) into a staging tile in the idle stage buffers, then C read, scaled
//              and written row by row (512 contiguous bytes per row and warp instruction);
//   warp 1     allocates 128 TMEM columns, and one thread issues the tcgen05.mma.kind::tf32
//              instructions (M = 128, N = 128, K = 8) and the tcgen05.commit arrivals that free the
//              stages and signal the epilogue.
// Every mbarrier wait is bounded (about one second of clock); a wait that gives up sets *err and the
// CTA drains what it started (bounded as well), frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "ocmp_internal.h"

namespace ocmp {
namespace {

constexpr int TBM = 128, TBN = 128, TBK = 32, TST = 3;
constexpr int kBoxBytes = TBM * TBK * 4;            // 16 KiB, one 128 x 32 FP32 box (A or B)
constexpr int kStageBytes = 4 * kBoxBytes;          // A, B, A_low, B_low
constexpr int kTcSmem = TST * kStageBytes + 1024 + 256;
constexpr int kTcThreads = 192;
constexpr long long kWaitCycles = 2000000000LL;     // about one second at the boost clock

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; false when it gave up or another role already did (*abort)
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int* abort) {
    const long long t0 = clock64();
    while (!mbar_try(a, parity)) {
        if (*abort) return false;
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

// K-major operand in the 128B-swizzle canonical layout: 8-row groups of 1024 bytes (SBO), rows of
// 128 bytes; start address in 16-byte units, descriptor version 1, layout type 2 (128B swizzle)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                    // leading-dimension offset (unused with swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride-dimension offset: next 8-row group
    d |= (uint64_t)1 << 46;                    // descriptor version
    d |= (uint64_t)2 << 61;                    // 128-byte swizzle
    return d;
}

// instruction descriptor: FP32 accumulator, TF32 A and B, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TBN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, 1)
    tc_gemm_nt_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int K,
                      float* __restrict__ C, int64_t ldc, float alpha, float beta, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = saddr(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    // layout: TST stages of [A | B | A_low | B_low], then barriers
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + TST * kStageBytes);
    const uint32_t bar0 = base + TST * kStageBytes;
    auto full_b = [&](int s) { return bar0 + 8u * s; };
    auto split_b = [&](int s) { return bar0 + 8u * (TST + s); };
    auto empty_b = [&](int s) { return bar0 + 8u * (2 * TST + s); };
    const uint32_t accum_b = bar0 + 8u * (3 * TST);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * TST + 1);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = K / TBK;
    const int m0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TST; s++) {
            mbar_init(full_b(s), 1);
            mbar_init(split_b(s), 4);
            mbar_init(empty_b(s), 1);
        }
        mbar_init(accum_b, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                     "r"(TBN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    auto give_up = [&]() {
        *abort = 1;
        atomicExch(err, 1);
    };

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < nk; kb++) {
                const int s = kb % TST, u = kb / TST;
                if (u > 0 && !mbar_wait(empty_b(s), (u - 1) & 1, abort)) {
                    give_up();
                    break;
                }
                const uint32_t st = base + s * kStageBytes;
                mbar_expect_tx(full_b(s), 2 * kBoxBytes);
                tma_load_2d(st, &ta, kb * TBK, m0, full_b(s));
                tma_load_2d(st + kBoxBytes, &tb, kb * TBK, n0, full_b(s));
                issued = kb + 1;
            }
            // drain: every issued box must have landed before the CTA may exit
            for (int kb = issued - TST < 0 ? 0 : issued - TST; kb < issued; kb++) {
                const long long t0 = clock64();
                while (!mbar_try(full_b(kb % TST), (kb / TST) & 1) && clock64() - t0 < kWaitCycles) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            for (int kb = 0; kb < nk; kb++) {
                const int s = kb % TST, u = kb / TST;
                if (!mbar_wait(split_b(s), u & 1, abort)) {
                    give_up();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = base + s * kStageBytes;
                const uint32_t a = st, b = st + kBoxBytes, al = st + 2 * kBoxBytes, bl = st + 3 * kBoxBytes;
#pragma unroll
                for (int kk = 0; kk < TBK / 8; kk++) {
                    const uint32_t off = kk * 32;  // 8 TF32 values along K
                    const uint32_t first = (kb > 0 || kk > 0) ? 1u : 0u;
                    mma_tf32(tmem, sdesc(a + off), sdesc(b + off), first);
                    mma_tf32(tmem, sdesc(a + off), sdesc(bl + off), 1u);
                    mma_tf32(tmem, sdesc(al + off), sdesc(b + off), 1u);
                }
                mma_commit(empty_b(s));
            }
            // the accumulator is complete once every MMA issued above has finished
            mma_commit(accum_b);
        }
        __syncwarp();
    } else {
        // warps 2..5: low parts of the staged boxes, then the epilogue
        const int t = threadIdx.x - 64;  // 0..127
        bool ok = true;
        for (int kb = 0; kb < nk && ok; kb++) {
            const int s = kb % TST, u = kb / TST;
            if (!mbar_wait(full_b(s), u & 1, abort)) {
                give_up();
                ok = false;
                break;
            }
            uint8_t* st = gbase + s * kStageBytes;
            const float4* src = reinterpret_cast<const float4*>(st);
            float4* dst = reinterpret_cast<float4*>(st + 2 * kBoxBytes);
            // A and B are adjacent, and so are A_low and B_low: one pass over 2 boxes
            for (int q = t; q < 2 * kBoxBytes / 16; q += 128) {
                const float4 v = src[q];
                float4 o;
                o.x = v.x - __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u);
                o.y = v.y - __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u);
                o.z = v.z - __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u);
                o.w = v.w - __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u);
                dst[q] = o;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(split_b(s));
        }
        if (ok && mbar_wait(accum_b, 0, abort)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // TMEM lanes 32q..32q+31 are the tile's rows; each thread takes its row's 128 columns
            // into a staging tile in the (now idle) stage buffers, then the warp writes C row by
            // row, 512 contiguous bytes per row
            const int q = warp & 3;
            constexpr int SLD = TBN + 4;            // 16-byte aligned rows, conflict-free float4 writes
            float* stg = reinterpret_cast<float*>(gbase) + q * (32 * SLD);
#pragma unroll 1
            for (int c0 = 0; c0 < TBN; c0 += 32) {
                uint32_t r[32];
                const uint32_t ta_ = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                    "[%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                      "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                      "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(ta_)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int v = 0; v < 32; v += 4)
                    *reinterpret_cast<float4*>(stg + lane * SLD + c0 + v) =
                        make_float4(__uint_as_float(r[v]), __uint_as_float(r[v + 1]), __uint_as_float(r[v + 2]),
                                    __uint_as_float(r[v + 3]));
            }
            __syncwarp();
#pragma unroll 4
            for (int rr = 0; rr < 32; rr++) {
                const float4 a = *reinterpret_cast<const float4*>(stg + rr * SLD + 4 * lane);
                float4* p = reinterpret_cast<float4*>(C + ((int64_t)m0 + 32 * q + rr) * ldc + n0) + lane;
                float4 o = beta != 0.f ? *p : make_float4(0.f, 0.f, 0.f, 0.f);
                o.x = alpha * a.x + beta * o.x;
                o.y = alpha * a.y + beta * o.y;
                o.z = alpha * a.z + beta * o.z;
                o.w = alpha * a.w + beta * o.w;
                *p = o;
            }
        } else if (ok) {
            give_up();
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort && warp == 1 && lane == 0) {
        // a role gave up: let the MMAs already issued finish before the tensor memory is released
        mma_commit(accum_b);
        const long long t0 = clock64();
        while (!mbar_try(accum_b, 0) && !mbar_try(accum_b, 1) && clock64() - t0 < kWaitCycles) {
        }
    }
    __syncwarp();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TBN) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
cudaError_t g_encode_err = cudaSuccess;

int get_encode() {
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        g_encode_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (g_encode_err == cudaSuccess && q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode) return fail(OCMP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return OCMP_OK;
}

// rows x cols FP32 row-major with leading dimension ld (elements); 128 x 32 boxes, 128B swizzle
int make_map(CUtensorMap* map, const float* p, int64_t rows, int64_t cols, int64_t ld) {
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {(cuuint32_t)TBK, (cuuint32_t)TBM};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(p), dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(OCMP_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return OCMP_OK;
}

}  // namespace

int tc_gemm_nt(int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
               float alpha, float beta, int* err, cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0 || M % TBM || N % TBN || K % TBK)
        return fail(OCMP_ERR_ARG, "tensor-core product: M, N must be multiples of 128 and K of 32");
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15 || (lda | ldb) & 3 || ldc & 3 ||
        reinterpret_cast<uintptr_t>(C) & 15)
        return fail(OCMP_ERR_ARG, "tensor-core product: operands must be 16-byte aligned");
    int r = get_encode();
    if (r) return r;
    static thread_local int attr_dev = -1;
    int dev = 0;
    OCMP_CUDA(cudaGetDevice(&dev));
    if (attr_dev != dev) {
        OCMP_CUDA(cudaFuncSetAttribute(tc_gemm_nt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
        attr_dev = dev;
    }
    CUtensorMap ta, tb;
    if ((r = make_map(&ta, A, M, K, lda))) return r;
    if ((r = make_map(&tb, B, N, K, ldb))) return r;
    const dim3 g(N / TBN, M / TBM);
    OCMP_LAUNCH(tc_gemm_nt_kernel<<<g, kTcThreads, kTcSmem, st>>>(ta, tb, K, C, ldc, alpha, beta, err));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

}  // namespace ocmp
