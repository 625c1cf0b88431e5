// Measurement probes of this GPU, for reporting rooflines (not used by the convolution path):
//   fvgb_ffma_probe       FP32 FMA rate
//   fvgb_row_gather_probe random 128-byte feature-row gathers into a 128B-swizzled shared-memory
//                         stage (the A-operand layout of the tensor-core kernels), by cp.async
//                         (the kernels' method) or by TMA tile::gather4 with 1, 8 or 32 issuing
//                         threads.  All waits are bounded; a wait that gives up sets *err.
#include <cuda.h>

#include <mutex>

#include "tc_common.cuh"

using namespace fvgb;

// ---------------------------------------------------------------------------------------------
// FP32 FMA rate probe: every thread runs 8 independent fma chains of `iters` steps (enough
// independent work to keep the FMA pipes full), 2 * 8 * iters FLOPs per thread.  The caller
// times the launch; the chains' sum is written so that nothing is optimised away.
namespace fvgb {
namespace {
__global__ void __launch_bounds__(256) ffma_probe_kernel(float *out, int64_t iters, float b, float c) {
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (float)(threadIdx.x + i);
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = fmaf(v[i], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += v[i];
    if (s == 12345.678f) out[0] = s;  // practically never true: keeps the chains live
    if (threadIdx.x == 0 && blockIdx.x == 0) out[1] = s;
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_ffma_probe(float *out, int64_t iters, int32_t blocks_per_sm, double *flops, fvgb_stream_t stream) {
    if (!out || iters < 1 || blocks_per_sm < 1 || blocks_per_sm > 64 || !flops) return FVGB_EINVAL;
    const int64_t blocks = (int64_t)device_sm_count() * blocks_per_sm;
    ffma_probe_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(out, iters, 0.999999f, 1e-7f);
    *flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
    count_launches(1);
    return launch_status();
}

namespace fvgb {
namespace {
using namespace tc;

constexpr int kProbeStages = 4, kProbeStage = 16384;

__device__ __forceinline__ void gather4_load(uint32_t dst, const void *tmap, int32_t c, int32_t r0, int32_t r1,
                                             int32_t r2, int32_t r3, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_u32(bar))
        : "memory");
}

// mode 0: one thread issues the 32 gather4 of a stage; 1: lane 0 of each of the 8 warps, 4 each;
// 2: the 32 lanes of warp 0, 1 each; 3: cp.async by the 8 warps (lane -> 16-byte piece of 4 rows);
// 4: both at once, rows 0-63 by gather4 (16 lanes of warp 0), rows 64-127 by cp.async (warps 4-7)
__global__ void __launch_bounds__(256, 1) row_gather_probe_kernel(const __grid_constant__ CUtensorMap tm,
                                                                  const uint8_t *__restrict__ x,
                                                                  const int32_t *__restrict__ rows, int32_t nlist,
                                                                  int32_t iters, int32_t mode, int32_t *err) {
    extern __shared__ uint8_t psm[];
    uint8_t *base = reinterpret_cast<uint8_t *>(((uintptr_t)psm + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(base + kProbeStages * kProbeStage);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0)
        for (int s = 0; s < kProbeStages; ++s) mbar_init(&full[s], mode == 3 ? 256 : (mode == 4 ? 129 : 1));
    __syncthreads();
    auto issue = [&](int it) {
        const int s = it % kProbeStages;
        const uint32_t st = smem_u32(base + s * kProbeStage);
        const int64_t rb = ((int64_t)blockIdx.x * iters * 128 + (int64_t)it * 128) % nlist;
        if (mode == 3) {
            const int j = lane & 7, rsub = lane >> 3;
            for (int q = 0; q < 4; ++q) {
                const int r = warp * 16 + rsub + 4 * q;
                const int32_t src = rows[(rb + r) % nlist];
                cp_async_16(st + sw128_offset(r, j), x + (int64_t)src * 128 + j * 16, 16u);
            }
            cp_async_arrive_noinc(&full[s]);
            return;
        }
        if (mode == 4) {
            if (tid == 0) mbar_arrive_expect_tx(&full[s], kProbeStage / 2);
            __syncwarp();
            if (warp == 0 && lane < 16) {
                const int64_t r = rb + 4 * lane;
                gather4_load(st + lane * 512, &tm, 0, rows[r % nlist], rows[(r + 1) % nlist], rows[(r + 2) % nlist],
                             rows[(r + 3) % nlist], &full[s]);
            }
            if (warp >= 4) {
                const int j = lane & 7, rsub = lane >> 3;
                for (int q = 0; q < 4; ++q) {
                    const int r = 64 + (warp - 4) * 16 + rsub + 4 * q;
                    const int32_t src = rows[(rb + r) % nlist];
                    cp_async_16(st + sw128_offset(r, j), x + (int64_t)src * 128 + j * 16, 16u);
                }
                cp_async_arrive_noinc(&full[s]);
            }
            return;
        }
        int g0 = 0, gn = 0;
        bool me = false;
        if (mode == 0) me = tid == 0, g0 = 0, gn = 32;
        if (mode == 1) me = lane == 0, g0 = warp * 4, gn = 4;
        if (mode == 2) me = warp == 0, g0 = lane, gn = 1;
        if (tid == 0) mbar_arrive_expect_tx(&full[s], kProbeStage);
        __syncwarp();
        if (me)
            for (int g = g0; g < g0 + gn; ++g) {
                const int64_t r = rb + 4 * g;
                gather4_load(st + g * 512, &tm, 0, rows[r % nlist], rows[(r + 1) % nlist], rows[(r + 2) % nlist],
                             rows[(r + 3) % nlist], &full[s]);
            }
    };
    for (int it = 0; it < kProbeStages && it < iters; ++it) issue(it);
    for (int it = 0; it < iters; ++it) {
        const int s = it % kProbeStages;
        long long n = 0;
        while (!mbar_try_wait(&full[s], (it / kProbeStages) & 1)) {
            if (++n > (1ll << 24)) {
                atomicExch(err, FVGB_ETIMEOUT);
                break;
            }
        }
        __syncthreads();  // every thread is done with stage s before it is refilled
        if (it + kProbeStages < iters) issue(it + kProbeStages);
    }
    // copies still in flight land before the CTA exits (bounded)
    for (int it = iters > kProbeStages ? iters - kProbeStages : 0; it < iters; ++it) {
        long long n = 0;
        while (!mbar_try_wait(&full[it % kProbeStages], (it / kProbeStages) & 1) && ++n < (1ll << 24)) {
        }
    }
}

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_row_gather_probe(int32_t mode, const void *x, int64_t n_rows, const int32_t *rows, int32_t nlist,
                                     int32_t iters, int32_t *err_dev, int64_t *bytes, fvgb_stream_t stream) {
    if (mode < 0 || mode > 4 || !x || n_rows < 1 || n_rows > INT32_MAX || !rows || nlist < 128 || iters < 1 ||
        !err_dev || !bytes || ((uintptr_t)x & 127))
        return FVGB_EINVAL;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        return FVGB_ECUDA;
    CUtensorMap tm;
    const cuuint64_t gd[2] = {64, (cuuint64_t)n_rows}, gs[1] = {128};
    const cuuint32_t box[2] = {64, 1}, es[2] = {1, 1};
    if (reinterpret_cast<EncodeFn>(p)(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(x), gd, gs, box, es,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return FVGB_EINVAL;
    const int smem = kProbeStages * kProbeStage + 1024 + 64;
    if (set_dynamic_smem(row_gather_probe_kernel, smem) != cudaSuccess)
        return launch_status();
    const int blocks = device_sm_count();
    row_gather_probe_kernel<<<blocks, 256, smem, as_stream(stream)>>>(tm, (const uint8_t *)x, rows, nlist, iters, mode,
                                                                      err_dev);
    *bytes = (int64_t)blocks * iters * kProbeStage;
    count_launches(1);
    return launch_status();
}
