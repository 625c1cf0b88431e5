// Tensor-core (tcgen05 / TMEM) weight gradient and FP8 quantisation for sm_103a.
// (The forward / data-gradient contraction lives in conv_fwd_tc.cu.)
#include <cuda_bf16.h>

#include "tc_common.cuh"

namespace fvgb {
namespace {

using namespace tc;

constexpr int kTileM = 128;
constexpr int kWgGatherWarps = 8;  // 256 gather threads: cp.async throughput grows with the issuing warps
constexpr int kWgMmaWarp = kWgGatherWarps;
constexpr int kThreads = (kWgGatherWarps + 1) * 32;

}  // namespace
}  // namespace fvgb

using namespace fvgb;

// ---------------------------------------------------------------------------------------------
// FP8-E4M3 quantisation: out[r, c] = e4m3(x[r, c] * inv_scale[c]) (round to nearest, saturate).
#include <cuda_fp8.h>

namespace fvgb {
namespace {
template <typename T>
__device__ __forceinline__ float to_f32(T v);
template <>
__device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename T>
__global__ void quantize_e4m3_kernel(const T *__restrict__ x, int64_t n, int32_t c, int64_t ldx,
                                     const float *__restrict__ inv_scale, uint8_t *__restrict__ out, int64_t ldo) {
    const int64_t total = n * c;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / c;
        const int32_t ch = (int32_t)(e - r * c);
        const float v = to_f32<T>(x[r * ldx + ch]) * inv_scale[ch];
        out[r * ldo + ch] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
    }
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_quantize_e4m3(int32_t dtype, const void *x, int64_t n, int32_t c, int64_t ldx,
                                  const float *inv_scale, void *out, int64_t ldo, fvgb_stream_t stream) {
    if (n < 0 || c < 1 || ldx < c || ldo < c || !inv_scale || (n > 0 && (!x || !out))) return FVGB_EINVAL;
    if (n == 0) return FVGB_OK;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n * c, 256), 148 * 64);
    cudaStream_t s = as_stream(stream);
    if (dtype == FVGB_F32)
        quantize_e4m3_kernel<float><<<blocks, 256, 0, s>>>((const float *)x, n, c, ldx, inv_scale, (uint8_t *)out, ldo);
    else if (dtype == FVGB_BF16)
        quantize_e4m3_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>((const __nv_bfloat16 *)x, n, c, ldx, inv_scale,
                                                                   (uint8_t *)out, ldo);
    else
        return FVGB_ETYPE;
    count_launches(1);
    return launch_status();
}

// ---------------------------------------------------------------------------------------------
// Tensor-core weight gradient (BF16 in, FP32 per-CTA partials, FP64 cross-CTA reduction):
//
//   dW[k, ci, co] = sum_m x[map[m,k], ci] * dy[m, co]
//
// One CTA owns a group of G = 128 / c_in kernel offsets and a chunk of output rows.  Per stage
// of 128 rows it gathers the G feature rows of every output row into an MN-major A operand
// (M = G*c_in stacked offsets, K = 128 rows) and the dy rows into an MN-major B operand
// (N = c_out), so dy is loaded once for all G offsets; D (M = 128, N = c_out) accumulates in
// TMEM across the chunk.  Stages whose 128 rows have none of the group's offsets (per-tile
// occupancy mask) are skipped.  The epilogue writes the chunk's partial dW slice in FP32; a
// second kernel sums the partials over chunks in FP64 in a fixed order.
// Replaces the split-K wgrad kernels conv_backward_cuda_setting{1,2}_mode{0,1}_*
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMMGrad.cu:115-4101,
// ...GradSorted.cu:115-4582) and their [32, K*Cin, Cout].sum(0).
namespace fvgb {
namespace {

constexpr int kMNAtom = 16384;

__device__ __forceinline__ void st_shared_zero16(uint32_t addr) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(addr), "r"(0) : "memory");
}  // 128 K-rows x 128 bytes: one 64-element-wide MN atom of a stage

// MN-major operand, 128B swizzle: MN atoms (64 elements) kMNAtom apart (LBO), 8-row K groups
// 1024 bytes apart (SBO).
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)(kMNAtom >> 4) << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// byte offset of 16-byte piece `e8` (element index e = 8*e8 along MN) of K-row r in an MN-major stage
__device__ __forceinline__ uint32_t mn_offset(uint32_t r, uint32_t e) {
    return (e >> 6) * kMNAtom + (r >> 3) * 1024u + (r & 7u) * 128u + ((((e & 63u) >> 3) ^ (r & 7u)) << 4);
}

struct WgArgs {
    const uint8_t *x;  // bf16 [n_x, cin]
    int64_t n_x, ldx_bytes;
    int32_t cin;
    const int32_t *map;
    int64_t n_out;
    int32_t K;
    const uint32_t *tile_mask;
    const uint8_t *dy;  // bf16 [n_out, cout]
    int64_t lddy_bytes;
    int32_t cout;
    int64_t rows_per_chunk;  // multiple of 128
    float *partials;         // [chunks][K][cin][cout]
    int32_t *err;
    int32_t stages;
};

template <int BN>
__host__ __device__ constexpr int wg_stage_bytes() {
    return 2 * kMNAtom + (BN / 64) * kMNAtom;
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_wgrad_kernel(WgArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kStage = wg_stage_bytes<BN>();
    constexpr int kBOff = 2 * kMNAtom;
    const int S = a.stages;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + S * kStage);
    uint64_t *empty = full + S, *accum = full + 2 * S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = 128 / a.cin;
    const int k0 = blockIdx.x * G;
    const int ng = min(G, a.K - k0);
    const int64_t r_begin = (int64_t)blockIdx.y * a.rows_per_chunk;
    const int64_t r_end = min(a.n_out, r_begin + a.rows_per_chunk);
    const uint32_t gbits = (a.K <= 32) ? (((1u << ng) - 1u) << k0) : 0xffffffffu;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], kWgGatherWarps);  // one arrival per gather warp
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort = 0;
    }
    if (warp == kWgMmaWarp) tmem_alloc(tmem_slot, BN);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int64_t n_tiles = (r_end - r_begin + kTileM - 1) / kTileM;

    auto tile_active = [&](int64_t t) -> bool {
        if (!a.tile_mask || a.K > 32) return true;
        return (a.tile_mask[(r_begin / kTileM) + t] & gbits) != 0;
    };

    int steps = 0;  // active stages: the gather warps run the same loop as the MMA warp
    if (warp < kWgGatherWarps) {
        // Lane -> (16-byte chunk jj of a 128-byte MN atom row, K-rows rsub + 4q of this warp's
        // 16): one warp instruction moves four whole 128-byte atom rows of an operand.  Atom a of
        // the A operand holds M elements a*64 .. a*64+63, i.e. offset (a*64 + 8*jj) / cin of the
        // group at channel (a*64 + 8*jj) % cin.
        const int jj = lane & 7, rsub = lane >> 3, row0 = warp * (kTileM / kWgGatherWarps);
        int joff[2], ci0[2];
#pragma unroll
        for (int at = 0; at < 2; ++at) {
            const int m0 = at * 64 + jj * 8;
            joff[at] = m0 / a.cin;
            ci0[at] = m0 - joff[at] * a.cin;
        }
        uint32_t it = 0, sig = 0, stage = 0, phase = 0, pstage = 0;
        for (int64_t t = 0; t < n_tiles; ++t)
            if (tile_active(t)) ++steps;
        // map entries of a tile for this lane's rows; loaded one active tile ahead, so their
        // latency overlaps the previous stage's copies instead of stalling the next
        auto load_src = [&](int64_t t, int32_t (&dst)[2][4]) {
#pragma unroll
            for (int at = 0; at < 2; ++at)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int64_t m = r_begin + t * kTileM + row0 + rsub + 4 * q;
                    int32_t v = -1;
                    if (m < r_end && joff[at] < ng) {
                        v = a.map[m * a.K + k0 + joff[at]];
                        if (v >= a.n_x) v = -1;
                    }
                    dst[at][q] = v;
                }
        };
        auto next_active = [&](int64_t t) {
            while (t < n_tiles && !tile_active(t)) ++t;
            return t;
        };
        int32_t src_next[2][4];
        int64_t t = next_active(0);
        if (t < n_tiles) load_src(t, src_next);
        for (; t < n_tiles && !*abort;) {
            int32_t src[2][4];
#pragma unroll
            for (int at = 0; at < 2; ++at)
#pragma unroll
                for (int q = 0; q < 4; ++q) src[at][q] = src_next[at][q];
            const int64_t t_next = next_active(t + 1);
            if (t_next < n_tiles) load_src(t_next, src_next);
            bool go = true;
            if (lane == 0) go = mbar_wait(&empty[stage], phase ^ 1, abort);
            go = __shfl_sync(0xffffffffu, go, 0);
            __syncwarp();
            if (!go) break;
            const uint32_t base = smem_u32(smem + stage * kStage);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = row0 + rsub + 4 * q;
                const int64_t m = r_begin + t * kTileM + r;
                // B: dy row m, all c_out channels (BN/64 atoms)
#pragma unroll
                for (int at = 0; at < BN / 64; ++at) {
                    const uint32_t dst = base + kBOff + mn_offset(r, at * 64 + jj * 8);
                    if (m < r_end)
                        cp_async_16(dst, a.dy + m * a.lddy_bytes + at * 128 + jj * 16, 16u);
                    else
                        st_shared_zero16(dst);
                }
                // A: the group's gathered feature rows, stacked along M
#pragma unroll
                for (int at = 0; at < 2; ++at) {
                    const uint32_t dst = base + mn_offset(r, at * 64 + jj * 8);
                    if (src[at][q] >= 0)
                        cp_async_16(dst, a.x + (int64_t)src[at][q] * a.ldx_bytes + ci0[at] * 2, 16u);
                    else
                        st_shared_zero16(dst);
                }
            }
            // cp.async and st.shared are generic-proxy writes: each warp fences its own copies to
            // the tensor core (async proxy), one stage late, so the MMA warp never fences
            cp_async_commit();
            ++it;
            if (++stage == (uint32_t)S) {
                stage = 0;
                phase ^= 1;
            }
            if (it - sig > 1) {
                cp_async_wait_group<1>();
                fence_proxy_async();
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[pstage]);
                ++sig;
                if (++pstage == (uint32_t)S) pstage = 0;
            }
            t = t_next;
        }
        cp_async_wait_group<0>();
        fence_proxy_async();
        __syncwarp();
        if (lane == 0)
            for (; sig < it; ++sig) {
                mbar_arrive(&full[pstage]);
                if (++pstage == (uint32_t)S) pstage = 0;
            }
    } else if (warp == kWgMmaWarp) {
        // the whole warp runs the issue loop (warp-uniform); one elected lane issues each tcgen05 op
        constexpr uint32_t idesc = idesc_m128(BN, 1, 1) | (1u << 15) | (1u << 16);  // bf16, A and B MN-major
        int it = 0;
        for (int64_t t = 0; t < n_tiles; ++t) {
            if (!tile_active(t)) continue;
            const int stage = it % S;
            if (!mbar_wait_warp(&full[stage], (it / S) & 1, abort)) break;
            tc_fence_after();
            const uint32_t As = smem_u32(smem + stage * kStage), Bs = As + kBOff;
#pragma unroll
            for (int q = 0; q < kTileM / 16; ++q)  // 16 rows of K per MMA = two 8-row groups
                mma_f16_warp(tmem, desc_sw128_mn(As + q * 2048), desc_sw128_mn(Bs + q * 2048), idesc,
                             (it > 0 || q > 0) ? 1u : 0u);
            mma_commit_warp(&empty[stage]);
            ++it;
        }
        // it == 0: nothing accumulated -- the epilogue writes zeros
        if (it > 0)
            mma_commit_warp(accum);
        else
            mbar_arrive_warp(accum);
    }
    if (warp < 4) {
        const bool have = __all_sync(0xffffffffu, mbar_wait(accum, 0, abort) && !*abort);
        tc_fence_after();
        const int row = warp * 32 + lane;  // M index = j * cin + ci
        const int j = row / a.cin, ci = row % a.cin;
        const int k = k0 + j;
        float *dst = a.partials + (((int64_t)blockIdx.y * a.K + k) * a.cin + ci) * a.cout;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (have && steps > 0) {
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (have && j < ng) {
#pragma unroll
                for (int i = 0; i < 16; i += 4)
                    *reinterpret_cast<float4 *>(dst + c0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kWgMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, BN);
    }
    if (threadIdx.x == 0 && *abort) atomicExch(a.err, FVGB_ETIMEOUT);
}

__global__ void wgrad_reduce_f64_kernel(const float *__restrict__ partials, int64_t chunks, int64_t per_chunk,
                                        float *__restrict__ dw) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per_chunk) return;
    double s = 0.0;
    for (int64_t c = 0; c < chunks; ++c) s += (double)partials[c * per_chunk + e];
    dw[e] = (float)s;
}

struct TcWgradPlan {
    int64_t groups, chunks, rows_per_chunk;
};

TcWgradPlan tc_wgrad_plan(int64_t n_out, int32_t K, int32_t cin) {
    TcWgradPlan p;
    const int G = 128 / cin;
    p.groups = ceil_div(K, G);
    const int64_t tiles = ceil_div(n_out > 0 ? n_out : 1, kTileM);
    int64_t chunks = ceil_div(4 * 148, p.groups);
    if (chunks > tiles) chunks = tiles;
    if (chunks < 1) chunks = 1;
    p.rows_per_chunk = ceil_div(tiles, chunks) * kTileM;
    p.chunks = ceil_div(n_out > 0 ? n_out : 1, p.rows_per_chunk);
    return p;
}

template <int BN>
int launch_wgrad(WgArgs a, int64_t groups, int64_t chunks, cudaStream_t s) {
    constexpr int kStage = wg_stage_bytes<BN>();
    int stages = 4;
    const int extra = 1024 + (2 * 4 + 1) * 8 + 32;
    while (stages > 2 && stages * kStage + extra > 227 * 1024) --stages;
    a.stages = stages;
    const int smem = stages * kStage + extra;
    auto kern = conv_tc_wgrad_kernel<BN>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return launch_status();
    kern<<<dim3((unsigned)groups, (unsigned)chunks), kThreads, smem, s>>>(a);
    return launch_status();
}

}  // namespace
}  // namespace fvgb

extern "C" int fvgb_tc_wgrad_workspace(int64_t n_out, int32_t K, int32_t c_in, int32_t c_out, size_t *bytes) {
    if (!bytes || K < 1 || n_out < 0 || (c_in != 32 && c_in != 64 && c_in != 128) ||
        (c_out != 64 && c_out != 128 && c_out != 256))
        return FVGB_EINVAL;
    const TcWgradPlan p = tc_wgrad_plan(n_out, K, c_in);
    *bytes = (size_t)p.chunks * K * c_in * c_out * 4 + 256;
    return FVGB_OK;
}

extern "C" int fvgb_conv_wgrad_tc(const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map,
                                  int64_t n_out, int32_t K, const uint32_t *tile_mask, const void *dy, int32_t c_out,
                                  int64_t lddy, float *dw, void *workspace, size_t workspace_bytes, int32_t *err_dev,
                                  fvgb_stream_t stream) {
    size_t need = 0;
    int st = fvgb_tc_wgrad_workspace(n_out, K, c_in, c_out, &need);
    if (st) return st;
    if (!dw || !err_dev || ldx < c_in || lddy < c_out || (ldx % 8) || (lddy % 8) || n_x < 0) return FVGB_EINVAL;
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    if (((uintptr_t)x & 15) || ((uintptr_t)dy & 15)) return FVGB_EINVAL;
    const TcWgradPlan p = tc_wgrad_plan(n_out, K, c_in);
    cudaStream_t s = as_stream(stream);
    float *part = reinterpret_cast<float *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    const int64_t per_chunk = (int64_t)K * c_in * c_out;
    int launched = 0;
    if (n_out > 0) {
        WgArgs a;
        a.x = (const uint8_t *)(n_x > 0 ? x : dy);
        a.n_x = n_x;
        a.ldx_bytes = ldx * 2;
        a.cin = c_in;
        a.map = map;
        a.n_out = n_out;
        a.K = K;
        a.tile_mask = tile_mask;
        a.dy = (const uint8_t *)dy;
        a.lddy_bytes = lddy * 2;
        a.cout = c_out;
        a.rows_per_chunk = p.rows_per_chunk;
        a.partials = part;
        a.err = err_dev;
        a.stages = 0;
        if (p.chunks > 65535) return FVGB_EINVAL;
        switch (c_out) {
            case 64: st = launch_wgrad<64>(a, p.groups, p.chunks, s); break;
            case 128: st = launch_wgrad<128>(a, p.groups, p.chunks, s); break;
            default: st = launch_wgrad<256>(a, p.groups, p.chunks, s); break;
        }
        if (st) return st;
        launched = 1;
    }
    wgrad_reduce_f64_kernel<<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>(part, n_out > 0 ? p.chunks : 0,
                                                                               per_chunk, dw);
    count_launches(launched + 1);
    return launch_status();
}

namespace fvgb {
namespace {
// One CTA: thread 0 waits on an mbarrier phase with the same bounded wait the tensor-core
// kernels use.  Without `arrive` nothing completes the phase, so the wait must give up after
// `budget` cycles and report FVGB_ETIMEOUT; with `arrive` the phase is already complete.
__global__ void selftest_wait_kernel(int32_t *err, long long budget, int32_t arrive) {
    __shared__ uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        abort_flag = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (arrive) tc::mbar_arrive(&bar);
        if (!tc::mbar_wait_budget(&bar, 0, &abort_flag, budget)) atomicExch(err, FVGB_ETIMEOUT);
    }
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_selftest_wait_timeout(int32_t *err_dev, int64_t budget_cycles, int32_t arrive,
                                          fvgb_stream_t stream) {
    if (!err_dev || budget_cycles < 1 || budget_cycles > ((int64_t)1 << 32)) return FVGB_EINVAL;
    fvgb::selftest_wait_kernel<<<1, 32, 0, fvgb::as_stream(stream)>>>(err_dev, (long long)budget_cycles, arrive);
    fvgb::count_launches(1);
    return fvgb::launch_status();
}
