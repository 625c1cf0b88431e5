// Tensor-core (tcgen05 / TMEM) weight gradient and FP8 quantisation for sm_103a.
// (The forward / data-gradient contraction lives in conv_fwd_tc.cu.)
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "tc_common.cuh"

namespace fvgb {
namespace {

using namespace tc;

constexpr int kTileM = 128;
constexpr int kWgGatherWarps = 8;  // 256 gather threads: cp.async throughput grows with the issuing warps
constexpr int kWgMmaWarp = kWgGatherWarps;

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
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n * c, 256), device_sm_count() * 64);
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
// A CTA owns a block of kernel offsets and a chunk of output rows.  The block's offsets form
// sub-groups of G = 128 / c_in offsets (G x c_in = one M = 128 MMA, MN-major A) and every
// sub-group accumulates in a TMEM accumulator of its own (512 / c_out of them, N = c_out
// columns each).  So a 128-row tile of dy -- one TMA tile load per 64 channels, 128-byte
// swizzle, straight into the MN-major B layout -- is loaded once and feeds every sub-group of
// the block, and the tile's map rows (one bulk copy, K <= 32) feed every sub-group's gather.
// Per (tile, sub-group) the gather warps copy the sub-group's source rows into an A stage;
// sub-groups with none of their offsets in the tile (per-tile occupancy mask) are skipped.
// The epilogue writes the block's partial dW slice in FP32; a second kernel sums the partials
// over chunks in FP64 in a fixed order (deterministic).
//
//   warps 0-7  gather the A operand with cp.async (lane -> 16-byte piece of four 128-byte MN
//              atom rows per instruction), publish each stage one stage late; then the epilogue
//   warp 8     MMA: owns the 512 TMEM columns; one elected lane issues, warp-uniform loop
//   warp 9     loader: per active tile, the dy TMA loads and the map-row bulk copy (double-
//              buffered, released by the tile's last MMA commit and the gather warps)
//
// Replaces the split-K wgrad kernels conv_backward_cuda_setting{1,2}_mode{0,1}_*
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMMGrad.cu:115-4101,
// ...GradSorted.cu:115-4582) and their [32, K*Cin, Cout].sum(0).
namespace fvgb {
namespace {

constexpr int kMNAtom = 16384;  // 128 K-rows x 128 bytes: one 64-element-wide MN atom of a stage
constexpr int kWgLoadWarp = kWgMmaWarp + 1;
constexpr int kWgThreads = (kWgLoadWarp + 1) * 32;
constexpr int kWgMaxMapK = 32;  // map tiles staged in shared memory up to K = 32

__device__ __forceinline__ void st_shared_zero16(uint32_t addr) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(addr), "r"(0) : "memory");
}

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
    const int32_t *map;  // [ceil(n_out/128)*128, K], padding rows -1
    int64_t n_out;
    int32_t K;
    const uint32_t *tile_mask;
    int32_t cout;
    int32_t G;               // offsets per sub-group (128 / cin)
    int32_t offs_per_cta;    // offsets per block (a multiple of G)
    int64_t rows_per_chunk;  // multiple of 128
    float *partials;         // [chunks][K][cin][cout]
    int32_t *err;
    int32_t stages;
    int32_t stage_map;
};

template <int BN>
__global__ void __launch_bounds__(kWgThreads, 1) conv_tc_wgrad_kernel(const __grid_constant__ CUtensorMap dy_map,
                                                                      WgArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kA = 2 * kMNAtom;           // A stage: M = 128 (two MN atoms) x K = 128 rows
    constexpr int kDy = (BN / 64) * kMNAtom;  // dy tile: 128 rows x BN channels
    const int S = a.stages;
    uint8_t *dybuf = smem + S * kA;
    const int map_words = a.stage_map ? kTileM * a.K : 0;  // per buffer
    int32_t *map_sm = reinterpret_cast<int32_t *>(dybuf + 2 * kDy);
    uint64_t *afull = reinterpret_cast<uint64_t *>(map_sm + 2 * map_words);
    uint64_t *aempty = afull + S, *tfull = aempty + S, *tempty = tfull + 2, *accum = tempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = a.G;
    const int k0 = blockIdx.x * a.offs_per_cta;
    const int k_end = min(a.K, k0 + a.offs_per_cta);
    const int nsg = (k_end - k0 + G - 1) / G;  // sub-groups of this block, <= 512 / BN
    const int64_t r_begin = (int64_t)blockIdx.y * a.rows_per_chunk;
    const int64_t r_end = min(a.n_out, r_begin + a.rows_per_chunk);
    const int64_t t_begin = r_begin / kTileM;
    const int64_t n_tiles = (r_end - r_begin + kTileM - 1) / kTileM;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&afull[s], kWgGatherWarps);  // one arrival per gather warp
            mbar_init(&aempty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 1 + kWgGatherWarps);  // the tile's last MMA commit + each gather warp
        }
        mbar_init(accum, 1);
        *abort = 0;
    }
    if (warp == kWgMmaWarp) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // sub-groups (bit g) of chunk tile t with at least one of their offsets present
    auto groups_of = [&](int64_t t) -> uint32_t {
        const uint32_t all = (1u << nsg) - 1u;
        if (!a.tile_mask || a.K > 32) return all;
        const uint32_t m = __ldg(a.tile_mask + t_begin + t);
        uint32_t r = 0;
        for (int g = 0; g < nsg; ++g) {
            const int kk = k0 + g * G, cnt = min(G, a.K - kk);
            if ((m >> kk) & ((1u << cnt) - 1u)) r |= 1u << g;
        }
        return r;
    };

    if (warp < kWgGatherWarps) {
        // Lane -> (16-byte piece jj of a 128-byte MN atom row, K-rows rsub + 4q of this warp's
        // 16): one warp instruction moves four whole 128-byte atom rows.  Atom `at` of the A
        // operand holds M elements at*64 .. at*64+63, i.e. sub-group offset (at*64 + 8*jj) / cin
        // at channel (at*64 + 8*jj) % cin.
        const int jj = lane & 7, rsub = lane >> 3, row0 = warp * (kTileM / kWgGatherWarps);
        int joff[2], ci0[2];
#pragma unroll
        for (int at = 0; at < 2; ++at) {
            const int m0 = at * 64 + jj * 8;
            joff[at] = m0 / a.cin;
            ci0[at] = m0 - joff[at] * a.cin;
        }
        uint32_t it = 0, sig = 0, stage = 0, phase = 0, pstage = 0, seen = 0;
        int i = 0;
        bool ok = true;
        for (int64_t t = 0; t < n_tiles && ok && !*abort; ++t) {
            uint32_t gm = groups_of(t);
            if (!gm) continue;
            seen |= gm;
            const int b = i & 1;
            if (a.stage_map && !mbar_wait_warp(&tfull[b], (i >> 1) & 1, abort)) break;
            const int32_t *mt = map_sm + b * map_words;
            const int64_t mrow0 = r_begin + t * kTileM;
            while (gm) {
                const int g = __ffs(gm) - 1;
                gm &= gm - 1;
                int32_t src[2][4];
#pragma unroll
                for (int at = 0; at < 2; ++at)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int r = row0 + rsub + 4 * q;
                        const int k = k0 + g * G + joff[at];
                        int32_t v = -1;
                        if (k < k_end) {
                            v = a.stage_map ? mt[r * a.K + k] : a.map[(mrow0 + r) * a.K + k];
                            if (v >= a.n_x) v = -1;
                        }
                        src[at][q] = v;
                    }
                if (!mbar_wait_warp(&aempty[stage], phase ^ 1, abort)) {
                    ok = false;
                    break;
                }
                const uint32_t base = smem_u32(smem + stage * kA);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = row0 + rsub + 4 * q;
#pragma unroll
                    for (int at = 0; at < 2; ++at) {
                        const uint32_t dst = base + mn_offset(r, at * 64 + jj * 8);
                        if (src[at][q] >= 0)
                            cp_async_16(dst, a.x + (int64_t)src[at][q] * a.ldx_bytes + ci0[at] * 2, 16u);
                        else
                            st_shared_zero16(dst);
                    }
                }
                // cp.async and st.shared are generic-proxy writes: each warp fences its own
                // copies to the tensor core (async proxy), one stage late
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
                    if (lane == 0) mbar_arrive(&afull[pstage]);
                    ++sig;
                    if (++pstage == (uint32_t)S) pstage = 0;
                }
            }
            // the tile's map rows were read into registers: release its buffers (with the MMA)
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
            ++i;
        }
        cp_async_wait_group<0>();
        fence_proxy_async();
        __syncwarp();
        if (lane == 0)
            for (; sig < it; ++sig) {
                mbar_arrive(&afull[pstage]);
                if (++pstage == (uint32_t)S) pstage = 0;
            }

        // ---------------------------------------------------------------- epilogue
        const bool have = __all_sync(0xffffffffu, mbar_wait(accum, 0, abort) && !*abort);
        tc_fence_after();
        const int lg = warp & 3;
        const int row = lg * 32 + lane;  // M index = j * cin + ci
        const int j = row / a.cin, ci = row % a.cin;
        for (int g = warp >> 2; g < nsg; g += 2) {
            const int k = k0 + g * G + j;
            const bool mine = have && k < k_end;
            const bool live = have && ((seen >> g) & 1u);  // warp-uniform
            float *dst = a.partials + (((int64_t)blockIdx.y * a.K + k) * a.cin + ci) * a.cout;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 16) {
                float v[16];
                if (live) {
                    tmem_ld16(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(g * BN + c0), v);
                } else {
#pragma unroll
                    for (int e = 0; e < 16; ++e) v[e] = 0.f;
                }
                if (mine) {
#pragma unroll
                    for (int e = 0; e < 16; e += 4)
                        *reinterpret_cast<float4 *>(dst + c0 + e) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
                }
            }
        }
    } else if (warp == kWgMmaWarp) {
        // the whole warp runs the issue loop (warp-uniform); one elected lane issues each tcgen05 op
        constexpr uint32_t idesc = idesc_m128(BN, 1, 1) | (1u << 15) | (1u << 16);  // bf16, A and B MN-major
        uint32_t inited = 0;
        int it = 0, i = 0;
        bool ok = true;
        for (int64_t t = 0; t < n_tiles && ok; ++t) {
            uint32_t gm = groups_of(t);
            if (!gm) continue;
            const int b = i & 1;
            if (!mbar_wait_warp(&tfull[b], (i >> 1) & 1, abort)) break;
            const uint32_t Bs = smem_u32(dybuf + b * kDy);
            while (gm) {
                const int g = __ffs(gm) - 1;
                gm &= gm - 1;
                const int stage = it % S;
                if (!mbar_wait_warp(&afull[stage], (it / S) & 1, abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t As = smem_u32(smem + stage * kA);
                const uint32_t d = tmem + (uint32_t)(g * BN);
                const uint32_t acc = (inited >> g) & 1u;
#pragma unroll
                for (int q = 0; q < kTileM / 16; ++q)  // 16 rows of K per MMA = two 8-row groups
                    mma_f16_warp(d, desc_sw128_mn(As + q * 2048), desc_sw128_mn(Bs + q * 2048), idesc,
                                 (acc || q > 0) ? 1u : 0u);
                inited |= 1u << g;
                mma_commit_warp(&aempty[stage]);
                ++it;
            }
            if (!ok) break;
            mma_commit_warp(&tempty[b]);  // dy tile consumed once these MMAs complete
            ++i;
        }
        // it == 0: nothing accumulated -- the epilogue writes zeros
        if (it > 0)
            mma_commit_warp(accum);
        else
            mbar_arrive_warp(accum);
    } else {
        // ---------------------------------------------------------------- loader
        if (lane == 0) {
            const uint32_t map_bytes = (uint32_t)map_words * 4;
            int i = 0;
            for (int64_t t = 0; t < n_tiles && !*abort; ++t) {
                if (!groups_of(t)) continue;
                const int b = i & 1;
                if (!mbar_wait_backoff(&tempty[b], ((i >> 1) & 1) ^ 1, abort, 64)) break;
                const int64_t m0 = r_begin + t * kTileM;
                mbar_arrive_expect_tx(&tfull[b], (uint32_t)kDy + map_bytes);
#pragma unroll
                for (int at = 0; at < BN / 64; ++at)
                    tma_load_2d(smem_u32(dybuf + b * kDy + at * kMNAtom), &dy_map, at * 64, (int32_t)m0, &tfull[b]);
                if (map_bytes) bulk_g2s(smem_u32(map_sm + b * map_words), a.map + m0 * a.K, map_bytes, &tfull[b]);
                ++i;
            }
            // the copies issued last land before the CTA exits (bounded: ~30 ms)
            for (int j = i > 2 ? i - 2 : 0; j < i; ++j) {
                int give_up = 0;
                mbar_wait_budget(&tfull[j & 1], (j >> 1) & 1, &give_up, 1ll << 26);
            }
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kWgMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
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
    int64_t blocks, chunks, rows_per_chunk;
    int32_t G, offs_per_cta;
};

// Offset blocks of balanced sub-group counts (<= 512 / c_out accumulators each), then row chunks
// so that blocks x chunks fills the SMs once.
TcWgradPlan tc_wgrad_plan(int64_t n_out, int32_t K, int32_t cin, int32_t cout) {
    TcWgradPlan p;
    p.G = 128 / cin;
    const int64_t subgroups = ceil_div(K, p.G), per_block_max = 512 / cout;
    const int64_t blocks0 = ceil_div(subgroups, per_block_max);
    p.offs_per_cta = (int32_t)(ceil_div(subgroups, blocks0) * p.G);
    p.blocks = ceil_div(K, p.offs_per_cta);
    const int64_t tiles = ceil_div(n_out > 0 ? n_out : 1, kTileM);
    int64_t chunks = ceil_div(device_sm_count(), p.blocks);
    if (chunks > tiles) chunks = tiles;
    if (chunks < 1) chunks = 1;
    p.rows_per_chunk = ceil_div(tiles, chunks) * kTileM;
    p.chunks = ceil_div(n_out > 0 ? n_out : 1, p.rows_per_chunk);
    return p;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

template <int BN>
int launch_wgrad(const CUtensorMap &dy_map, WgArgs a, int64_t blocks, int64_t chunks, cudaStream_t s) {
    constexpr int kA = 2 * kMNAtom, kDy = (BN / 64) * kMNAtom;
    const int map_bytes = a.stage_map ? 2 * kTileM * a.K * 4 : 0;
    const int extra = 1024 + map_bytes + (2 * 4 + 4 + 1) * 8 + 16;
    int stages = 4;
    while (stages > 2 && stages * kA + 2 * kDy + extra > 227 * 1024) --stages;
    if (stages * kA + 2 * kDy + extra > 227 * 1024) return FVGB_EINVAL;
    a.stages = stages;
    const int smem = stages * kA + 2 * kDy + extra;
    auto kern = conv_tc_wgrad_kernel<BN>;
    if (set_dynamic_smem(kern, smem) != cudaSuccess)
        return launch_status();
    kern<<<dim3((unsigned)blocks, (unsigned)chunks), kWgThreads, smem, s>>>(dy_map, a);
    return launch_status();
}

}  // namespace
}  // namespace fvgb

extern "C" int fvgb_tc_wgrad_workspace(int64_t n_out, int32_t K, int32_t c_in, int32_t c_out, size_t *bytes) {
    if (!bytes || K < 1 || n_out < 0 || (c_in != 32 && c_in != 64 && c_in != 128) ||
        (c_out != 64 && c_out != 128 && c_out != 256))
        return FVGB_EINVAL;
    const TcWgradPlan p = tc_wgrad_plan(n_out, K, c_in, c_out);
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
    if (n_out > 0 && (!map || !dy)) return FVGB_EINVAL;
    if (n_out > INT32_MAX - kTileM) return FVGB_EINVAL;
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    if (((uintptr_t)x & 15) || ((uintptr_t)dy & 15) || ((uintptr_t)map & 15)) return FVGB_EINVAL;
    const TcWgradPlan p = tc_wgrad_plan(n_out, K, c_in, c_out);
    cudaStream_t s = as_stream(stream);
    float *part = reinterpret_cast<float *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    const int64_t per_chunk = (int64_t)K * c_in * c_out;
    int launched = 0;
    if (n_out > 0) {
        // dy as a 2-D tensor [n_out rows, c_out channels], boxes of 128 rows x 64 channels,
        // 128-byte swizzle: each box is one MN atom of the B operand; rows past n_out read zero
        EncodeTiledFn enc = encode_tiled();
        if (!enc) {
            record_message("cuTensorMapEncodeTiled is not available from the CUDA driver");
            return FVGB_ECUDA;
        }
        CUtensorMap dy_map;
        const cuuint64_t gdim[2] = {(cuuint64_t)c_out, (cuuint64_t)n_out};
        const cuuint64_t gstride[1] = {(cuuint64_t)lddy * 2};
        const cuuint32_t box[2] = {64, (cuuint32_t)kTileM};
        const cuuint32_t estride[2] = {1, 1};
        if (enc(&dy_map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(dy), gdim, gstride, box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
            record_message("cuTensorMapEncodeTiled rejected the dy tensor");
            return FVGB_EINVAL;
        }
        WgArgs a;
        a.x = (const uint8_t *)(n_x > 0 ? x : dy);
        a.n_x = n_x;
        a.ldx_bytes = ldx * 2;
        a.cin = c_in;
        a.map = map;
        a.n_out = n_out;
        a.K = K;
        a.tile_mask = tile_mask;
        a.cout = c_out;
        a.G = p.G;
        a.offs_per_cta = p.offs_per_cta;
        a.rows_per_chunk = p.rows_per_chunk;
        a.partials = part;
        a.err = err_dev;
        a.stages = 0;
        a.stage_map = K <= kWgMaxMapK ? 1 : 0;
        if (p.chunks > 65535 || p.blocks > 65535) return FVGB_EINVAL;
        switch (c_out) {
            case 64: st = launch_wgrad<64>(dy_map, a, p.blocks, p.chunks, s); break;
            case 128: st = launch_wgrad<128>(dy_map, a, p.blocks, p.chunks, s); break;
            default: st = launch_wgrad<256>(dy_map, a, p.blocks, p.chunks, s); break;
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
