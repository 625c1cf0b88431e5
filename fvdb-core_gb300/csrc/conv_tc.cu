// Tensor-core (tcgen05 / TMEM) implicit-GEMM sparse convolution for sm_103a.
//
//   y[m, :] = scale * sum_k x[map[m,k], :] . W[k]        (BF16 or FP8-E4M3 in, FP32 accumulate)
//
// One CTA owns 128 output rows and all (<= 256) output channels, so every output row is
// written exactly once, without atomics.  The reduction dimension runs over (offset k,
// channel chunk c); offsets whose 128 map entries are all -1 (per-tile occupancy mask from
// the kernel-map build) are skipped.
//
// Warp roles (160 threads):
//   warps 0-3  gather: thread r owns row r of the tile; per step it reads map[m0+r, k] from
//              shared memory and issues 16-byte cp.async copies of the gathered feature row
//              straight into the 128B-swizzled K-major operand layout (zero-filled where the
//              map is -1), then arrives on the stage's mbarrier when its copies land.  Thread 0
//              also fetches the stage's weight tile with one bulk async copy of a pre-packed,
//              pre-swizzled image.  After the main loop these warps are the epilogue: TMEM ->
//              registers (tcgen05.ld) -> scale/convert -> global.
//   warp 4     TMEM allocation and the single MMA-issuing thread (tcgen05.mma M=128, N=BN).
//
// Reference kernels replaced: conv_forward_cuda_setting{1,2,3}_mode{0,1}_{bf16,f16,tf32,f32}
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMM.cu:120-3826 and
// SparseConvolutionImplicitGEMMSorted.cu:115-4639), sm_80 mma.sync code.
#include <cuda_bf16.h>

#include "tc_common.cuh"

namespace fvgb {
namespace {

using namespace tc;

constexpr int kTileM = 128;
constexpr int kRowBytes = 128;  // one swizzle row = 64 bf16 or 128 fp8 elements
constexpr int kThreads = 160;
constexpr int kABytes = kTileM * kRowBytes;

struct TcArgs {
    const uint8_t *x;
    int64_t n_x;
    int64_t ldx_bytes;
    int32_t cin;
    const int32_t *map;
    int64_t n_out;
    int32_t K;
    const uint32_t *tile_mask;  // may be null (or K > 32): no skipping
    const uint8_t *wpack;       // [K][nchunks][BN rows][128 B]
    int32_t nchunks;
    int32_t cout;
    uint8_t *y;                 // bf16 [n_out, ldy]
    int64_t ldy;
    const float *scale;         // per output channel, may be null
    int32_t *err;
    int32_t stages;
    int32_t stage_map;          // 1: map tile staged in shared memory (K <= 32)
};

template <int BN>
__host__ __device__ constexpr int stage_bytes() {
    return kABytes + BN * kRowBytes;
}

// ebytes: element size (2 = bf16, 1 = e4m3)
template <int BN, int EBYTES>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_fwd_kernel(TcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kStage = stage_bytes<BN>();
    const int S = a.stages;
    int32_t *map_tile = reinterpret_cast<int32_t *>(smem + S * kStage);
    uint64_t *bars = reinterpret_cast<uint64_t *>(map_tile + (a.stage_map ? kTileM * a.K : 0));
    uint64_t *full = bars, *empty = bars + S, *accum = bars + 2 * S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kTileM;
    constexpr uint32_t kTmemCols = BN < 32 ? 32 : BN;
    constexpr int kChunkElems = kRowBytes / EBYTES;

    const uint32_t kbits = a.K >= 32 ? 0xffffffffu : ((1u << a.K) - 1u);
    const uint32_t tmask = (a.tile_mask && a.K <= 32) ? (a.tile_mask[blockIdx.x] & kbits) : kbits;
    const int n_k = a.K <= 32 ? __popc(tmask) : a.K;
    const int n_steps = n_k * a.nchunks;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], kTileM + 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort = 0;
    }
    if (warp == 4) tmem_alloc(tmem_slot, kTmemCols);
    if (a.stage_map) {
        for (int e = threadIdx.x; e < kTileM * a.K; e += kThreads) {
            const int64_t row = m0 + e / a.K;
            int32_t v = row < a.n_out ? a.map[row * a.K + (e % a.K)] : -1;
            map_tile[e] = (v >= 0 && v < a.n_x) ? v : -1;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < 4) {
        // ------------------------------------------------------------- gather producer
        const int r = threadIdx.x;
        const int64_t row = m0 + r;
        uint32_t kb = tmask;
        int it = 0;
        for (int kk = 0; kk < n_k && !*abort; ++kk) {
            int k;
            if (a.K <= 32) {
                k = __ffs(kb) - 1;
                kb &= kb - 1;
            } else {
                k = kk;
            }
            int32_t src;
            if (a.stage_map) {
                src = map_tile[r * a.K + k];
            } else {
                src = row < a.n_out ? a.map[row * a.K + k] : -1;
                if (src >= a.n_x) src = -1;
            }
            const uint8_t *src_row = src >= 0 ? a.x + (int64_t)src * a.ldx_bytes : a.x;
            for (int c = 0; c < a.nchunks; ++c, ++it) {
                const int stage = it % S;
                if (!mbar_wait(&empty[stage], ((it / S) & 1) ^ 1, abort)) break;
                uint8_t *As = smem + stage * kStage;
                const int width = min(kChunkElems, a.cin - c * kChunkElems);
                const int nch = (width * EBYTES) >> 4;
                const uint32_t dst = smem_u32(As);
                for (int j = 0; j < nch; ++j) {
                    const uint8_t *g = src >= 0 ? src_row + (int64_t)c * kRowBytes + j * 16 : a.x;
                    cp_async_16(dst + sw128_offset(r, j), g, src >= 0 ? 16u : 0u);
                }
                cp_async_arrive_noinc(&full[stage]);
                if (r == 0) {
                    mbar_arrive_expect_tx(&full[stage], BN * kRowBytes);
                    bulk_g2s(dst + kABytes, a.wpack + ((int64_t)k * a.nchunks + c) * (BN * kRowBytes), BN * kRowBytes,
                             &full[stage]);
                }
            }
        }
        cp_async_wait_all();
    } else if (warp == 4 && lane == 0) {
        // ------------------------------------------------------------- MMA issuer
        constexpr uint32_t idesc = EBYTES == 2 ? idesc_m128(BN, 1, 1) : idesc_m128(BN, 0, 0);
        int it = 0;
        bool ok = true;
        for (int kk = 0; kk < n_k && ok; ++kk) {
            for (int c = 0; c < a.nchunks; ++c, ++it) {
                const int stage = it % S;
                if (!mbar_wait(&full[stage], (it / S) & 1, abort)) {
                    ok = false;
                    break;
                }
                fence_proxy_async();
                tc_fence_after();
                const uint32_t As = smem_u32(smem + stage * kStage);
                const uint32_t Bs = As + kABytes;
                const int width = min(kChunkElems, a.cin - c * kChunkElems);
                const int nmma = (width * EBYTES) >> 5;  // 32 bytes of K per MMA
                for (int q = 0; q < nmma; ++q) {
                    const uint64_t ad = desc_sw128(As + q * 32), bd = desc_sw128(Bs + q * 32);
                    if (EBYTES == 2)
                        mma_f16(tmem, ad, bd, idesc, (it > 0 || q > 0) ? 1u : 0u);
                    else
                        mma_f8(tmem, ad, bd, idesc, (it > 0 || q > 0) ? 1u : 0u);
                }
                mma_commit(&empty[stage]);
            }
        }
        if (n_steps > 0 && it > 0)
            mma_commit(accum);
        else
            mbar_arrive(accum);
    }

    if (warp < 4) {
        // ------------------------------------------------------------- epilogue
        // warp-uniform: tcgen05.ld below is a .sync.aligned warp instruction
        const bool have = __all_sync(0xffffffffu, mbar_wait(accum, 0, abort) && !*abort);
        tc_fence_after();
        const int r = warp * 32 + lane;
        const int64_t row = m0 + r;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        __nv_bfloat16 *yrow = reinterpret_cast<__nv_bfloat16 *>(a.y) + row * a.ldy;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (n_steps > 0 && have) {
                tmem_ld16(tbase + c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (row < a.n_out && have) {
                if (c0 + 16 <= a.cout && (a.ldy % 8) == 0) {
                    uint32_t packed[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        float lo = v[2 * i], hi = v[2 * i + 1];
                        if (a.scale) {
                            lo *= a.scale[c0 + 2 * i];
                            hi *= a.scale[c0 + 2 * i + 1];
                        }
                        __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
                        packed[i] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(yrow + c0);
                    dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                } else {
                    for (int i = 0; i < 16 && c0 + i < a.cout; ++i)
                        yrow[c0 + i] = __float2bfloat16_rn(a.scale ? v[i] * a.scale[c0 + i] : v[i]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
    if (threadIdx.x == 0 && *abort) atomicExch(a.err, FVGB_ETIMEOUT);
}

// Packed weight image: for every (k, chunk c): BN rows (output channel n) x 128 bytes holding
// W[k][c*CE + e][n] for e in [0, CE) (CE = 128/ebytes), laid out exactly as the 128B-swizzled
// K-major shared-memory operand (zero where c*CE+e >= cin or n >= cout).
__global__ void pack_weights_kernel(const uint8_t *__restrict__ w, int64_t K, int32_t cin, int32_t cout,
                                    int64_t wsk, int64_t wsci, int64_t wsco, int32_t ebytes, int32_t BN,
                                    int32_t nchunks, uint8_t *__restrict__ out) {
    const int64_t total = K * nchunks * BN * 128 / ebytes;  // elements of the image
    const int ce = 128 / ebytes;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tilei = e / ((int64_t)BN * ce);
        const int64_t rem = e % ((int64_t)BN * ce);
        const int n = (int)(rem / ce), kk = (int)(rem % ce);
        const int64_t k = tilei / nchunks;
        const int c = (int)(tilei % nchunks);
        const int ci = c * ce + kk;
        const uint32_t byte = (uint32_t)kk * ebytes;
        const uint32_t off = sw128_offset((uint32_t)n, byte >> 4) + (byte & 15);
        uint8_t *dst = out + tilei * (int64_t)BN * 128 + off;
        const bool ok = ci < cin && n < cout;
        const int64_t src = (k * wsk + (int64_t)ci * wsci + (int64_t)n * wsco) * ebytes;
        if (ebytes == 2) {
            *reinterpret_cast<uint16_t *>(dst) = ok ? *reinterpret_cast<const uint16_t *>(w + src) : (uint16_t)0;
        } else {
            *dst = ok ? w[src] : (uint8_t)0;
        }
    }
}

int tile_n(int32_t cout) {
    if (cout <= 32) return 32;
    if (cout <= 64) return 64;
    if (cout <= 128) return 128;
    if (cout <= 256) return 256;
    return -1;
}

template <int BN, int EB>
int launch_fwd(TcArgs a, cudaStream_t s) {
    constexpr int kStage = stage_bytes<BN>();
    const int map_bytes = a.stage_map ? kTileM * a.K * 4 : 0;
    int stages = BN >= 256 ? 4 : (BN >= 128 ? 3 : 4);
    const int extra = 1024 + map_bytes + (2 * 6 + 1) * 8 + 16;
    while (stages > 2 && stages * kStage + extra > 227 * 1024) --stages;
    a.stages = stages;
    const int smem = stages * kStage + extra;
    auto kern = conv_tc_fwd_kernel<BN, EB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return launch_status();
    const int64_t tiles = ceil_div(a.n_out, kTileM);
    kern<<<(unsigned)tiles, kThreads, smem, s>>>(a);
    count_launches(1);
    return launch_status();
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_tc_weight_bytes(int32_t dtype, int64_t K, int32_t cin, int32_t cout, size_t *bytes) {
    if (!bytes || K < 1 || cin < 1 || cout < 1) return FVGB_EINVAL;
    const int eb = dtype == FVGB_E4M3 ? 1 : (dtype == FVGB_BF16 ? 2 : 0);
    if (!eb) return FVGB_ETYPE;
    const int BN = tile_n(cout);
    if (BN < 0) return FVGB_EINVAL;
    const int64_t nchunks = ceil_div((int64_t)cin * eb, 128);
    *bytes = (size_t)(K * nchunks * BN * 128);
    return FVGB_OK;
}

extern "C" int fvgb_tc_pack_weights(int32_t dtype, const void *w, int64_t K, int32_t cin, int32_t cout, int64_t wsk,
                                    int64_t wsci, int64_t wsco, void *packed, size_t packed_bytes,
                                    fvgb_stream_t stream) {
    size_t need = 0;
    int st = fvgb_tc_weight_bytes(dtype, K, cin, cout, &need);
    if (st) return st;
    if (!w || !packed || packed_bytes < need) return FVGB_EINVAL;
    const int eb = dtype == FVGB_E4M3 ? 1 : 2;
    const int BN = tile_n(cout);
    const int nchunks = (int)ceil_div((int64_t)cin * eb, 128);
    const int64_t total = (int64_t)need / eb;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(total, 256), 4096);
    pack_weights_kernel<<<blocks, 256, 0, as_stream(stream)>>>((const uint8_t *)w, K, cin, cout, wsk, wsci, wsco, eb, BN,
                                                               nchunks, (uint8_t *)packed);
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_conv_fwd_tc(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                const int32_t *map, int64_t n_out, int32_t K, const uint32_t *tile_mask,
                                const void *packed_w, int32_t c_out, void *y, int64_t ldy, const float *out_scale,
                                int32_t *err_dev, fvgb_stream_t stream) {
    const int eb = dtype == FVGB_E4M3 ? 1 : (dtype == FVGB_BF16 ? 2 : 0);
    if (!eb) return FVGB_ETYPE;
    if (c_in < 1 || c_out < 1 || K < 1 || n_out < 0 || n_x < 0 || ldx < c_in || ldy < c_out || !err_dev)
        return FVGB_EINVAL;
    // each MMA consumes 32 bytes of K and every gathered row is copied in 16-byte pieces
    if (((int64_t)c_in * eb) % 32 != 0 || (ldx * eb) % 16 != 0) return FVGB_EINVAL;
    const int BN = tile_n(c_out);
    if (BN < 0) return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    if (!map || !packed_w || !y || (n_x > 0 && !x)) return FVGB_EINVAL;
    if (((uintptr_t)x & 15) || ((uintptr_t)packed_w & 15) || ((uintptr_t)y & 15)) return FVGB_EINVAL;
    TcArgs a;
    // with no input rows every map entry is -1 and nothing is read; keep a valid address anyway
    a.x = (const uint8_t *)(n_x > 0 ? x : y);
    a.n_x = n_x;
    a.ldx_bytes = ldx * eb;
    a.cin = c_in;
    a.map = map;
    a.n_out = n_out;
    a.K = K;
    a.tile_mask = tile_mask;
    a.wpack = (const uint8_t *)packed_w;
    a.nchunks = (int32_t)ceil_div((int64_t)c_in * eb, 128);
    a.cout = c_out;
    a.y = (uint8_t *)y;
    a.ldy = ldy;
    a.scale = out_scale;
    a.err = err_dev;
    a.stages = 0;
    a.stage_map = K <= 32 ? 1 : 0;
    cudaStream_t s = as_stream(stream);
    if (eb == 2) {
        switch (BN) {
            case 32: return launch_fwd<32, 2>(a, s);
            case 64: return launch_fwd<64, 2>(a, s);
            case 128: return launch_fwd<128, 2>(a, s);
            default: return launch_fwd<256, 2>(a, s);
        }
    }
    switch (BN) {
        case 32: return launch_fwd<32, 1>(a, s);
        case 64: return launch_fwd<64, 1>(a, s);
        case 128: return launch_fwd<128, 1>(a, s);
        default: return launch_fwd<256, 1>(a, s);
    }
}
