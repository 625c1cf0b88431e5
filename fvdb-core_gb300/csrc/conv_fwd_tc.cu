// Tensor-core (tcgen05 / TMEM) implicit-GEMM sparse convolution, forward and data gradient.
//
//   y[m, :] = scale (.) sum_k x[map[m,k], :] . W[k]       (BF16 or FP8-E4M3 in, FP32 accumulate)
//
// Persistent kernel, one CTA per SM, looping over 128-row output tiles (tile t = blockIdx.x +
// i * gridDim.x).  Each tile owns all (<= 256) output channels, so every output row is written
// exactly once, without atomics.  The reduction dimension runs over (kernel offset, 128-byte
// channel chunk); when a feature row is shorter than 128 bytes (c_in*elem = 64 or 32 bytes),
// two or four kernel offsets share one 128-byte swizzle row of the A operand.  Offsets absent
// from all 128 rows of a tile (per-tile occupancy mask) are skipped.
//
// Warp roles (320 threads):
//   warps 0-3  gather: thread r owns row r of the tile.  Per step it issues 16-byte cp.async
//              copies (L2 evict_last: the input features stay L2-resident while the map and
//              output stream) of the gathered feature rows into the 128B-swizzled K-major A
//              layout, zero-filled where the map is -1.  cp.async writes belong to the generic
//              proxy, so each thread publishes a stage to the tensor core (async proxy) itself,
//              kLag steps late: cp.async.wait_group, fence.proxy.async, then mbarrier arrive.
//              The MMA thread therefore never fences and its MMAs stream back to back.
//   warp 4     TMEM allocation (2 x N columns) and the single MMA-issuing thread; tile i
//              accumulates into TMEM buffer i % 2.
//   warps 5-8  epilogue: tcgen05.ld of the finished buffer -> scale -> BF16 -> a shared-memory
//              copy of the output tile -> one bulk async store of the tile's contiguous rows;
//              overlaps the next tile's main loop.
//   warp 9     loader: bulk async copies of each tile's map rows (double-buffered) and of each
//              step's pre-packed, pre-swizzled weight tiles.
//
// Every mbarrier wait is bounded (about a second); on expiry the CTA stops, waits for its
// issued work, frees TMEM and raises *err = FVGB_ETIMEOUT.
//
// Reference kernels replaced: conv_forward_cuda_setting{1,2,3}_mode{0,1}_{bf16,f16,tf32,f32}
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMM.cu:120-3826,
// SparseConvolutionImplicitGEMMSorted.cu:115-4639), sm_80 mma.sync code.
#include <cuda_bf16.h>

#include <mutex>

#include "tc_common.cuh"

namespace fvgb {
namespace {

using namespace tc;

constexpr int kTileM = 128;
constexpr int kRowBytes = 128;  // one swizzle row = 64 bf16 or 128 fp8 elements
constexpr int kABytes = kTileM * kRowBytes;
constexpr int kThreads = 320;  // 4 gather + 1 MMA + 4 epilogue + 1 loader warps
constexpr int kMaxMapStage = 32;  // map tiles staged in shared memory up to K = 32
constexpr int kLag = 2;  // cp.async groups a gather thread keeps in flight before publishing a stage

struct FwdArgs {
    const uint8_t *x;
    int64_t n_x;
    int64_t ldx_bytes;
    int32_t cin;
    const int32_t *map;  // [ceil(n_out/128)*128, K], padding rows -1
    int64_t n_out;
    int32_t K;
    const uint32_t *tile_mask;  // may be null (or K > 32): no skipping
    const uint8_t *wpack;       // [K][nchunks][BN rows][128 B]
    int32_t nchunks;
    int32_t pack;        // kernel offsets per 128-byte A row (1, 2 or 4); pack > 1 => nchunks == 1
    int32_t row_bytes;   // c_in * elem
    int32_t cout;
    uint8_t *y;          // bf16 [n_out, ldy]
    int64_t ldy;
    const float *scale;  // per output channel, may be null
    int32_t *err;
    int32_t stages;
    int64_t n_tiles;
    int32_t direct_store;  // 1: output rows contiguous (ldy == cout, cout % 8 == 0): one bulk store per tile
};

struct Steps {
    uint32_t kbits;  // active offsets (K <= 32)
    int n_act;       // number of active offsets
    int n_steps;
};

__device__ __forceinline__ uint32_t load_mask(const FwdArgs &a, int64_t tile) {
    if (a.K > 32) return 0;
    const uint32_t all = a.K == 32 ? 0xffffffffu : ((1u << a.K) - 1u);
    return a.tile_mask ? (__ldg(a.tile_mask + tile) & all) : all;
}

__device__ __forceinline__ Steps make_steps(const FwdArgs &a, uint32_t mask) {
    Steps s;
    if (a.K <= 32) {
        s.kbits = mask;
        s.n_act = __popc(mask);
    } else {
        s.kbits = 0;
        s.n_act = a.K;
    }
    s.n_steps = a.pack > 1 ? (s.n_act + a.pack - 1) / a.pack : s.n_act * a.nchunks;
    return s;
}

// Walks the (offset, chunk) sequence of a tile; next() returns the offsets of one step.
struct StepWalker {
    uint32_t kb;
    int k_lin;  // offset counter when K > 32
    int chunk;
    int cur_k;
    __device__ __forceinline__ int pop(const FwdArgs &a) {
        if (a.K <= 32) {
            if (!kb) return -1;
            const int k = __ffs(kb) - 1;
            kb &= kb - 1;
            return k;
        }
        return k_lin < a.K ? k_lin++ : -1;
    }
    // fills ks[0..pack) (-1 for absent) and the chunk index
    __device__ __forceinline__ void next(const FwdArgs &a, int (&ks)[4], int &c) {
        if (a.pack > 1) {
#pragma unroll
            for (int p = 0; p < 4; ++p) ks[p] = p < a.pack ? pop(a) : -1;
            c = 0;
            return;
        }
        if (chunk == 0) cur_k = pop(a);
        ks[0] = cur_k;
        ks[1] = ks[2] = ks[3] = -1;
        c = chunk;
        chunk = (chunk + 1 == a.nchunks) ? 0 : chunk + 1;
    }
};

template <int BN, int EBYTES>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_fwd_kernel(FwdArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kBTile = BN * kRowBytes;
    const int S = a.stages;
    const int kStage = kABytes + a.pack * kBTile;
    const bool stage_map = a.K <= kMaxMapStage;
    const int map_words = stage_map ? kTileM * a.K : 0;  // per buffer; 512*K bytes, 16-byte aligned
    int32_t *map_sm = reinterpret_cast<int32_t *>(smem + S * kStage);
    uint8_t *ystage = reinterpret_cast<uint8_t *>(map_sm + 2 * map_words);  // [128 rows x cout] bf16
    uint64_t *bars = reinterpret_cast<uint64_t *>(ystage + (a.direct_store ? kTileM * BN * 2 : 0));
    uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = tfull + 2, *mfull = tempty + 2,
             *mempty = mfull + 2, *fin = mempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr uint32_t kTmemCols = 2 * BN;
    const int64_t stride = gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], kTileM + 1);  // 128 gather threads + the loader's expect_tx
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kTileM);
            mbar_init(&mfull[b], 1);
            mbar_init(&mempty[b], kTileM);
        }
        mbar_init(fin, 1);
        *abort = 0;
    }
    if (warp == 4) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < 4) {
        // ----------------------------------------------------------------- gather (A operand)
        const int r = threadIdx.x;
        const uint64_t keep = policy_evict_last();
        uint32_t it = 0, sig = 0;
        int64_t tile = blockIdx.x;
        uint32_t mask_cur = tile < a.n_tiles ? load_mask(a, tile) : 0;
        for (int i = 0; tile < a.n_tiles && !*abort; tile += stride, ++i) {
            const uint32_t mask_next = tile + stride < a.n_tiles ? load_mask(a, tile + stride) : 0;
            const int64_t row = tile * kTileM + r;
            const int mb = i & 1;
            if (stage_map && !mbar_wait(&mfull[mb], (i >> 1) & 1, abort)) break;
            const int32_t *mrow = map_sm + mb * map_words + r * a.K;
            const Steps st = make_steps(a, mask_cur);
            StepWalker w{st.kbits, 0, 0, -1};
            bool ok = true;
            for (int s = 0; s < st.n_steps; ++s) {
                int ks[4], c;
                w.next(a, ks, c);
                const int stage = it % S;
                if (!mbar_wait(&empty[stage], ((it / S) & 1) ^ 1, abort)) {
                    ok = false;
                    break;
                }
                const uint32_t As = smem_u32(smem + stage * kStage);
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    if (p >= a.pack || ks[p] < 0) continue;
                    int32_t src;
                    if (stage_map) {
                        src = mrow[ks[p]];
                    } else {
                        src = row < a.n_out ? a.map[row * a.K + ks[p]] : -1;
                    }
                    if (src >= a.n_x) src = -1;
                    const uint8_t *g = a.x + (src >= 0 ? (int64_t)src * a.ldx_bytes + (int64_t)c * kRowBytes : 0);
                    const int bytes = min(kRowBytes, a.row_bytes - c * kRowBytes);
                    const int j0 = p * (a.row_bytes >> 4);
                    for (int j = 0; j < (bytes >> 4); ++j)
                        cp_async_16_hint(As + sw128_offset(r, j0 + j), g + j * 16, src >= 0 ? 16u : 0u, keep);
                }
                cp_async_commit();
                ++it;
                if (it - sig > kLag) {
                    // the copies of step `sig` have landed: publish them to the async proxy (tcgen05.mma)
                    cp_async_wait_group<kLag>();
                    fence_proxy_async();
                    mbar_arrive(&full[sig % S]);
                    ++sig;
                }
            }
            if (stage_map) mbar_arrive(&mempty[mb]);
            if (!ok) break;
            mask_cur = mask_next;
        }
        cp_async_wait_group<0>();
        fence_proxy_async();
        for (; sig < it; ++sig) mbar_arrive(&full[sig % S]);
    } else if (warp == 4) {
        // ----------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = EBYTES == 2 ? idesc_m128(BN, 1, 1) : idesc_m128(BN, 0, 0);
            uint32_t it = 0;
            bool ok = true;
            int64_t tile = blockIdx.x;
            uint32_t mask_cur = tile < a.n_tiles ? load_mask(a, tile) : 0;
            for (int i = 0; tile < a.n_tiles && ok; tile += stride, ++i) {
                const uint32_t mask_next = tile + stride < a.n_tiles ? load_mask(a, tile + stride) : 0;
                const int b = i & 1;
                if (!mbar_wait(&tempty[b], ((i >> 1) & 1) ^ 1, abort)) break;
                tc_fence_after();
                const uint32_t d = tmem + b * BN;
                const Steps st = make_steps(a, mask_cur);
                StepWalker w{st.kbits, 0, 0, -1};
                uint32_t acc = 0;
                for (int s = 0; s < st.n_steps; ++s, ++it) {
                    int ks[4], c;
                    w.next(a, ks, c);
                    const int stage = it % S;
                    if (!mbar_wait(&full[stage], (it / S) & 1, abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t As = smem_u32(smem + stage * kStage);
                    const int bytes = min(kRowBytes, a.row_bytes - c * kRowBytes);
                    int q = 0;
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        if (p >= a.pack || ks[p] < 0) continue;
                        const uint32_t Ap = As + p * a.row_bytes, Bp = As + kABytes + q * kBTile;
                        for (int h = 0; h < (bytes >> 5); ++h) {  // 32 bytes of K per MMA
                            const uint64_t ad = desc_sw128(Ap + h * 32), bd = desc_sw128(Bp + h * 32);
                            if (EBYTES == 2)
                                mma_f16(d, ad, bd, idesc, acc);
                            else
                                mma_f8(d, ad, bd, idesc, acc);
                            acc = 1;
                        }
                        ++q;
                    }
                    mma_commit(&empty[stage]);
                }
                if (!ok) break;
                if (acc)
                    mma_commit(&tfull[b]);
                else
                    mbar_arrive(&tfull[b]);
                mask_cur = mask_next;
            }
            // all issued MMAs complete before TMEM is released
            mma_commit(fin);
            const long long t0 = clock64();
            while (!mbar_try_wait(fin, 0) && clock64() - t0 < kWaitCycles) {
            }
        }
        __syncwarp();
    } else if (warp < 9) {
        // ----------------------------------------------------------------- epilogue
        const int et = threadIdx.x - 160;  // 0..127
        const int q4 = warp & 3;           // TMEM lane quarter this warp may access
        const int rt = q4 * 32 + lane;     // row of the tile this thread drains
        int64_t tile = blockIdx.x;
        uint32_t mask_cur = tile < a.n_tiles ? load_mask(a, tile) : 0;
        for (int i = 0; tile < a.n_tiles; tile += stride, ++i) {
            const uint32_t mask_next = tile + stride < a.n_tiles ? load_mask(a, tile + stride) : 0;
            const int b = i & 1;
            const bool ready = __all_sync(0xffffffffu, mbar_wait(&tfull[b], (i >> 1) & 1, abort) && !*abort);
            if (!ready) break;
            tc_fence_after();
            const Steps st = make_steps(a, mask_cur);
            const int64_t m0 = tile * kTileM;
            const int64_t left = a.n_out - m0;
            const int rows = left < kTileM ? (int)left : kTileM;
            const uint32_t tbase = tmem + b * BN + ((uint32_t)(q4 * 32) << 16);
            if (a.direct_store) {
                if (et == 0) bulk_wait_read<0>();  // the staging tile of the previous store has been read
                named_barrier(1, kTileM);
            }
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 16) {
                float v[16];
                if (st.n_steps > 0) {
                    tmem_ld16(tbase + c0, v);
                } else {
#pragma unroll
                    for (int t = 0; t < 16; ++t) v[t] = 0.f;
                }
                if (rt >= rows || c0 >= a.cout) continue;
                uint32_t packed[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int cc = c0 + 2 * t;
                    float lo = v[2 * t], hi = v[2 * t + 1];
                    if (a.scale) {
                        lo *= cc < a.cout ? a.scale[cc] : 0.f;
                        hi *= cc + 1 < a.cout ? a.scale[cc + 1] : 0.f;
                    }
                    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
                    packed[t] = *reinterpret_cast<uint32_t *>(&h);
                }
                if (a.direct_store) {
                    // cout % 8 == 0: whole 16-byte groups; the last group of a 16-wide block may be cut
                    uint4 *dst = reinterpret_cast<uint4 *>(ystage + ((size_t)rt * a.cout + c0) * 2);
                    dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    if (c0 + 8 < a.cout) dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                } else {
                    __nv_bfloat16 *yrow = reinterpret_cast<__nv_bfloat16 *>(a.y) + (m0 + rt) * a.ldy;
                    const __nv_bfloat16 *hv = reinterpret_cast<const __nv_bfloat16 *>(packed);
                    for (int t = 0; t < 16 && c0 + t < a.cout; ++t) yrow[c0 + t] = hv[t];
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[b]);
            if (a.direct_store) {
                fence_proxy_async();  // staging writes -> visible to the bulk store (async proxy)
                named_barrier(1, kTileM);
                if (et == 0) {
                    bulk_s2g(a.y + m0 * a.ldy * 2, smem_u32(ystage), (uint32_t)(rows * a.cout * 2));
                    bulk_commit();
                }
            }
            mask_cur = mask_next;
        }
        if (a.direct_store && et == 0) bulk_wait<0>();
    } else {
        // ----------------------------------------------------------------- loader (bulk copies)
        if (lane == 0) {
            uint32_t it = 0;
            int64_t tile = blockIdx.x;
            const uint32_t map_bytes = (uint32_t)map_words * 4;
            if (stage_map && tile < a.n_tiles) {
                mbar_arrive_expect_tx(&mfull[0], map_bytes);
                bulk_g2s(smem_u32(map_sm), a.map + tile * kTileM * a.K, map_bytes, &mfull[0]);
            }
            uint32_t mask_cur = tile < a.n_tiles ? load_mask(a, tile) : 0;
            for (int i = 0; tile < a.n_tiles && !*abort; tile += stride, ++i) {
                const int64_t nxt = tile + stride;
                const uint32_t mask_next = nxt < a.n_tiles ? load_mask(a, nxt) : 0;
                if (stage_map && nxt < a.n_tiles) {
                    const int nb = (i + 1) & 1;
                    if (!mbar_wait(&mempty[nb], (((i + 1) >> 1) & 1) ^ 1, abort)) break;
                    mbar_arrive_expect_tx(&mfull[nb], map_bytes);
                    bulk_g2s(smem_u32(map_sm + nb * map_words), a.map + nxt * kTileM * a.K, map_bytes, &mfull[nb]);
                }
                const Steps st = make_steps(a, mask_cur);
                StepWalker w{st.kbits, 0, 0, -1};
                bool ok = true;
                for (int s = 0; s < st.n_steps; ++s, ++it) {
                    int ks[4], c;
                    w.next(a, ks, c);
                    const int stage = it % S;
                    if (!mbar_wait(&empty[stage], ((it / S) & 1) ^ 1, abort)) {
                        ok = false;
                        break;
                    }
                    int nb = 0;
#pragma unroll
                    for (int p = 0; p < 4; ++p) nb += (p < a.pack && ks[p] >= 0) ? 1 : 0;
                    mbar_arrive_expect_tx(&full[stage], nb * kBTile);
                    const uint32_t Bs = smem_u32(smem + stage * kStage) + kABytes;
                    int q = 0;
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        if (p >= a.pack || ks[p] < 0) continue;
                        bulk_g2s(Bs + q * kBTile, a.wpack + ((int64_t)ks[p] * a.nchunks + c) * kBTile, kBTile,
                                 &full[stage]);
                        ++q;
                    }
                }
                if (!ok) break;
                mask_cur = mask_next;
            }
        }
        __syncwarp();
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

int sm_count() {
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

template <int BN, int EB>
int launch_fwd(FwdArgs a, cudaStream_t s) {
    const int stage = kABytes + a.pack * BN * kRowBytes;
    const int map_bytes = a.K <= kMaxMapStage ? 2 * kTileM * a.K * 4 : 0;
    a.direct_store = (a.direct_store && BN <= 128) ? 1 : 0;  // staging tile only where it fits
    const int fixed = 1024 + map_bytes + (a.direct_store ? kTileM * BN * 2 : 0) + (2 * 8 + 9) * 8 + 16;
    int stages = 8;
    while (stages > kLag + 1 && stages * stage + fixed > 227 * 1024) --stages;
    // a gather thread publishes a stage kLag steps late, so the ring needs more than kLag stages
    if (stages < kLag + 1 || stages * stage + fixed > 227 * 1024) return FVGB_EINVAL;
    a.stages = stages;
    const int smem = stages * stage + fixed;
    auto kern = conv_tc_fwd_kernel<BN, EB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return launch_status();
    const int64_t grid = std::min<int64_t>(a.n_tiles, sm_count());
    kern<<<(unsigned)grid, kThreads, smem, s>>>(a);
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
    const int64_t row_bytes = (int64_t)c_in * eb;
    // each MMA consumes 32 bytes of K; rows shorter than 128 bytes must tile a 128-byte row
    if (row_bytes % 32 != 0 || (row_bytes < 128 && 128 % row_bytes != 0) || (ldx * eb) % 16 != 0) return FVGB_EINVAL;
    const int BN = tile_n(c_out);
    if (BN < 0) return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    if (!map || !packed_w || !y || (n_x > 0 && !x)) return FVGB_EINVAL;
    if (((uintptr_t)x & 15) || ((uintptr_t)packed_w & 15) || ((uintptr_t)y & 15) || ((uintptr_t)map & 15))
        return FVGB_EINVAL;
    FwdArgs a;
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
    a.nchunks = (int32_t)ceil_div(row_bytes, 128);
    a.pack = row_bytes < 128 ? (int32_t)(128 / row_bytes) : 1;
    if (a.pack > 4) return FVGB_EINVAL;
    a.row_bytes = (int32_t)row_bytes;
    a.cout = c_out;
    a.y = (uint8_t *)y;
    a.ldy = ldy;
    a.scale = out_scale;
    a.err = err_dev;
    a.stages = 0;
    a.n_tiles = ceil_div(n_out, kTileM);
    a.direct_store = (ldy == c_out && c_out % 8 == 0) ? 1 : 0;
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
