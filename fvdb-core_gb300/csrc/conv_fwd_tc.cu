// Tensor-core (tcgen05 / TMEM) implicit-GEMM sparse convolution, forward and data gradient.
//
//   y[m, :] = scale (.) sum_k x[map[m,k], :] . W[k]       (BF16 or FP8-E4M3 in, FP32 accumulate)
//
// Persistent kernel, one CTA per SM, looping over 128-row output tiles (tile t = blockIdx.x +
// i * gridDim.x).  Each tile owns all (<= 256) output channels, so every output row is written
// exactly once, without atomics.  The reduction dimension is cut into units of 128 bytes: one
// 128-byte channel chunk of one kernel offset, or, when a feature row is 64 or 32 bytes, a fixed
// group of 2 or 4 consecutive offsets whose rows share one 128-byte A row (one weight image per
// group, so no half-empty weight tiles).  Units absent from all 128 rows of a tile (per-tile
// occupancy mask) are skipped.  A pipeline stage carries U units (2 for N <= 64), so every
// barrier round trip feeds 8 MMAs: the per-stage handshakes, not bytes, set the pace of this
// kernel, and tcgen05.mma with N <= 128 costs the same ~60-80 cycles whatever N is.
//
// Warp roles (448 threads):
//   warps 0-7  gather: each warp fills 16 rows of every unit's A tile.  Lane l copies chunk l%8 of
//              rows l/8, l/8+4, l/8+8, l/8+12, so one warp instruction moves four whole 128-byte
//              A rows (per-SM cp.async throughput is set by the number of issuing warps and the
//              distinct lines per instruction, not by bytes).  Copies are 16-byte cp.async (L2
//              evict_last: the input features stay L2-resident while the map and output stream)
//              into the 128B-swizzled K-major A layout; absent entries (map -1) are zero-stored
//              with st.shared.  Both are generic-proxy writes, so each warp publishes a stage to
//              the tensor core (async proxy) itself, kLag stages late: cp.async.wait_group,
//              fence.proxy.async, __syncwarp, one mbarrier arrive.  The MMA warp never fences
//              and its MMAs stream back to back.  Map entries are read before the stage wait so
//              their latency overlaps it.
//   warp 8     TMEM allocation (2 x N columns) and the MMA issuer: the whole warp runs the
//              issue loop and one elected lane issues each tcgen05.mma; tile i accumulates into
//              TMEM buffer i % 2.
//   warps 9-12 epilogue: tcgen05.ld of the finished buffer -> scale -> BF16 -> a shared-memory
//              copy of the output tile -> one bulk async store of the tile's contiguous rows;
//              overlaps the next tile's main loop.
//   warp 13    loader: bulk async copies of each tile's map rows (double-buffered) and of each
//              unit's pre-packed, pre-swizzled weight image.
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
constexpr int kGatherWarps = 8;   // 256 gather threads: cp.async throughput grows with the issuing warps
constexpr int kRowsPerWarp = kTileM / kGatherWarps;
constexpr int kMmaWarp = kGatherWarps;
constexpr int kEpiWarps = 4;
constexpr int kThreads = (kGatherWarps + 1 + kEpiWarps + 1) * 32;  // + loader warp
constexpr int kMaxMapStage = 32;  // map tiles staged in shared memory up to K = 32
constexpr int kLag = 1;  // cp.async groups a gather thread keeps in flight before publishing a stage

// A "unit" is 128 bytes of the reduction dimension for all 128 rows of a tile: one 128-byte
// channel chunk of one kernel offset (rows of >= 128 bytes), or a fixed group of `pack`
// consecutive offsets whose rows share one 128-byte A row (rows of 64 or 32 bytes).  Each unit
// has one pre-packed [BN x 128 B] weight image; a pipeline stage holds U units.
struct FwdArgs {
    const uint8_t *x;
    int64_t n_x;
    int64_t ldx_bytes;
    int32_t cin;
    const int32_t *map;  // [ceil(n_out/128)*128, K], padding rows -1
    int64_t n_out;
    int32_t K;
    const uint32_t *tile_mask;  // may be null (or K > 32): no skipping
    const uint8_t *wpack;       // [units][BN rows][128 B]
    int32_t nchunks;            // 128-byte chunks per row (pack == 1)
    int32_t pack;               // kernel offsets per 128-byte A row (1, 2 or 4); pack > 1 => nchunks == 1
    int32_t groups;             // offset groups (pack > 1): ceil(K / pack)
    int32_t row_bytes;          // c_in * elem
    int32_t cout;
    uint8_t *y;                 // bf16 [n_out, ldy]
    int64_t ldy;
    const float *scale;         // per output channel, may be null
    const float *bias;          // per output channel, added after the scale, may be null
    int32_t relu;               // 1: max(., 0) after the bias (fused activation)
    int32_t *err;
    int32_t stages;
    int64_t n_tiles;
    int32_t direct_store;  // 1: output rows contiguous (ldy == cout, cout % 8 == 0): one bulk store per tile
    const int32_t *out_rows;  // null: map row m computes output row m; else output row out_rows[m] (-1 = none)
};

// Active units of one tile: a bit set (K <= 32 with a mask) or all units in order.
struct Units {
    uint32_t bits;  // pack > 1: active groups; pack == 1: active offsets
    int n;          // number of units
};

template <int PACK>
__device__ __forceinline__ Units tile_units(const FwdArgs &a, int64_t tile) {
    Units u;
    if (a.K > 32) {
        u.bits = 0;
        u.n = PACK > 1 ? a.groups : a.K * a.nchunks;
        return u;
    }
    const uint32_t all = a.K == 32 ? 0xffffffffu : ((1u << a.K) - 1u);
    const uint32_t mask = a.tile_mask ? (__ldg(a.tile_mask + tile) & all) : all;
    if (PACK > 1) {
        uint32_t gm = 0;
        for (int g = 0; g < a.groups; ++g)
            if ((mask >> (g * PACK)) & ((1u << PACK) - 1u)) gm |= 1u << g;
        u.bits = gm;
        u.n = __popc(gm);
    } else {
        u.bits = mask;
        u.n = __popc(mask) * a.nchunks;
    }
    return u;
}

// Walks a tile's units in order: the weight image index, the first kernel offset and the chunk.
template <int PACK>
struct UnitWalker {
    uint32_t bits;
    int lin;    // unit counter when K > 32
    int chunk;  // pack == 1
    int cur;    // pack == 1: current offset
    __device__ __forceinline__ void next(const FwdArgs &a, int &image, int &k0, int &c) {
        if (PACK > 1) {
            int g;
            if (a.K <= 32) {
                g = __ffs(bits) - 1;
                bits &= bits - 1;
            } else {
                g = lin++;
            }
            image = g;
            k0 = g * PACK;
            c = 0;
            return;
        }
        if (chunk == 0) {
            if (a.K <= 32) {
                cur = __ffs(bits) - 1;
                bits &= bits - 1;
            } else {
                cur = lin++;
            }
        }
        image = cur * a.nchunks + chunk;
        k0 = cur;
        c = chunk;
        chunk = (chunk + 1 == a.nchunks) ? 0 : chunk + 1;
    }
};

__device__ __forceinline__ void st_shared_zero16(uint32_t addr) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(addr), "r"(0) : "memory");
}

template <int BN, int EBYTES, int PACK, int U>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_fwd_kernel(FwdArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kBTile = BN * kRowBytes;
    constexpr int kStage = U * (kABytes + kBTile);          // [U A tiles][U B tiles]
    constexpr int kSlotBytes = kRowBytes / PACK;             // one offset's share of an A row
    constexpr int kCpr = PACK > 1 ? kSlotBytes / 16 : 8;     // 16-byte chunks per offset slot
    constexpr int kCopies = kRowsPerWarp / 4;                // rows per lane per unit
    const int S = a.stages;
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
            mbar_init(&full[s], kGatherWarps + 1);  // one lane per gather warp + the loader's expect_tx
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpiWarps);  // one lane per epilogue warp
            mbar_init(&mfull[b], 1);
            mbar_init(&mempty[b], kGatherWarps);
        }
        mbar_init(fin, 1);
        *abort = 0;
    }
    if (warp == kMmaWarp) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < kGatherWarps) {
        // ----------------------------------------------------------------- gather (A operand)
        // Lane -> (16-byte chunk j of the 128-byte A row, rows rsub, rsub+4, rsub+8, rsub+12 of
        // this warp's 16): one warp instruction moves four whole A rows.
        const uint64_t keep = policy_evict_last();
        const int j = lane & 7;
        const int rsub = lane >> 3;
        const int row0 = warp * kRowsPerWarp;
        const int slot = j / kCpr;         // offset slot of chunk j within a group
        const int jj = j - slot * kCpr;    // chunk within that offset's row
        uint32_t it = 0, sig = 0, stage = 0, phase = 0, pstage = 0;
        int64_t tile = blockIdx.x;
        for (int i = 0; tile < a.n_tiles && !*abort; tile += stride, ++i) {
            const int mb = i & 1;
            if (stage_map && !__all_sync(0xffffffffu, mbar_wait_backoff(&mfull[mb], (i >> 1) & 1, abort, 64))) break;
            const int32_t *mtile = map_sm + mb * map_words;
            const Units un = tile_units<PACK>(a, tile);
            UnitWalker<PACK> w{un.bits, 0, 0, -1};
            bool ok = true;
            for (int u0 = 0; u0 < un.n; u0 += U) {
                // map entries first: their latency overlaps the wait for the stage
                int32_t src[U][kCopies];
                bool on[U];
                int64_t colb[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    int image = -1, k0 = 0, c = 0;
                    if (u0 + u < un.n) w.next(a, image, k0, c);
                    const int k = k0 + (PACK > 1 ? slot : 0);
                    const int bytes = PACK > 1 ? kSlotBytes : min(kRowBytes, a.row_bytes - c * kRowBytes);
                    // chunks past a short last chunk are never read by the MMA; group members past
                    // K are zero-stored (their weights are zero, but stale A bytes could be NaN)
                    on[u] = image >= 0 && (PACK > 1 || j * 16 < bytes);
                    colb[u] = PACK > 1 ? (int64_t)jj * 16 : (int64_t)c * kRowBytes + j * 16;
#pragma unroll
                    for (int q = 0; q < kCopies; ++q) {
                        const int r = row0 + rsub + 4 * q;
                        int32_t v = -1;
                        if (on[u] && k < a.K) {
                            if (stage_map) {
                                v = mtile[r * a.K + k];
                            } else {
                                const int64_t row = tile * kTileM + r;
                                v = row < a.n_out ? a.map[row * a.K + k] : -1;
                            }
                        }
                        src[u][q] = v;
                    }
                }
                bool go = true;
                if (lane == 0) go = mbar_wait(&empty[stage], phase ^ 1, abort);
                go = __shfl_sync(0xffffffffu, go, 0);
                __syncwarp();
                if (!go) {
                    ok = false;
                    break;
                }
                const uint32_t As = smem_u32(smem + stage * kStage);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (!on[u]) continue;
#pragma unroll
                    for (int q = 0; q < kCopies; ++q) {
                        const uint32_t dst = As + u * kABytes + sw128_offset(row0 + rsub + 4 * q, j);
                        if (src[u][q] >= 0 && src[u][q] < a.n_x)
                            cp_async_16_hint(dst, a.x + (int64_t)src[u][q] * a.ldx_bytes + colb[u], 16u, keep);
                        else
                            st_shared_zero16(dst);
                    }
                }
                cp_async_commit();
                ++it;
                if (++stage == (uint32_t)S) {
                    stage = 0;
                    phase ^= 1;
                }
                if (it - sig > kLag) {
                    // the copies of stage `sig` have landed: publish them to the async proxy (tcgen05.mma)
                    cp_async_wait_group<kLag>();
                    fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&full[pstage]);
                    ++sig;
                    if (++pstage == (uint32_t)S) pstage = 0;
                }
            }
            __syncwarp();
            if (stage_map && lane == 0) mbar_arrive(&mempty[mb]);
            if (!ok) break;
        }
        cp_async_wait_group<0>();
        fence_proxy_async();
        __syncwarp();
        if (lane == 0)
            for (; sig < it; ++sig) {
                mbar_arrive(&full[pstage]);
                if (++pstage == (uint32_t)S) pstage = 0;
            }
    } else if (warp == kMmaWarp) {
        // ----------------------------------------------------------------- MMA issuer
        // The whole warp runs this loop (warp-uniform control flow, operands in uniform
        // registers); one elected lane issues each tcgen05 instruction.  Descriptors are
        // advanced by constant offsets (16-byte units) from one base: shared addresses stay
        // below 2^18, so the 14-bit start-address field never carries.
        {
            constexpr uint32_t idesc = EBYTES == 2 ? idesc_m128(BN, 1, 1) : idesc_m128(BN, 0, 0);
            constexpr uint32_t kStageD = kStage >> 4, kAD = kABytes >> 4, kBOffD = (U * kABytes) >> 4,
                               kBTileD = kBTile >> 4;
            const uint64_t adesc0 = desc_sw128(smem_u32(smem));
            const int last_k32 = (a.row_bytes - (a.nchunks - 1) * kRowBytes) >> 5;  // pack == 1: last chunk
            uint32_t stage = 0, phase = 0;
            bool ok = true;
            int64_t tile = blockIdx.x;
            for (int i = 0; tile < a.n_tiles && ok; tile += stride, ++i) {
                const int b = i & 1;
                if (!mbar_wait_warp(&tempty[b], ((i >> 1) & 1) ^ 1, abort)) break;
                tc_fence_after();
                const uint32_t d = tmem + b * BN;
                const int n_units = tile_units<PACK>(a, tile).n;
                uint32_t acc = 0;
                int c = 0;
                for (int u0 = 0; u0 < n_units; u0 += U) {
                    if (!mbar_wait_warp(&full[stage], phase, abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t ad = adesc0 + stage * kStageD, bd = ad + kBOffD;
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (u0 + u >= n_units) break;
                        int nk = 4;
                        if (PACK == 1) {
                            nk = c == a.nchunks - 1 ? last_k32 : 4;
                            c = c + 1 == a.nchunks ? 0 : c + 1;
                        }
#pragma unroll
                        for (int h = 0; h < 4; ++h) {  // 32 bytes of K per MMA
                            if (h >= nk) break;
                            if (EBYTES == 2)
                                mma_f16_warp(d, ad + u * kAD + 2 * h, bd + u * kBTileD + 2 * h, idesc, acc);
                            else
                                mma_f8_warp(d, ad + u * kAD + 2 * h, bd + u * kBTileD + 2 * h, idesc, acc);
                            acc = 1;
                        }
                    }
                    mma_commit_warp(&empty[stage]);
                    if (++stage == (uint32_t)S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (!ok) break;
                if (acc)
                    mma_commit_warp(&tfull[b]);
                else
                    mbar_arrive_warp(&tfull[b]);
            }
            // all issued MMAs complete before TMEM is released
            mma_commit_warp(fin);
            const long long t0 = clock64();
            while (!mbar_try_wait_sleep(fin, 0, kSuspendNs) && clock64() - t0 < kWaitCycles) {
            }
        }
        __syncwarp();
    } else if (warp < kMmaWarp + 1 + kEpiWarps) {
        // ----------------------------------------------------------------- epilogue
        const int et = threadIdx.x - (kMmaWarp + 1) * 32;  // 0..127
        const int q4 = warp & 3;                           // TMEM lane quarter this warp may access
        const int rt = q4 * 32 + lane;                     // row of the tile this thread drains
        int64_t tile = blockIdx.x;
        for (int i = 0; tile < a.n_tiles; tile += stride, ++i) {
            const int b = i & 1;
            const bool ready =
                __all_sync(0xffffffffu, mbar_wait_backoff(&tfull[b], (i >> 1) & 1, abort, 128) && !*abort);
            if (!ready) break;
            tc_fence_after();
            const int n_units = tile_units<PACK>(a, tile).n;
            const int64_t m0 = tile * kTileM;
            const int64_t left = a.n_out - m0;
            const int rows = left < kTileM ? (int)left : kTileM;
            const uint32_t tbase = tmem + b * BN + ((uint32_t)(q4 * 32) << 16);
            // the output row this thread drains (rows of a given order: one bulk store per row)
            const int64_t yrow_i = rt >= rows ? -1 : (a.out_rows ? (int64_t)__ldg(a.out_rows + m0 + rt) : m0 + rt);
            if (a.direct_store) {
                // the staging tile of the previous store has been read
                if (a.out_rows || et == 0) bulk_wait_read<0>();
                named_barrier(1, kTileM);
            }
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 16) {
                float v[16];
                if (n_units > 0) {
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
                    if (a.bias) {
                        lo += cc < a.cout ? a.bias[cc] : 0.f;
                        hi += cc + 1 < a.cout ? a.bias[cc + 1] : 0.f;
                    }
                    if (a.relu) {  // NaN passes through, as torch.relu
                        lo = lo < 0.f ? 0.f : lo;
                        hi = hi < 0.f ? 0.f : hi;
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
                    __nv_bfloat16 *yrow = reinterpret_cast<__nv_bfloat16 *>(a.y) + yrow_i * a.ldy;
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        const __nv_bfloat162 h2 = *reinterpret_cast<const __nv_bfloat162 *>(&packed[t]);
                        if (c0 + 2 * t < a.cout) yrow[c0 + 2 * t] = h2.x;
                        if (c0 + 2 * t + 1 < a.cout) yrow[c0 + 2 * t + 1] = h2.y;
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
            if (a.direct_store) {
                fence_proxy_async();  // staging writes -> visible to the bulk store (async proxy)
                named_barrier(1, kTileM);
                if (a.out_rows) {
                    if (yrow_i >= 0) {
                        bulk_s2g(a.y + yrow_i * a.ldy * 2, smem_u32(ystage + (size_t)rt * a.cout * 2),
                                 (uint32_t)(a.cout * 2));
                        bulk_commit();
                    }
                } else if (et == 0) {
                    bulk_s2g(a.y + m0 * a.ldy * 2, smem_u32(ystage), (uint32_t)(rows * a.cout * 2));
                    bulk_commit();
                }
            }
        }
        if (a.direct_store && (a.out_rows || et == 0)) bulk_wait<0>();
    } else {
        // ----------------------------------------------------------------- loader (bulk copies)
        if (lane == 0) {
            uint32_t stage = 0, phase = 0;
            int64_t tile = blockIdx.x;
            const uint32_t map_bytes = (uint32_t)map_words * 4;
            if (stage_map && tile < a.n_tiles) {
                mbar_arrive_expect_tx(&mfull[0], map_bytes);
                bulk_g2s(smem_u32(map_sm), a.map + tile * kTileM * a.K, map_bytes, &mfull[0]);
            }
            for (int i = 0; tile < a.n_tiles && !*abort; tile += stride, ++i) {
                const int64_t nxt = tile + stride;
                if (stage_map && nxt < a.n_tiles) {
                    const int nb = (i + 1) & 1;
                    if (!mbar_wait_backoff(&mempty[nb], (((i + 1) >> 1) & 1) ^ 1, abort, 32)) break;
                    mbar_arrive_expect_tx(&mfull[nb], map_bytes);
                    bulk_g2s(smem_u32(map_sm + nb * map_words), a.map + nxt * kTileM * a.K, map_bytes, &mfull[nb]);
                }
                const Units un = tile_units<PACK>(a, tile);
                UnitWalker<PACK> w{un.bits, 0, 0, -1};
                bool ok = true;
                for (int u0 = 0; u0 < un.n; u0 += U) {
                    if (!mbar_wait(&empty[stage], phase ^ 1, abort)) {
                        ok = false;
                        break;
                    }
                    const int nu = min(U, un.n - u0);
                    mbar_arrive_expect_tx(&full[stage], nu * kBTile);
                    const uint32_t Bs = smem_u32(smem + stage * kStage) + U * kABytes;
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (u >= nu) break;
                        int image, k0, c;
                        w.next(a, image, k0, c);
                        bulk_g2s(Bs + u * kBTile, a.wpack + (int64_t)image * kBTile, kBTile, &full[stage]);
                    }
                    if (++stage == (uint32_t)S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (!ok) break;
            }
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
    if (threadIdx.x == 0 && *abort) atomicExch(a.err, FVGB_ETIMEOUT);
}

// Packed weight image: per unit one [BN rows (output channel n) x 128 bytes] block laid out
// exactly as the 128B-swizzled K-major shared-memory operand.  pack == 1: unit (k, chunk c)
// holds W[k][c*CE + e][n] for e in [0, CE) (CE = 128/ebytes); pack > 1: unit g holds
// W[g*pack + p][e][n] at element p*cin + e of the row.  Zero where the channel, the offset or
// n is out of range.
__global__ void pack_weights_kernel(const uint8_t *__restrict__ w, int64_t K, int32_t cin, int32_t cout,
                                    int64_t wsk, int64_t wsci, int64_t wsco, int32_t ebytes, int32_t BN,
                                    int32_t nchunks, int32_t pack, int64_t units, uint8_t *__restrict__ out) {
    const int ce = 128 / ebytes;
    const int64_t total = units * BN * ce;  // elements of the image
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tilei = e / ((int64_t)BN * ce);
        const int64_t rem = e % ((int64_t)BN * ce);
        const int n = (int)(rem / ce), kk = (int)(rem % ce);
        int64_t k;
        int ci;
        if (pack > 1) {
            const int p = kk / cin;
            k = tilei * pack + p;
            ci = kk - p * cin;
        } else {
            k = tilei / nchunks;
            ci = (int)(tilei % nchunks) * ce + kk;
        }
        const uint32_t byte = (uint32_t)kk * ebytes;
        const uint32_t off = sw128_offset((uint32_t)n, byte >> 4) + (byte & 15);
        uint8_t *dst = out + tilei * (int64_t)BN * 128 + off;
        const bool ok = k < K && ci < cin && n < cout;
        const int64_t src = ok ? (k * wsk + (int64_t)ci * wsci + (int64_t)n * wsco) * ebytes : 0;
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

// Units of the packed weight image for (K, c_in*elem bytes).
int64_t weight_units(int64_t K, int64_t row_bytes, int *pack, int *nchunks) {
    *pack = row_bytes < 128 ? (int)(128 / row_bytes) : 1;
    *nchunks = (int)ceil_div(row_bytes, 128);
    return *pack > 1 ? ceil_div(K, (int64_t)*pack) : K * *nchunks;
}

int sm_count() { return device_sm_count(); }

template <int BN, int EB, int PACK>
int launch_fwd(FwdArgs a, cudaStream_t s) {
    // two units per stage where both fit next to a deep enough ring; one for wide outputs
    constexpr int U = BN <= 64 ? 2 : 1;
    constexpr int stage = U * (kABytes + BN * kRowBytes);
    const int map_bytes = a.K <= kMaxMapStage ? 2 * kTileM * a.K * 4 : 0;
    a.direct_store = (a.direct_store && BN <= 128) ? 1 : 0;  // staging tile only where it fits
    const int fixed = 1024 + map_bytes + (a.direct_store ? kTileM * BN * 2 : 0) + (2 * 8 + 9) * 8 + 16;
    int stages = 8;
    while (stages > kLag + 1 && stages * stage + fixed > 227 * 1024) --stages;
    // a gather thread publishes a stage kLag stages late, so the ring needs more than kLag stages
    if (stages < kLag + 1 || stages * stage + fixed > 227 * 1024) return FVGB_EINVAL;
    a.stages = stages;
    const int smem = stages * stage + fixed;
    auto kern = conv_tc_fwd_kernel<BN, EB, PACK, U>;
    if (set_dynamic_smem(kern, smem) != cudaSuccess)
        return launch_status();
    const int64_t grid = std::min<int64_t>(a.n_tiles, sm_count());
    kern<<<(unsigned)grid, kThreads, smem, s>>>(a);
    count_launches(1);
    return launch_status();
}

template <int EB, int PACK>
int dispatch_bn(int BN, FwdArgs a, cudaStream_t s) {
    switch (BN) {
        case 32: return launch_fwd<32, EB, PACK>(a, s);
        case 64: return launch_fwd<64, EB, PACK>(a, s);
        case 128: return launch_fwd<128, EB, PACK>(a, s);
        default: return launch_fwd<256, EB, PACK>(a, s);
    }
}

template <int EB>
int dispatch_pack(int BN, int pack, FwdArgs a, cudaStream_t s) {
    switch (pack) {
        case 1: return dispatch_bn<EB, 1>(BN, a, s);
        case 2: return dispatch_bn<EB, 2>(BN, a, s);
        default: return dispatch_bn<EB, 4>(BN, a, s);
    }
}

int dispatch_fwd(int eb, int BN, int pack, FwdArgs a, cudaStream_t s) {
    return eb == 2 ? dispatch_pack<2>(BN, pack, a, s) : dispatch_pack<1>(BN, pack, a, s);
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
    int pack = 1, nchunks = 1;
    *bytes = (size_t)(weight_units(K, (int64_t)cin * eb, &pack, &nchunks) * BN * 128);
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
    int pack = 1, nchunks = 1;
    const int64_t units = weight_units(K, (int64_t)cin * eb, &pack, &nchunks);
    const int64_t total = (int64_t)need / eb;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(total, 256), 4096);
    pack_weights_kernel<<<blocks, 256, 0, as_stream(stream)>>>((const uint8_t *)w, K, cin, cout, wsk, wsci, wsco, eb, BN,
                                                               nchunks, pack, units, (uint8_t *)packed);
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_conv_fwd_tc(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                const int32_t *map, int64_t n_out, int32_t K, const uint32_t *tile_mask,
                                const void *packed_w, int32_t c_out, void *y, int64_t ldy, const float *out_scale,
                                int32_t *err_dev, fvgb_stream_t stream) {
    return fvgb_conv_fwd_tc_bias(dtype, x, n_x, c_in, ldx, map, n_out, K, tile_mask, packed_w, c_out, y, ldy,
                                 out_scale, nullptr, err_dev, stream);
}

extern "C" int fvgb_conv_fwd_tc_bias(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                     const int32_t *map, int64_t n_out, int32_t K, const uint32_t *tile_mask,
                                     const void *packed_w, int32_t c_out, void *y, int64_t ldy,
                                     const float *out_scale, const float *bias, int32_t *err_dev,
                                     fvgb_stream_t stream) {
    return fvgb_conv_fwd_tc_epilogue(dtype, x, n_x, c_in, ldx, map, n_out, K, tile_mask, packed_w, c_out, y, ldy,
                                     out_scale, bias, 0, err_dev, stream);
}

extern "C" int fvgb_conv_fwd_tc_epilogue(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                         const int32_t *map, int64_t n_out, int32_t K, const uint32_t *tile_mask,
                                         const void *packed_w, int32_t c_out, void *y, int64_t ldy,
                                         const float *out_scale, const float *bias, int32_t relu, int32_t *err_dev,
                                         fvgb_stream_t stream) {
    return fvgb_conv_fwd_tc_rows(dtype, x, n_x, c_in, ldx, map, n_out, K, nullptr, tile_mask, packed_w, c_out, y, ldy,
                                 out_scale, bias, relu, err_dev, stream);
}

extern "C" int fvgb_conv_fwd_tc_rows(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                     const int32_t *map, int64_t n_out, int32_t K, const int32_t *rows,
                                     const uint32_t *tile_mask, const void *packed_w, int32_t c_out, void *y,
                                     int64_t ldy, const float *out_scale, const float *bias, int32_t relu,
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
    a.out_rows = rows;
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
    int pack = 1, nchunks = 1;
    weight_units(K, row_bytes, &pack, &nchunks);
    if (pack > 4) return FVGB_EINVAL;
    a.nchunks = nchunks;
    a.pack = pack;
    a.groups = (int32_t)ceil_div((int64_t)K, (int64_t)pack);
    // the group bit set of a K <= 32 mask has at most 16 bits; K > 32 walks units linearly
    a.row_bytes = (int32_t)row_bytes;
    a.cout = c_out;
    a.y = (uint8_t *)y;
    a.ldy = ldy;
    a.scale = out_scale;
    a.bias = bias;
    a.relu = relu ? 1 : 0;
    a.err = err_dev;
    a.stages = 0;
    a.n_tiles = ceil_div(n_out, kTileM);
    a.direct_store = (ldy == c_out && c_out % 8 == 0) ? 1 : 0;
    cudaStream_t s = as_stream(stream);
    return dispatch_fwd(eb, BN, a.pack, a, s);
}
