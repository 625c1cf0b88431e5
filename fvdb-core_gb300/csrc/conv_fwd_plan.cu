// Tensor-core implicit-GEMM sparse convolution over a tile plan: forward and data gradient.
//
//   y[m, :] = scale (.) sum_k x[map[m,k], :] . W[k] + bias      (BF16 or FP8-E4M3 in, FP32 accumulate)
//
// The 128 output rows of a tile read only a few hundred distinct input rows (NanoVDB order keeps
// a tile spatially compact: on surface grids about 2.3 distinct source rows per output row for a
// 3x3x3 kernel, against about 13 map entries per row).  A tile plan, built once per kernel map,
// lists each tile's distinct source rows and gives every map entry a 16-bit index into that list.
// The convolution kernel then
//   * stages the distinct rows of a tile in shared memory once (cp.async, double-buffered, so
//     the next tile's rows load while this tile computes) instead of gathering every map entry
//     from L2, and
//   * builds the A operand (the gathered rows of one 128-byte unit of the reduction) in tensor
//     memory with tcgen05.st from the staged rows, so the tensor core reads A from TMEM
//     (tcgen05.mma with [a-tmem]) and no generic-to-async proxy fence is needed per stage.
// A tile whose distinct rows exceed the staging buffer is split into phases (consecutive offset
// groups whose rows fit); the phases of a tile accumulate into the same TMEM accumulator.
//
// Warp roles (576 threads):
//   warps 0-7   builders: warp w fills lane quarter w % 4 (rows 32*(w%4) .. +31) and 64-byte half
//               w / 4 of every unit's 128-byte A row; a thread reads its row's local index from
//               the tile's plan, 64 bytes of the staged row (or zeros), and tcgen05.st's them.
//               U units per pipeline stage share one handshake (tcgen05.wait::st, one mbarrier
//               arrive per warp); the ring holds 3 stages of 4 units (N <= 64) or 2 of 2, deep
//               enough to hide the L2-to-shared latency of the weight images behind the MMAs.
//   warp 8      TMEM allocation and the MMA issuer: warp-uniform loop, one elected lane issues
//               tcgen05.mma (A from TMEM, B = the unit's pre-packed weight image in shared
//               memory); tile i accumulates into TMEM buffer i % 2.
//   warps 9-12  epilogue: tcgen05.ld -> scale -> bias -> BF16 -> shared staging -> one bulk store.
//   warp 13     loader: the weight images.  When all of them fit in shared memory (up to 112 KB:
//               e.g. 3x3x3, 32->64) they are copied once and stay resident; otherwise each unit's
//               image is bulk-copied into its stage's B slot of the ring.
//   warps 14-17 stagers: bulk copy of each tile's local map and header, cp.async of each phase's
//               distinct rows into a staging buffer (a thread loads a batch of row indices
//               before issuing their copies); they run a phase ahead of the builders.
// Every mbarrier wait is bounded (about a second); on expiry the CTA stops, waits for its
// issued MMAs, frees TMEM and raises *err = FVGB_ETIMEOUT.
//
// Reference kernels replaced: conv_forward_cuda_setting{1,2,3}_mode{0,1}_{bf16,f16,tf32,f32}
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMM.cu:120-3826,
// SparseConvolutionImplicitGEMMSorted.cu:115-4639).
#include <cuda_bf16.h>

#include <mutex>

#include "tc_common.cuh"

namespace fvgb {
namespace {

using namespace tc;

constexpr int kTile = 128;
constexpr int kUnitBytes = 128;       // one 128-byte slice of the reduction for all rows of a tile
constexpr int kHdrWords = 68;         // per tile: [0] group mask, [1] phases, [4+2p] group end, [5+2p] rows
constexpr int kMaxGroups = 32;
constexpr int kStageBuf = 40 * 1024;  // bytes of one staging buffer
constexpr int kResidentBytes = 112 * 1024;  // weight images up to this size stay in shared memory
constexpr int kBuilderWarps = 8;
constexpr int kMmaWarpP = 8;
constexpr int kEpiWarpsP = 4;
constexpr int kLoaderWarp = 13;
constexpr int kStagerWarps = 4;
constexpr int kStagerThreads = kStagerWarps * 32;
constexpr int kStageBatch = 16;  // row indices a stager thread loads before issuing their copies
constexpr int kThreadsP = (kLoaderWarp + 1 + kStagerWarps) * 32;

__host__ __device__ inline int row_stride_of(int row_bytes) { return row_bytes + 16; }
__host__ __device__ inline int pack_of(int row_bytes) { return row_bytes < kUnitBytes ? kUnitBytes / row_bytes : 1; }
// Distinct rows one staging buffer holds (a multiple of 32; at least the 128*pack rows of one group).
__host__ __device__ inline int cap_of(int row_bytes) { return (kStageBuf / row_stride_of(row_bytes)) & ~31; }

struct PlanLayout {
    int64_t n_tiles, lmap_off, hdr_off, src_off, bytes;
};
PlanLayout plan_layout(int64_t n_rows, int K) {
    PlanLayout L;
    L.n_tiles = ceil_div(n_rows, kTile);
    L.lmap_off = 0;                                          // uint16 [n_tiles][128][K]
    L.hdr_off = L.lmap_off + L.n_tiles * kTile * K * 2;       // int32 [n_tiles][68]
    L.src_off = L.hdr_off + L.n_tiles * kHdrWords * 4;        // int32 [n_tiles][128*K] (worst case)
    L.bytes = L.src_off + L.n_tiles * kTile * K * 4;
    return L;
}

__device__ __forceinline__ uint32_t plan_hash(int32_t v) { return ((uint32_t)v * 0x9E3779B1u) >> 20; }

// One CTA per tile, one thread per output row (its K map entries are one contiguous, coalesced
// read).  Fast path: every distinct source row of the tile goes into one phase; when they do not
// fit the staging buffer (`cap` rows), the tile is redone group by group: groups of `pack`
// consecutive offsets are taken in order and a group's distinct rows join the current phase
// unless that would exceed `cap`, in which case a new phase starts at the group.  Writes the
// tile's local map (index into its phase's row list, 0xFFFF = absent), its header and its row
// lists (phase after phase).  The local map and the fast path's row list are assembled in
// shared memory and written out with whole 16-byte stores (scattered 2- and 4-byte stores to
// global memory would cost a read-modify-write of each sector).
constexpr int kPlanSlots = 2048;  // shared hash slots; at most cap + 512 <= 1344 keys are live
constexpr int kPlanList = 1024;   // row-list entries kept in shared memory (fast path: <= cap)

__global__ void __launch_bounds__(kTile) tile_plan_kernel(const int32_t *__restrict__ map, int64_t n_rows, int32_t K,
                                                          int32_t pack, int32_t cap, uint16_t *__restrict__ lmap,
                                                          int32_t *__restrict__ hdr, int32_t *__restrict__ src) {
    __shared__ int32_t keys[kPlanSlots];
    __shared__ int16_t locs[kPlanSlots];
    __shared__ __align__(16) uint16_t lm_s[kTile * kMaxGroups];
    __shared__ __align__(16) int32_t list_s[kPlanList];
    __shared__ int32_t s_cnt;
    __shared__ uint32_t s_gmask;
    __shared__ int32_t s_over;
    const int64_t t = blockIdx.x;
    const int r = threadIdx.x, lane = r & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const int64_t row = t * kTile + r;
    const int G = (K + pack - 1) / pack;
    int32_t e[kMaxGroups];
#pragma unroll
    for (int k = 0; k < kMaxGroups; ++k) e[k] = (k < K && row < n_rows) ? __ldg(map + row * K + k) : -1;
    uint32_t gm = 0;
#pragma unroll
    for (int k = 0; k < kMaxGroups; ++k)
        if (e[k] >= 0) gm |= 1u << (k / pack);
    for (int i = r; i < kPlanSlots; i += kTile) keys[i] = -1;
    if (r == 0) {
        s_cnt = 0;
        s_gmask = 0;
        s_over = 0;
    }
    __syncthreads();
    if (gm) atomicOr(&s_gmask, gm);
    int32_t *tsrc = src + t * (int64_t)kTile * K;
    int base = 0;
    // inserts this thread's entries k in [kb, ke); new keys are numbered (one shared atomic per
    // warp and offset) and listed at base + index (fast: in list_s; slow: in global memory).  The
    // fast path stops creating keys once the count passes `cap` (the tile then takes the slow path).
    auto insert = [&](int kb, int ke, bool fast) {
#pragma unroll
        for (int k = 0; k < kMaxGroups; ++k) {
            if (k < kb || k >= ke) continue;  // uniform across the CTA
            int created = -1;
            if (e[k] >= 0 && !(fast && *reinterpret_cast<volatile int32_t *>(&s_over))) {
                uint32_t h = plan_hash(e[k]) & (kPlanSlots - 1);
                for (int probe = 0; probe < kPlanSlots; ++probe) {
                    const int32_t prev = atomicCAS(&keys[h], -1, e[k]);
                    if (prev == -1) {
                        created = (int)h;
                        break;
                    }
                    if (prev == e[k]) break;
                    h = (h + 1) & (kPlanSlots - 1);
                }
            }
            const uint32_t ball = __ballot_sync(0xffffffffu, created >= 0);
            int first = 0;
            if (lane == 0 && ball) {
                first = atomicAdd(&s_cnt, __popc(ball));
                if (fast && first + __popc(ball) > cap) s_over = 1;
            }
            first = __shfl_sync(0xffffffffu, first, 0);
            if (created >= 0) {
                const int loc = first + __popc(ball & lt);
                locs[created] = (int16_t)loc;
                if (!fast) tsrc[base + loc] = e[k];
                else if (loc < kPlanList) list_s[loc] = e[k];
            }
        }
    };
    // local index of every entry k in [kb, ke), written over e[k] (0xFFFF = absent)
    auto lookup = [&](int kb, int ke) {
#pragma unroll
        for (int k = 0; k < kMaxGroups; ++k) {
            if (k < kb || k >= ke) continue;
            int32_t loc = 0xFFFF;
            if (e[k] >= 0) {
                uint32_t h = plan_hash(e[k]) & (kPlanSlots - 1);
                for (int probe = 0; probe < kPlanSlots && keys[h] != e[k]; ++probe) h = (h + 1) & (kPlanSlots - 1);
                loc = (uint16_t)locs[h];
            }
            e[k] = loc;
        }
    };
    auto clear = [&]() {
        __syncthreads();
        for (int i = r; i < kPlanSlots; i += kTile) keys[i] = -1;
        if (r == 0) s_cnt = 0;
        __syncthreads();
    };
    int32_t *th = hdr + t * kHdrWords;
    insert(0, K, true);
    __syncthreads();
    const int total = s_cnt;
    int nph = 1;
    if (total <= cap && !s_over) {
        lookup(0, K);
        if (r == 0) {
            th[4] = G;
            th[5] = total;
        }
        // the row list, 16 bytes per store (the tile's region is 512*K bytes, 16-aligned)
        const int n16 = (total + 3) / 4;
        for (int i = r; i < n16; i += kTile) reinterpret_cast<int4 *>(tsrc)[i] = reinterpret_cast<const int4 *>(list_s)[i];
    } else {
        clear();
        int before = 0;
        nph = 0;
        for (int g = 0; g < G; ++g) {
            const int kb = g * pack, ke = min(K, kb + pack);
            insert(kb, ke, false);
            __syncthreads();
            int cnt = s_cnt;
            if (cnt > cap) {
                if (r == 0) {
                    th[4 + 2 * nph] = g;
                    th[5 + 2 * nph] = before;
                }
                ++nph;
                base += before;
                clear();
                insert(kb, ke, false);
                __syncthreads();
                cnt = s_cnt;
            }
            before = cnt;
            lookup(kb, ke);
            __syncthreads();
        }
        if (r == 0) {
            th[4 + 2 * nph] = G;
            th[5 + 2 * nph] = before;
        }
        ++nph;
    }
    // the local map: assembled in shared memory, written with 16-byte stores (256*K bytes per tile)
#pragma unroll
    for (int k = 0; k < kMaxGroups; ++k)
        if (k < K) lm_s[r * K + k] = (uint16_t)e[k];
    __syncthreads();
    int4 *tl = reinterpret_cast<int4 *>(lmap + t * (int64_t)kTile * K);
    for (int i = r; i < kTile * K * 2 / 16; i += kTile) tl[i] = reinterpret_cast<const int4 *>(lm_s)[i];
    if (r == 0) {
        th[0] = (int32_t)s_gmask;
        th[1] = nph;
        th[2] = 0;
        th[3] = 0;
    }
}

struct PlanArgs {
    const uint8_t *x;
    int64_t n_x;
    int64_t ldx_bytes;
    const uint16_t *lmap;
    const int32_t *hdr;
    const int32_t *src;
    int64_t n_out;
    int32_t K;
    int32_t row_bytes;
    int32_t nchunks;  // 128-byte chunks per row (pack == 1)
    int32_t stride;   // staged row stride in bytes
    const uint8_t *wpack;
    int32_t cout;
    uint8_t *y;
    int64_t ldy;
    const float *scale;
    const float *bias;
    int32_t relu;  // 1: max(., 0) after the bias (fused activation)
    int32_t *err;
    int64_t n_tiles;
    int32_t direct_store;
    int32_t resident;  // 1: all weight images stay in shared memory for the whole kernel
    int32_t n_images;  // weight images (units of the reduction): groups x chunks
};

__device__ __forceinline__ bool warp_wait_lane0(uint64_t *bar, uint32_t parity, volatile int *abort, int lane) {
    bool ok = true;
    if (lane == 0) ok = mbar_wait(bar, parity, abort);
    return __shfl_sync(0xffffffffu, ok, 0);
}

// 64 bytes of a staged row starting at byte `b0` (zeros past row_bytes), as 16 registers.
__device__ __forceinline__ void load64(const uint8_t *row, int b0, int row_bytes, uint32_t (&v)[16], int base_reg) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint4 q = make_uint4(0, 0, 0, 0);
        if (b0 + 16 * c < row_bytes) q = *reinterpret_cast<const uint4 *>(row + b0 + 16 * c);
        v[base_reg + 4 * c + 0] = q.x;
        v[base_reg + 4 * c + 1] = q.y;
        v[base_reg + 4 * c + 2] = q.z;
        v[base_reg + 4 * c + 3] = q.w;
    }
}

// 64 bytes (half hh of the 128-byte unit) of this thread's A row for unit (group g, chunk c),
// read from the staged rows through the tile's local map row `lm`; zeros for absent entries and
// for offsets past K.
template <int PACK>
__device__ __forceinline__ void gather_unit(const uint8_t *stg, const uint16_t *lm, int g, int c, int hh,
                                            const PlanArgs &a, uint32_t (&v)[16]) {
    if (PACK == 1) {
        const uint16_t loc = lm[g];
        if (loc != 0xFFFF) {
            load64(stg + (int)loc * a.stride, c * kUnitBytes + 64 * hh, a.row_bytes, v, 0);
        } else {
#pragma unroll
            for (int t = 0; t < 16; ++t) v[t] = 0u;
        }
    } else if (PACK == 2) {
        const int k = 2 * g + hh;
        const uint16_t loc = k < a.K ? lm[k] : (uint16_t)0xFFFF;
        if (loc != 0xFFFF) {
            load64(stg + (int)loc * a.stride, 0, 64, v, 0);
        } else {
#pragma unroll
            for (int t = 0; t < 16; ++t) v[t] = 0u;
        }
    } else {
        // PACK == 4: two 32-byte offsets per half
#pragma unroll
        for (int o = 0; o < 2; ++o) {
            const int k = 4 * g + 2 * hh + o;
            const uint16_t loc = k < a.K ? lm[k] : (uint16_t)0xFFFF;
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                uint4 qv = make_uint4(0, 0, 0, 0);
                if (loc != 0xFFFF) qv = *reinterpret_cast<const uint4 *>(stg + (int)loc * a.stride + 16 * cc);
                v[8 * o + 4 * cc + 0] = qv.x;
                v[8 * o + 4 * cc + 1] = qv.y;
                v[8 * o + 4 * cc + 2] = qv.z;
                v[8 * o + 4 * cc + 3] = qv.w;
            }
        }
    }
}

template <int BN, int EBYTES, int PACK>
__global__ void __launch_bounds__(kThreadsP, 1) conv_plan_fwd_kernel(PlanArgs a) {
    constexpr int U = BN <= 64 ? 4 : 2;  // units per pipeline stage
    constexpr int S = BN <= 64 ? 3 : 2;  // stages in the ring
    constexpr int NSLOT = U * S;         // A slots in TMEM and B slots in shared memory
    constexpr int kBTile = BN * kUnitBytes;
    constexpr int kAcol = 2 * BN;        // A ring follows the two accumulators in TMEM
    static_assert(kAcol + 32 * NSLOT <= 512, "TMEM budget");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *bring = smem;  // resident: every unit's [BN x 128 B] image; else NSLOT ring slots
    uint8_t *stage_s = bring + (a.resident ? a.n_images : NSLOT) * kBTile;  // 2 x kStageBuf
    // 2 x ([128 x K] local map, then the tile's 68-word header)
    uint8_t *lbuf_s = stage_s + 2 * kStageBuf;
    const int lwords = kTile * a.K;
    const uint32_t lmap_bytes = (uint32_t)lwords * 2, lbuf_bytes = lmap_bytes + kHdrWords * 4;
    uint8_t *ystage = lbuf_s + 2 * lbuf_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(ystage + (a.direct_store ? kTile * BN * 2 : 0));
    uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = tfull + 2, *lfull = tempty + 2,
             *lempty = lfull + 2, *sfull = lempty + 2, *sempty = sfull + 2, *fin = sempty + 2, *wfull = fin + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(wfull + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t stride = gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            // one arrival per builder warp (+ the loader's expect_tx when weights stream through the ring)
            mbar_init(&full[s], kBuilderWarps + (a.resident ? 0 : 1));
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpiWarpsP);
            mbar_init(&lfull[b], 1);
            mbar_init(&lempty[b], kBuilderWarps);
            mbar_init(&sfull[b], kStagerThreads);  // cp.async arrivals of every stager thread
            mbar_init(&sempty[b], kBuilderWarps);
        }
        mbar_init(fin, 1);
        mbar_init(wfull, 1);
        *abort = 0;
    }
    if (warp == kMmaWarpP) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < kBuilderWarps) {
        // ----------------------------------------------------------------- builders (A in TMEM)
        const int q = warp & 3, hh = warp >> 2, r = q * 32 + lane;
        const uint32_t arow = tmem + ((uint32_t)(q * 32) << 16) + kAcol + 16 * hh;
        uint32_t s = 0, ph = 0, pseq = 0;
        bool ok = true;
        int64_t tile = blockIdx.x;
        for (int i = 0; tile < a.n_tiles && ok; tile += stride, ++i) {
            if (!warp_wait_lane0(&lfull[i & 1], (i >> 1) & 1, abort, lane)) break;
            const uint8_t *lb = lbuf_s + (i & 1) * lbuf_bytes;
            const int32_t *th = reinterpret_cast<const int32_t *>(lb + lmap_bytes);
            const uint32_t gmask = (uint32_t)th[0];
            const int nph = th[1];
            const int n_units = __popc(gmask) * a.nchunks;
            const uint16_t *lm = reinterpret_cast<const uint16_t *>(lb) + r * a.K;
            int u = 0;
            // stores unit u's 64 bytes of this thread's A row into its TMEM slot; opens the stage
            // (waits for the slot) at its first unit and publishes it after its last
            auto emit = [&](const uint32_t (&v)[16]) -> bool {
                const int su = u % U;
                if (su == 0) {
                    if (!warp_wait_lane0(&empty[s], ph ^ 1, abort, lane)) return false;
                    tc_fence_after();
                }
                tmem_st16(arow + 32 * (s * U + su), v);
                if (su == U - 1 || u == n_units - 1) {
                    tmem_wait_st();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&full[s]);
                    if (++s == (uint32_t)S) {
                        s = 0;
                        ph ^= 1;
                    }
                }
                ++u;
                return true;
            };
            for (int p = 0; p < nph && ok; ++p, ++pseq) {
                const int gb = p == 0 ? 0 : th[4 + 2 * (p - 1)], ge = th[4 + 2 * p];
                if (!warp_wait_lane0(&sfull[pseq & 1], (pseq >> 1) & 1, abort, lane)) {
                    ok = false;
                    break;
                }
                const uint8_t *stg = stage_s + (pseq & 1) * kStageBuf;
                // software pipeline: the next unit's shared-memory reads are issued before the
                // current unit's tcgen05.st, so their latency overlaps it
                uint32_t v[16];
                bool have = false;
                for (int g = gb; g < ge && ok; ++g) {
                    if (!((gmask >> g) & 1u)) continue;
                    for (int c = 0; c < a.nchunks; ++c) {
                        uint32_t vn[16];
                        gather_unit<PACK>(stg, lm, g, c, hh, a, vn);
                        if (have && !emit(v)) {
                            ok = false;
                            break;
                        }
#pragma unroll
                        for (int t = 0; t < 16; ++t) v[t] = vn[t];
                        have = true;
                    }
                }
                if (ok && have && !emit(v)) ok = false;
                // this phase's staged rows are no longer read (their values are in registers / TMEM)
                __syncwarp();
                if (lane == 0) mbar_arrive(&sempty[pseq & 1]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&lempty[i & 1]);
        }
        tmem_wait_st();  // no store of this thread is in flight when TMEM is released
    } else if (warp == kMmaWarpP) {
        // ----------------------------------------------------------------- MMA issuer (warp-uniform)
        constexpr uint32_t idesc = EBYTES == 2 ? idesc_m128(BN, 1, 1) : idesc_m128(BN, 0, 0);
        constexpr uint32_t kBTileD = kBTile >> 4;
        const uint64_t bdesc0 = desc_sw128(smem_u32(bring));
        const int last_k32 = (a.row_bytes - (a.nchunks - 1) * kUnitBytes) >> 5;
        uint32_t s = 0, ph = 0;
        bool ok = true;
        if (a.resident && !mbar_wait_warp(wfull, 0, abort)) ok = false;
        int64_t tile = blockIdx.x;
        uint32_t gm_next = tile < a.n_tiles ? (uint32_t)__ldg(a.hdr + tile * kHdrWords) : 0u;
        for (int i = 0; tile < a.n_tiles && ok; tile += stride, ++i) {
            const int b = i & 1;
            const uint32_t gm_tile = gm_next;
            const int n_units = __popc(gm_tile) * a.nchunks;
            if (tile + stride < a.n_tiles) gm_next = (uint32_t)__ldg(a.hdr + (tile + stride) * kHdrWords);
            if (!mbar_wait_warp(&tempty[b], ((i >> 1) & 1) ^ 1, abort)) break;
            tc_fence_after();
            const uint32_t d = tmem + b * BN;
            uint32_t acc = 0;
            // resident weights: the image of each unit, in the units' order (groups ascending)
            uint32_t gbits = gm_tile;
            int cur_g = 0, cur_c = a.nchunks;
            for (int u0 = 0; u0 < n_units; u0 += U) {
                if (!mbar_wait_warp(&full[s], ph, abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
#pragma unroll
                for (int su = 0; su < U; ++su) {
                    if (u0 + su >= n_units) break;
                    int nk = 4;
                    if (PACK == 1) nk = ((u0 + su) % a.nchunks == a.nchunks - 1) ? last_k32 : 4;
                    const uint32_t aslot = tmem + kAcol + 32 * (s * U + su);
                    uint64_t bd;
                    if (a.resident) {
                        if (cur_c == a.nchunks) {
                            cur_g = __ffs(gbits) - 1;
                            gbits &= gbits - 1;
                            cur_c = 0;
                        }
                        bd = bdesc0 + (uint64_t)(cur_g * a.nchunks + cur_c) * kBTileD;
                        ++cur_c;
                    } else {
                        bd = bdesc0 + (s * U + su) * kBTileD;
                    }
#pragma unroll
                    for (int h = 0; h < 4; ++h) {  // 32 bytes of K (8 TMEM columns) per MMA
                        if (h >= nk) break;
                        if (EBYTES == 2)
                            mma_f16_ts_warp(d, aslot + 8 * h, bd + 2 * h, idesc, acc);
                        else
                            mma_f8_ts_warp(d, aslot + 8 * h, bd + 2 * h, idesc, acc);
                        acc = 1;
                    }
                }
                mma_commit_warp(&empty[s]);
                if (++s == (uint32_t)S) {
                    s = 0;
                    ph ^= 1;
                }
            }
            if (!ok) break;
            if (acc)
                mma_commit_warp(&tfull[b]);
            else
                mbar_arrive_warp(&tfull[b]);
        }
        mma_commit_warp(fin);
        const long long t0 = clock64();
        while (!mbar_try_wait_sleep(fin, 0, kSuspendNs) && clock64() - t0 < kWaitCycles) {
        }
        __syncwarp();
    } else if (warp < kMmaWarpP + 1 + kEpiWarpsP) {
        // ----------------------------------------------------------------- epilogue
        const int et = threadIdx.x - (kMmaWarpP + 1) * 32;  // 0..127
        const int q4 = warp & 3;                             // TMEM lane quarter of this warp
        const int rt = q4 * 32 + lane;
        int64_t tile = blockIdx.x;
        uint32_t gm_next = tile < a.n_tiles ? (uint32_t)__ldg(a.hdr + tile * kHdrWords) : 0u;
        for (int i = 0; tile < a.n_tiles; tile += stride, ++i) {
            const int b = i & 1;
            const int n_units = __popc(gm_next);
            if (tile + stride < a.n_tiles) gm_next = (uint32_t)__ldg(a.hdr + (tile + stride) * kHdrWords);
            const bool ready =
                __all_sync(0xffffffffu, mbar_wait_backoff(&tfull[b], (i >> 1) & 1, abort, 128) && !*abort);
            if (!ready) break;
            tc_fence_after();
            const int64_t m0 = tile * kTile;
            const int64_t left = a.n_out - m0;
            const int rows = left < kTile ? (int)left : kTile;
            const uint32_t tbase = tmem + b * BN + ((uint32_t)(q4 * 32) << 16);
            if (a.direct_store) {
                if (et == 0) bulk_wait_read<0>();
                named_barrier(1, kTile);
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
                    __nv_bfloat162 h2 = __floats2bfloat162_rn(lo, hi);
                    packed[t] = *reinterpret_cast<uint32_t *>(&h2);
                }
                if (a.direct_store) {
                    uint4 *dst = reinterpret_cast<uint4 *>(ystage + ((size_t)rt * a.cout + c0) * 2);
                    dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    if (c0 + 8 < a.cout) dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                } else {
                    __nv_bfloat16 *yrow = reinterpret_cast<__nv_bfloat16 *>(a.y) + (m0 + rt) * a.ldy;
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
                fence_proxy_async();
                named_barrier(1, kTile);
                if (et == 0) {
                    bulk_s2g(a.y + m0 * a.ldy * 2, smem_u32(ystage), (uint32_t)(rows * a.cout * 2));
                    bulk_commit();
                }
            }
        }
        if (a.direct_store && et == 0) bulk_wait<0>();
    } else if (warp == kLoaderWarp) {
        // ----------------------------------------------------------------- loader (bulk copies)
        if (lane == 0 && a.resident) {
            // every weight image once, for the whole kernel
            mbar_arrive_expect_tx(wfull, (uint32_t)(a.n_images * kBTile));
            for (int im = 0; im < a.n_images; ++im)
                bulk_g2s(smem_u32(bring + im * kBTile), a.wpack + (int64_t)im * kBTile, kBTile, wfull);
        } else if (lane == 0) {
            uint32_t s = 0, ph = 0;
            int64_t tile = blockIdx.x;
            bool ok = true;
            for (int i = 0; tile < a.n_tiles && ok && !*abort; tile += stride, ++i) {
                const int32_t *th = a.hdr + tile * kHdrWords;
                const uint32_t gmask = (uint32_t)__ldg(th);
                const int n_units = __popc(gmask) * a.nchunks;
                int u = 0;
                for (uint32_t gm = gmask; gm && ok; gm &= gm - 1) {
                    const int g = __ffs(gm) - 1;
                    for (int c = 0; c < a.nchunks; ++c, ++u) {
                        const int su = u % U;
                        if (su == 0) {
                            if (!mbar_wait(&empty[s], ph ^ 1, abort)) {
                                ok = false;
                                break;
                            }
                            mbar_arrive_expect_tx(&full[s], (uint32_t)(min(U, n_units - u) * kBTile));
                        }
                        bulk_g2s(smem_u32(bring + (s * U + su) * kBTile), a.wpack + (int64_t)(g * a.nchunks + c) * kBTile,
                                 kBTile, &full[s]);
                        if (su == U - 1 || u == n_units - 1) {
                            if (++s == (uint32_t)S) {
                                s = 0;
                                ph ^= 1;
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();
    } else {
        // ----------------------------------------------------------------- stagers (distinct rows)
        const int st = threadIdx.x - (kLoaderWarp + 1) * 32;  // 0 .. kStagerThreads-1
        const uint64_t keep = policy_evict_last();
        const int cpr = a.row_bytes >> 4;  // 16-byte chunks per row
        uint32_t pseq = 0;
        int64_t tile = blockIdx.x;
        bool ok = true;
        for (int i = 0; tile < a.n_tiles && ok && !*abort; tile += stride, ++i) {
            // the tile's local map and header: loaded by the stagers, which run a phase ahead of
            // the builders, so the copy overlaps the previous tile's work
            if (st == 0) {
                const int buf = i & 1;
                if (mbar_wait_backoff(&lempty[buf], ((i >> 1) & 1) ^ 1, abort, 32)) {
                    mbar_arrive_expect_tx(&lfull[buf], lbuf_bytes);
                    bulk_g2s(smem_u32(lbuf_s + buf * lbuf_bytes), a.lmap + tile * lwords, lmap_bytes, &lfull[buf]);
                    bulk_g2s(smem_u32(lbuf_s + buf * lbuf_bytes + lmap_bytes), a.hdr + tile * kHdrWords,
                             kHdrWords * 4, &lfull[buf]);
                }
            }
            const int32_t *th = a.hdr + tile * kHdrWords;
            const int nph = __ldg(th + 1);
            const int32_t *tsrc = a.src + tile * (int64_t)kTile * a.K;
            int base = 0;
            for (int p = 0; p < nph; ++p, ++pseq) {
                const int cnt = __ldg(th + 5 + 2 * p);
                if (!warp_wait_lane0(&sempty[pseq & 1], ((pseq >> 1) & 1) ^ 1, abort, lane)) {
                    ok = false;
                    break;
                }
                const uint32_t dst0 = smem_u32(stage_s + (pseq & 1) * kStageBuf);
                const int total = cnt * cpr;
                for (int i0 = 0; i0 < total; i0 += kStagerThreads * kStageBatch) {
                    // the row indices first (independent loads in flight together), then the copies
                    int32_t v[kStageBatch];
#pragma unroll
                    for (int j = 0; j < kStageBatch; ++j) {
                        const int idx = i0 + st + j * kStagerThreads;
                        v[j] = idx < total ? __ldg(tsrc + base + idx / cpr) : -2;
                    }
#pragma unroll
                    for (int j = 0; j < kStageBatch; ++j) {
                        if (v[j] == -2) continue;
                        const int idx = i0 + st + j * kStagerThreads;
                        const int row = idx / cpr, ch = idx - row * cpr;
                        const uint32_t dst = dst0 + row * a.stride + ch * 16;
                        if (v[j] >= 0 && v[j] < a.n_x)
                            cp_async_16_hint(dst, a.x + (int64_t)v[j] * a.ldx_bytes + ch * 16, 16u, keep);
                        else
                            cp_async_16(dst, a.x, 0u);  // zero fill, nothing read
                    }
                }
                cp_async_arrive_noinc(&sfull[pseq & 1]);
                base += cnt;
            }
        }
        cp_async_wait_all();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarpP) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (threadIdx.x == 0 && *abort) atomicExch(a.err, FVGB_ETIMEOUT);
}

int plan_tile_n(int32_t cout) {
    if (cout <= 32) return 32;
    if (cout <= 64) return 64;
    if (cout <= 128) return 128;
    return -1;
}

int sm_count_p() { return device_sm_count(); }

template <int BN, int EB, int PACK>
int launch_plan(PlanArgs a, cudaStream_t s) {
    constexpr int U = BN <= 64 ? 4 : 2;
    constexpr int NSLOT = U * (BN <= 64 ? 3 : 2);
    a.direct_store = a.direct_store ? 1 : 0;
    // weight images stay resident in shared memory when they fit next to the staging buffers
    // (the ring would stream them from L2 again for every tile)
    const int fixed = 1024 + 2 * kStageBuf + 2 * (kTile * a.K * 2 + kHdrWords * 4) +
                      (a.direct_store ? kTile * BN * 2 : 0) + (2 * 3 + 6 * 2 + 2) * 8 + 16;
    const int64_t res_bytes = (int64_t)a.n_images * BN * kUnitBytes;
    a.resident = (res_bytes <= kResidentBytes && fixed + res_bytes <= 227 * 1024) ? 1 : 0;
    const int smem = fixed + (a.resident ? (int)res_bytes : NSLOT * BN * kUnitBytes);
    if (smem > 227 * 1024) return FVGB_EINVAL;
    auto kern = conv_plan_fwd_kernel<BN, EB, PACK>;
    if (set_dynamic_smem(kern, smem) != cudaSuccess)
        return launch_status();
    const int64_t grid = std::min<int64_t>(a.n_tiles, sm_count_p());
    kern<<<(unsigned)grid, kThreadsP, smem, s>>>(a);
    count_launches(1);
    return launch_status();
}

template <int EB, int PACK>
int plan_dispatch_bn(int BN, PlanArgs a, cudaStream_t s) {
    switch (BN) {
        case 32: return launch_plan<32, EB, PACK>(a, s);
        case 64: return launch_plan<64, EB, PACK>(a, s);
        default: return launch_plan<128, EB, PACK>(a, s);
    }
}

template <int EB>
int plan_dispatch_pack(int BN, int pack, PlanArgs a, cudaStream_t s) {
    switch (pack) {
        case 1: return plan_dispatch_bn<EB, 1>(BN, a, s);
        case 2: return plan_dispatch_bn<EB, 2>(BN, a, s);
        default: return plan_dispatch_bn<EB, 4>(BN, a, s);
    }
}

// Row sizes the planned kernel takes: multiples of 32 bytes up to 256, and rows shorter than
// 128 bytes must tile a 128-byte unit.
bool plan_row_ok(int64_t row_bytes) {
    return row_bytes >= 32 && row_bytes <= 256 && row_bytes % 32 == 0 && (row_bytes >= 128 || 128 % row_bytes == 0);
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_tc_plan_supported(int32_t dtype, int32_t K, int32_t c_in, int32_t c_out) {
    const int eb = dtype == FVGB_E4M3 ? 1 : (dtype == FVGB_BF16 ? 2 : 0);
    if (!eb) return FVGB_ETYPE;
    if (K < 1 || K > kMaxGroups || c_in < 1 || c_out < 1 || plan_tile_n(c_out) < 0 || !plan_row_ok((int64_t)c_in * eb))
        return FVGB_EINVAL;
    return FVGB_OK;
}

extern "C" int fvgb_tc_plan_bytes(int64_t n_rows, int32_t K, int32_t row_bytes, size_t *bytes) {
    if (!bytes || n_rows < 0 || K < 1 || K > kMaxGroups || !plan_row_ok(row_bytes)) return FVGB_EINVAL;
    *bytes = (size_t)plan_layout(n_rows, K).bytes;
    return FVGB_OK;
}

extern "C" int fvgb_tc_plan_build(const int32_t *map, int64_t n_rows, int32_t K, int32_t row_bytes, void *plan,
                                  size_t plan_bytes, fvgb_stream_t stream) {
    size_t need = 0;
    const int st = fvgb_tc_plan_bytes(n_rows, K, row_bytes, &need);
    if (st) return st;
    if (plan_bytes < need || (n_rows > 0 && (!map || !plan)) || ((uintptr_t)plan & 15)) return FVGB_EINVAL;
    if (n_rows == 0) return FVGB_OK;
    const PlanLayout L = plan_layout(n_rows, K);
    const int pack = pack_of(row_bytes), cap = cap_of(row_bytes);
    if (cap < kTile * pack || cap + kTile * pack > kPlanSlots * 2 / 3 || cap > kPlanList) return FVGB_EINVAL;
    uint8_t *p = reinterpret_cast<uint8_t *>(plan);
    if (L.n_tiles > 0x7fffffff) return FVGB_EINVAL;
    tile_plan_kernel<<<(unsigned)L.n_tiles, kTile, 0, as_stream(stream)>>>(
        map, n_rows, K, pack, cap, reinterpret_cast<uint16_t *>(p + L.lmap_off),
        reinterpret_cast<int32_t *>(p + L.hdr_off), reinterpret_cast<int32_t *>(p + L.src_off));
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_conv_fwd_tc_planned(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                        const void *plan, int64_t n_out, int32_t K, const void *packed_w,
                                        int32_t c_out, void *y, int64_t ldy, const float *out_scale,
                                        const float *bias, int32_t relu, int32_t *err_dev, fvgb_stream_t stream) {
    int st = fvgb_tc_plan_supported(dtype, K, c_in, c_out);
    if (st) return st;
    const int eb = dtype == FVGB_E4M3 ? 1 : 2;
    if (n_out < 0 || n_x < 0 || ldx < c_in || ldy < c_out || !err_dev || (ldx * eb) % 16 != 0) return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    if (!plan || !packed_w || !y || (n_x > 0 && !x)) return FVGB_EINVAL;
    if (((uintptr_t)x & 15) || ((uintptr_t)packed_w & 15) || ((uintptr_t)y & 15) || ((uintptr_t)plan & 15))
        return FVGB_EINVAL;
    const int32_t row_bytes = c_in * eb;
    const PlanLayout L = plan_layout(n_out, K);
    const uint8_t *p = reinterpret_cast<const uint8_t *>(plan);
    PlanArgs a;
    a.x = (const uint8_t *)(n_x > 0 ? x : y);
    a.n_x = n_x;
    a.ldx_bytes = ldx * eb;
    a.lmap = reinterpret_cast<const uint16_t *>(p + L.lmap_off);
    a.hdr = reinterpret_cast<const int32_t *>(p + L.hdr_off);
    a.src = reinterpret_cast<const int32_t *>(p + L.src_off);
    a.n_out = n_out;
    a.K = K;
    a.row_bytes = row_bytes;
    a.nchunks = (int32_t)ceil_div(row_bytes, kUnitBytes);
    a.n_images = (int32_t)ceil_div(K, pack_of(row_bytes)) * a.nchunks;
    a.stride = row_stride_of(row_bytes);
    a.wpack = (const uint8_t *)packed_w;
    a.cout = c_out;
    a.y = (uint8_t *)y;
    a.ldy = ldy;
    a.scale = out_scale;
    a.bias = bias;
    a.relu = relu ? 1 : 0;
    a.err = err_dev;
    a.n_tiles = L.n_tiles;
    a.direct_store = (ldy == c_out && c_out % 8 == 0) ? 1 : 0;
    const int BN = plan_tile_n(c_out);
    const int pack = pack_of(row_bytes);
    cudaStream_t s = as_stream(stream);
    return eb == 2 ? plan_dispatch_pack<2>(BN, pack, a, s) : plan_dispatch_pack<1>(BN, pack, a, s);
}
