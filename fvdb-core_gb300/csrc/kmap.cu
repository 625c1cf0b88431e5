// Kernel-map construction (integer hot path).
//
// Reference: dispatchConvolutionKernelMap<kCUDA>
// (src/fvdb/detail/ops/convolution/pack_info/ConvolutionKernelMap.cu:14-58,104-138) runs one
// thread per (leaf, voxel slot) -- inactive slots included -- and each active thread makes K
// independent root-to-leaf NanoVDB accessor probes.
//
// Here one CTA owns one target leaf.  It stages the window of source leaves that the leaf's
// kernel footprint can touch (masks, bases, per-word prefix counts) in shared memory with one
// hash probe per source leaf, lists the leaf's active voxels, and then every thread produces
// map entries (row r, offset k) with consecutive threads writing consecutive int32s of the
// row-major [N_out, K] map: the only global traffic is the coalesced map write.
#include <cub/cub.cuh>

#include "common.cuh"

namespace fvgb {
namespace {

constexpr int kKmapThreads = 128;
constexpr int kMaxWindow = 216;  // 6x6x6 source leaves (e.g. k<=9, stride<=4); larger: hash per entry
constexpr int kMaxKSmem = 1024;  // per-offset counters kept in shared memory

struct KmapParams {
    FvgbGrid src, tgt;
    int32_t K0, K1, K2;     // user kernel size (k0 acts on ijk axis 2)
    int32_t S0, S1, S2;     // user stride (s0 acts on ijk axis 2)
    int32_t st0, st1, st2;  // floor(-k/2 + 1) per user component
    int32_t K;
    int64_t ld;
    int32_t *kmap;
    int32_t *nbsizes;
    uint32_t *tile_mask;    // OR of row occupancy per 128-row tile (K <= 32), may be null
    int32_t window;         // source leaves staged per CTA (0: not staged)
    int32_t disp_table;     // 1: per-offset displacements tabulated in shared memory
};

struct WinLeaf {
    uint64_t mask[8];
    int64_t base;  // -1: absent
    uint32_t prefix[4];  // two uint16 per word
};

__device__ inline uint32_t win_prefix(const WinLeaf &w, uint32_t word) {
    return (w.prefix[word >> 1] >> ((word & 1) * 16)) & 0xffffu;
}

// Shared memory: WinLeaf[window] | uint16 slots[512] | int32 counts[K] | uint32 tmask[8] | int32 disp[K]
__global__ void __launch_bounds__(kKmapThreads) kmap_leaf_kernel(KmapParams p) {
    extern __shared__ __align__(16) uint8_t kmap_smem[];
    WinLeaf *win = reinterpret_cast<WinLeaf *>(kmap_smem);
    uint16_t *slots = reinterpret_cast<uint16_t *>(win + p.window);
    int32_t *counts = reinterpret_cast<int32_t *>(slots + 512);
    const int nk_smem = p.nbsizes ? min(p.K, kMaxKSmem) : 0;
    uint32_t *tmask = reinterpret_cast<uint32_t *>(counts + nk_smem);
    // per-offset displacement (dx, dy, dz), 10 bits each biased by 512 (kernel extents <= 511)
    int32_t *kdisp = p.disp_table ? reinterpret_cast<int32_t *>(tmask + 8) : nullptr;
    __shared__ int32_t s_count;

    const int64_t leaf_id = blockIdx.x;
    const FvgbLeaf &tl = p.tgt.leaves[leaf_id];
    const int32_t ox = tl.origin[0], oy = tl.origin[1], oz = tl.origin[2], b = tl.batch;
    const int64_t tbase = tl.base;

    // Source coordinate range of the footprint, per ijk axis.  Axis 0 (x) uses s2/k2, axis 2 (z) s0/k0.
    const int32_t lo_x = ox * p.S2 + p.st2, hi_x = (ox + 7) * p.S2 + p.st2 + p.K2 - 1;
    const int32_t lo_y = oy * p.S1 + p.st1, hi_y = (oy + 7) * p.S1 + p.st1 + p.K1 - 1;
    const int32_t lo_z = oz * p.S0 + p.st0, hi_z = (oz + 7) * p.S0 + p.st0 + p.K0 - 1;
    const int32_t lx0 = lo_x >> 3, ly0 = lo_y >> 3, lz0 = lo_z >> 3;
    const int32_t wx = (hi_x >> 3) - lx0 + 1, wy = (hi_y >> 3) - ly0 + 1, wz = (hi_z >> 3) - lz0 + 1;
    const int32_t W = wx * wy * wz;
    const bool staged = W <= p.window;

    if (threadIdx.x == 0) s_count = 0;
    if (threadIdx.x < 8) tmask[threadIdx.x] = 0;
    if (kdisp)
        for (int k = threadIdx.x; k < p.K; k += blockDim.x) {
            const int32_t i2 = k / (p.K0 * p.K1), i1 = (k / p.K0) % p.K1, i0 = k % p.K0;
            kdisp[k] = ((p.st2 + i2 + 512) << 20) | ((p.st1 + i1 + 512) << 10) | (p.st0 + i0 + 512);
        }
    for (int k = threadIdx.x; k < nk_smem; k += blockDim.x) counts[k] = 0;
    if (staged) {
        for (int w = threadIdx.x; w < W; w += blockDim.x) {
            const int32_t ix = w / (wy * wz), iy = (w / wz) % wy, iz = w % wz;
            const int32_t id = find_leaf(p.src, b, lx0 + ix, ly0 + iy, lz0 + iz);
            WinLeaf &dst = win[w];
            if (id < 0) {
                dst.base = -1;
                continue;
            }
            const FvgbLeaf &sl = p.src.leaves[id];
#pragma unroll
            for (int q = 0; q < 8; ++q) dst.mask[q] = sl.mask[q];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dst.prefix[q] = (uint32_t)sl.prefix[2 * q] | ((uint32_t)sl.prefix[2 * q + 1] << 16);
            dst.base = sl.base;
        }
    }
    // Active voxel slots of the target leaf, in index (bit) order.
    for (int s = threadIdx.x; s < 512; s += blockDim.x) {
        const uint64_t m = tl.mask[s >> 6];
        if ((m >> (s & 63)) & 1ull) {
            const uint32_t r = tl.prefix[s >> 6] + __popcll((s & 63) ? (m & ((1ull << (s & 63)) - 1ull)) : 0ull);
            slots[r] = (uint16_t)s;
            atomicAdd(&s_count, 1);
        }
    }
    __syncthreads();

    const int32_t cnt = s_count;
    const int32_t total = cnt * p.K;
    const int64_t t0 = tbase >> 7;  // first 128-row tile this leaf's rows touch
    // (row, offset) of entry e = threadIdx.x + j * blockDim.x, advanced without divisions
    const int32_t dr = blockDim.x / p.K, dk = blockDim.x % p.K;
    int32_t r = threadIdx.x / p.K, k = threadIdx.x % p.K;
    int64_t my_tile = -1;
    uint32_t my_bits = 0;
    for (int32_t e = threadIdx.x; e < total; e += blockDim.x) {
        const uint32_t s = slots[r];
        const int32_t tx = ox + (int32_t)(s >> 6), ty = oy + (int32_t)((s >> 3) & 7), tz = oz + (int32_t)(s & 7);
        int32_t dx, dy, dz;
        if (kdisp) {
            const int32_t d = kdisp[k];
            dx = (d >> 20) - 512;
            dy = ((d >> 10) & 1023) - 512;
            dz = (d & 1023) - 512;
        } else {
            // kIdx = (i2*K1 + i1)*K0 + i0 with i2 offsetting x (extent k2) and i0 offsetting z
            dx = p.st2 + k / (p.K0 * p.K1);
            dy = p.st1 + (k / p.K0) % p.K1;
            dz = p.st0 + k % p.K0;
        }
        const int32_t sx = tx * p.S2 + dx, sy = ty * p.S1 + dy, sz = tz * p.S0 + dz;
        int64_t idx = -1;
        if (staged) {
            const int32_t w = (((sx >> 3) - lx0) * wy + ((sy >> 3) - ly0)) * wz + ((sz >> 3) - lz0);
            const WinLeaf &wl = win[w];
            if (wl.base >= 0) {
                const uint32_t bit = leaf_bit(sx, sy, sz), word = bit >> 6;
                const uint64_t m = wl.mask[word];
                if ((m >> (bit & 63)) & 1ull)
                    idx = wl.base + win_prefix(wl, word) +
                          __popcll((bit & 63) ? (m & ((1ull << (bit & 63)) - 1ull)) : 0ull);
            }
        } else {
            const int32_t id = find_leaf(p.src, b, sx >> 3, sy >> 3, sz >> 3);
            if (id >= 0) idx = leaf_voxel_index(p.src.leaves[id], leaf_bit(sx, sy, sz));
        }
        p.kmap[(tbase + r) * p.ld + k] = (int32_t)idx;
        if (idx >= 0) {
            if (p.nbsizes) {
                if (k < kMaxKSmem) atomicAdd(&counts[k], 1);
                else atomicAdd(p.nbsizes + k, 1);
            }
            if (p.tile_mask) {
                const int64_t t = (tbase + r) >> 7;
                if (t != my_tile) {
                    if (my_bits) atomicOr(&tmask[my_tile - t0], my_bits);
                    my_tile = t;
                    my_bits = 0;
                }
                my_bits |= 1u << k;
            }
        }
        k += dk;
        r += dr;
        if (k >= p.K) {
            k -= p.K;
            ++r;
        }
    }
    if (my_bits) atomicOr(&tmask[my_tile - t0], my_bits);
    if (p.nbsizes || p.tile_mask) {
        __syncthreads();
        for (int k = threadIdx.x; k < nk_smem; k += blockDim.x)
            if (counts[k]) atomicAdd(p.nbsizes + k, counts[k]);
        if (p.tile_mask && threadIdx.x < 8 && tmask[threadIdx.x]) atomicOr(p.tile_mask + t0 + threadIdx.x, tmask[threadIdx.x]);
    }
}

constexpr int kWarpLeaves = 4;      // target leaves (one per warp) per CTA
constexpr int kMaxWindowWarp = 64;  // source leaves a warp stages

// One warp per target leaf, four per CTA, with warp-private shared memory and no CTA-wide
// barrier: a leaf has ~50 active voxels on surface grids, so a whole CTA per leaf idles most of
// its threads at barriers while one warp resolves the window.  Each warp stages its source-leaf
// window (one hash probe per lane), ranks the target leaf's active slots (16 per lane), then
// builds 32 rows at a time, one lane per row: the row's window-local coordinates are computed
// once and the three offset components are walked as nested loops, so an entry costs a
// window-leaf lookup, one mask-word test and a popcount.  Rows are assembled in shared memory
// (odd row stride: no bank conflicts) and written out coalesced.
// Per-warp shared memory: WinLeaf[window] | uint16 slots[512] | int32 rows[32][K|1] |
//                         uint32 tmask[8] | int32 counts[K] (nbsizes only)
// KS > 0: cubic KS^3 kernel (loops unrolled at compile time); KS == 0: any kernel size.
template <int KS>
__global__ void __launch_bounds__(32 * kWarpLeaves) kmap_warp_kernel(KmapParams p, int32_t warp_bytes) {
    extern __shared__ __align__(16) uint8_t kmap_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t leaf_id = (int64_t)blockIdx.x * kWarpLeaves + warp;
    if (leaf_id >= p.tgt.num_leaves) return;  // warp-uniform
    const int K0 = KS ? KS : p.K0, K1 = KS ? KS : p.K1, K2 = KS ? KS : p.K2;
    const int K = KS ? KS * KS * KS : p.K, Kp = K | 1;
    uint8_t *base = kmap_smem + (size_t)warp * warp_bytes;
    WinLeaf *win = reinterpret_cast<WinLeaf *>(base);
    uint16_t *slots = reinterpret_cast<uint16_t *>(win + p.window);
    int32_t *rows = reinterpret_cast<int32_t *>(slots + 512);
    uint32_t *tmask = reinterpret_cast<uint32_t *>(rows + 32 * Kp);
    int32_t *counts = reinterpret_cast<int32_t *>(tmask + 8);

    const FvgbLeaf &tl = p.tgt.leaves[leaf_id];
    const int32_t ox = tl.origin[0], oy = tl.origin[1], oz = tl.origin[2], b = tl.batch;
    const int64_t tbase = tl.base;
    // source footprint per ijk axis (axis 0 uses s2/k2, axis 2 s0/k0) and its leaf window
    const int32_t lx0 = (ox * p.S2 + p.st2) >> 3, ly0 = (oy * p.S1 + p.st1) >> 3, lz0 = (oz * p.S0 + p.st0) >> 3;
    const int32_t wx = (((ox + 7) * p.S2 + p.st2 + p.K2 - 1) >> 3) - lx0 + 1;
    const int32_t wy = (((oy + 7) * p.S1 + p.st1 + p.K1 - 1) >> 3) - ly0 + 1;
    const int32_t wz = (((oz + 7) * p.S0 + p.st0 + p.K0 - 1) >> 3) - lz0 + 1;
    const int32_t W = wx * wy * wz;  // == p.window (the same for every leaf)

    if (lane < 8) tmask[lane] = 0;
    if (p.nbsizes)
        for (int k = lane; k < K; k += 32) counts[k] = 0;
    for (int w = lane; w < W; w += 32) {
        const int32_t ix = w / (wy * wz), iy = (w / wz) % wy, iz = w % wz;
        const int32_t id = find_leaf(p.src, b, lx0 + ix, ly0 + iy, lz0 + iz);
        WinLeaf &dst = win[w];
        if (id < 0) {
            dst.base = -1;
            continue;
        }
        const FvgbLeaf &sl = p.src.leaves[id];
#pragma unroll
        for (int q = 0; q < 8; ++q) dst.mask[q] = sl.mask[q];
#pragma unroll
        for (int q = 0; q < 4; ++q) dst.prefix[q] = (uint32_t)sl.prefix[2 * q] | ((uint32_t)sl.prefix[2 * q + 1] << 16);
        dst.base = sl.base;
    }
    {
        // active slots in index (bit) order: lane covers slots [16*lane, 16*lane + 16)
        const int word = lane >> 2, sh = (lane & 3) * 16;
        const uint64_t m = tl.mask[word];
        uint32_t bits16 = (uint32_t)(m >> sh) & 0xffffu;
        uint32_t r = (uint32_t)tl.prefix[word] + (uint32_t)__popcll(m & ((1ull << sh) - 1ull));
        while (bits16) {
            const int bp = __ffs(bits16) - 1;
            bits16 &= bits16 - 1;
            slots[r++] = (uint16_t)(16 * lane + bp);
        }
    }
    const int32_t cnt = (int32_t)tl.prefix[7] + __popcll(tl.mask[7]);
    __syncwarp();

    const int64_t t0 = tbase >> 7;  // first 128-row tile this leaf's rows touch
    const int32_t bx0 = 8 * lx0 - p.st2, by0 = 8 * ly0 - p.st1, bz0 = 8 * lz0 - p.st0;
    for (int32_t r0 = 0; r0 < cnt; r0 += 32) {
        const int32_t r = r0 + lane;
        if (r < cnt) {
            const uint32_t s = slots[r];
            // source coordinate of offset (0,0,0), relative to the window's first voxel (>= 0)
            const int32_t ux = (ox + (int32_t)(s >> 6)) * p.S2 - bx0;
            const int32_t uy = (oy + (int32_t)((s >> 3) & 7)) * p.S1 - by0;
            const int32_t uz = (oz + (int32_t)(s & 7)) * p.S0 - bz0;
            int32_t *dst = rows + lane * Kp;
            uint32_t bits = 0;
            int k = 0;
#pragma unroll
            for (int i2 = 0; i2 < K2; ++i2) {  // kIdx = (i2*K1 + i1)*K0 + i0
                const int32_t vx = ux + i2;
                const int32_t wxv = (vx >> 3) * wy;
                const uint32_t bxv = (uint32_t)(vx & 7) << 6;
#pragma unroll
                for (int i1 = 0; i1 < K1; ++i1) {
                    const int32_t vy = uy + i1;
                    const int32_t wxy = (wxv + (vy >> 3)) * wz;
                    const uint32_t bxy = bxv | ((uint32_t)(vy & 7) << 3);
#pragma unroll
                    for (int i0 = 0; i0 < K0; ++i0, ++k) {
                        const int32_t vz = uz + i0;
                        const WinLeaf &wl = win[wxy + (vz >> 3)];
                        const uint32_t bit = bxy | (uint32_t)(vz & 7);
                        const uint64_t m = wl.mask[bit >> 6];
                        int32_t idx = -1;
                        if (wl.base >= 0 && ((m >> (bit & 63)) & 1ull)) {
                            idx = (int32_t)wl.base + (int32_t)win_prefix(wl, bit >> 6) +
                                  __popcll(m & ((1ull << (bit & 63)) - 1ull));
                            bits |= 1u << k;
                            if (p.nbsizes) atomicAdd(&counts[k], 1);
                        }
                        dst[k] = idx;
                    }
                }
            }
            if (p.tile_mask && bits) atomicOr(&tmask[((tbase + r) >> 7) - t0], bits);
        }
        __syncwarp();
        const int32_t nrows = min(32, cnt - r0);
        if (p.ld == K && (KS > 0 || Kp == K)) {
            int32_t *g = p.kmap + (tbase + r0) * K;  // the block of rows is contiguous in the map
            for (int32_t e = lane; e < nrows * K; e += 32) {
                const int32_t rr = e / K;  // a constant divisor when KS > 0
                g[e] = rows[rr * Kp + (e - rr * K)];
            }
        } else {
            for (int32_t rr = 0; rr < nrows; ++rr) {
                int32_t *g = p.kmap + (tbase + r0 + rr) * p.ld;
                for (int c = lane; c < K; c += 32) g[c] = rows[rr * Kp + c];
            }
        }
        __syncwarp();
    }
    if (p.nbsizes)
        for (int k = lane; k < K; k += 32)
            if (counts[k]) atomicAdd(p.nbsizes + k, counts[k]);
    if (p.tile_mask && lane < 8 && tmask[lane]) atomicOr(p.tile_mask + t0 + lane, tmask[lane]);
}

__global__ void fill_kernel(int32_t *__restrict__ p, int64_t n, int32_t v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void transpose_kernel(const int32_t *__restrict__ kmap, int64_t n_out, int32_t K, int64_t ld,
                                 int32_t *__restrict__ mapT, int64_t n_in, int64_t ldT) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_out * K) return;
    const int64_t o = e / K;
    const int32_t k = (int32_t)(e - o * K);
    const int32_t i = kmap[o * ld + k];
    if (i >= 0 && i < n_in) mapT[(int64_t)i * ldT + k] = (int32_t)o;
}

// ---- gather-scatter neighbour map (per offset, ordered by output row) --------------------
constexpr int kNbRows = 256;

// counts[k * nblk + blk] = valid entries of column k in rows [blk*256, blk*256+256)
__global__ void __launch_bounds__(256) nb_count_kernel(const int32_t *__restrict__ kmap, int64_t n_out,
                                                       int32_t K, int64_t ld, int64_t nblk,
                                                       int32_t *__restrict__ counts) {
    const int64_t blk = blockIdx.x;
    const int64_t r0 = blk * kNbRows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = warp; k < K; k += blockDim.x / 32) {
        int c = 0;
        for (int r = lane; r < kNbRows; r += 32) {
            const int64_t row = r0 + r;
            if (row < n_out && kmap[row * ld + k] >= 0) ++c;
        }
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) counts[(int64_t)k * nblk + blk] = c;
    }
}

__global__ void __launch_bounds__(256) nb_write_kernel(const int32_t *__restrict__ kmap, int64_t n_out,
                                                       int32_t K, int64_t ld, int64_t nblk,
                                                       const int32_t *__restrict__ offs,
                                                       int32_t *__restrict__ nbmap) {
    const int64_t blk = blockIdx.x;
    const int64_t r0 = blk * kNbRows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = warp; k < K; k += blockDim.x / 32) {
        int64_t base = offs[(int64_t)k * nblk + blk];
        for (int r = lane; r < kNbRows; r += 32) {
            const int64_t row = r0 + r;
            const int32_t v = row < n_out ? kmap[row * ld + k] : -1;
            const unsigned bal = __ballot_sync(0xffffffffu, v >= 0);
            if (v >= 0) {
                const int64_t pos = base + __popc(bal & ((1u << lane) - 1u));
                nbmap[2 * pos] = v;
                nbmap[2 * pos + 1] = (int32_t)row;
            }
            base += __popc(bal);
        }
    }
}

__global__ void nb_offsets_kernel(const int32_t *__restrict__ offs, int32_t K, int64_t nblk,
                                  int64_t *__restrict__ nboffsets) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > K) return;
    nboffsets[k] = offs[(int64_t)k * nblk];  // offs has K*nblk + 1 entries (exclusive scan)
}

__global__ void masks_kernel(const int32_t *__restrict__ kmap, int64_t n_out, int32_t K, int64_t ld,
                             uint32_t *__restrict__ row_mask, uint32_t *__restrict__ tile_mask) {
    __shared__ uint32_t wm[4];
    const int64_t row = (int64_t)blockIdx.x * 128 + threadIdx.x;
    uint32_t m = 0;
    if (row < n_out)
        for (int k = 0; k < K; ++k) m |= (kmap[row * ld + k] >= 0 ? 1u : 0u) << k;
    if (row_mask && row < n_out) row_mask[row] = m;
    for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, o);
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0 && tile_mask) tile_mask[blockIdx.x] = wm[0] | wm[1] | wm[2] | wm[3];
}

// Row order of the contraction tiles: rows sorted by their occupancy mask (descending), so the
// 128 rows of a tile tend to share their present offsets and the per-tile mask skips more.
__global__ void iota_kernel(int32_t *__restrict__ v, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (int32_t)i;
}

// tile t of the sorted order: OR of its rows' masks; padding rows of the last tile get -1
__global__ void order_tiles_kernel(const uint32_t *__restrict__ sorted_mask, int64_t n_out, int32_t *__restrict__ rows,
                                   uint32_t *__restrict__ tile_mask) {
    __shared__ uint32_t wm[4];
    const int64_t r = (int64_t)blockIdx.x * 128 + threadIdx.x;
    uint32_t m = r < n_out ? sorted_mask[r] : 0u;
    if (r >= n_out) rows[r] = -1;
    for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, o);
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) tile_mask[blockIdx.x] = wm[0] | wm[1] | wm[2] | wm[3];
}

// map rows in the given order: out[128t + r] = kmap[rows[128t + r]] (-1 rows for padding)
__global__ void permute_rows_kernel(const int32_t *__restrict__ kmap, int64_t ld, int32_t K,
                                    const int32_t *__restrict__ rows, int64_t n_pad, int32_t *__restrict__ out) {
    const int64_t total = n_pad * K;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / K;
        const int k = (int)(e - r * K);
        const int32_t src = rows[r];
        out[e] = src >= 0 ? kmap[(int64_t)src * ld + k] : -1;
    }
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_kmap_row_order_workspace(int64_t n_out, int32_t K, size_t *bytes) {
    if (!bytes || n_out < 0 || n_out > INT32_MAX || K < 1 || K > 32) return FVGB_EINVAL;
    size_t cub_bytes = 0;
    if (cub::DeviceRadixSort::SortPairsDescending(nullptr, cub_bytes, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                                  (const int32_t *)nullptr, (int32_t *)nullptr, (int)n_out, 0, K) !=
        cudaSuccess)
        return FVGB_ECUDA;
    const size_t n = (size_t)n_out;
    *bytes = n * 4 /* row masks */ + n * 4 /* sorted masks */ + n * 4 /* iota */ + cub_bytes + 4 * 256;
    return FVGB_OK;
}

extern "C" int fvgb_kmap_row_order(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *rows,
                                   uint32_t *tile_mask, int32_t *sorted_map, void *workspace, size_t workspace_bytes,
                                   fvgb_stream_t stream) {
    size_t need = 0;
    int st = fvgb_kmap_row_order_workspace(n_out, K, &need);
    if (st) return st;
    if (ld < K || !rows || !tile_mask) return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    if (!kmap) return FVGB_EINVAL;
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    cudaStream_t s = as_stream(stream);
    auto carve = [](uint8_t *&p, size_t bytes) {
        uint8_t *q = p;
        p += (bytes + 255) & ~(size_t)255;
        return q;
    };
    uint8_t *p = reinterpret_cast<uint8_t *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    const size_t n = (size_t)n_out;
    uint32_t *mask = (uint32_t *)carve(p, n * 4);
    uint32_t *smask = (uint32_t *)carve(p, n * 4);
    int32_t *iota = (int32_t *)carve(p, n * 4);
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairsDescending(nullptr, cub_bytes, mask, smask, iota, rows, (int)n_out, 0, K, s);
    if ((size_t)(p - (uint8_t *)workspace) + cub_bytes > workspace_bytes) return FVGB_ENOSPACE;
    const unsigned tiles = (unsigned)ceil_div(n_out, 128);
    masks_kernel<<<tiles, 128, 0, s>>>(kmap, n_out, K, ld, mask, nullptr);
    iota_kernel<<<(unsigned)ceil_div(n_out, 256), 256, 0, s>>>(iota, n_out);
    if (cub::DeviceRadixSort::SortPairsDescending(p, cub_bytes, mask, smask, iota, rows, (int)n_out, 0, K, s) !=
        cudaSuccess)
        return launch_status();
    order_tiles_kernel<<<tiles, 128, 0, s>>>(smask, n_out, rows, tile_mask);
    int launched = 3;
    if (sorted_map) {
        const int64_t n_pad = (int64_t)tiles * 128;
        const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n_pad * K, 256), (int64_t)device_sm_count() * 16);
        permute_rows_kernel<<<blocks, 256, 0, s>>>(kmap, ld, K, rows, n_pad, sorted_map);
        ++launched;
    }
    count_launches(launched);
    return launch_status();
}

extern "C" int fvgb_kmap_build(const FvgbGrid *src, const FvgbGrid *tgt, const int32_t ksize[3],
                               const int32_t stride[3], int32_t *kmap, int64_t ld, int32_t *nbsizes,
                               uint32_t *tile_mask, fvgb_stream_t stream) {
    if (!src || !tgt || !ksize || !stride) return FVGB_EINVAL;
    for (int a = 0; a < 3; ++a)
        if (ksize[a] < 1 || stride[a] < 1) return FVGB_EINVAL;
    if (src->num_grids != tgt->num_grids) return FVGB_EINVAL;
    const int64_t K = (int64_t)ksize[0] * ksize[1] * ksize[2];
    if (K > (1 << 20) || ld < K) return FVGB_EINVAL;
    if (tile_mask && K > 32) return FVGB_EINVAL;
    if (tgt->num_voxels == 0 || tgt->num_leaves == 0) return FVGB_OK;
    if (!kmap) return FVGB_EINVAL;
    if (tgt->num_leaves > INT32_MAX) return FVGB_EINVAL;
    KmapParams p;
    p.src = *src;
    p.tgt = *tgt;
    p.K0 = ksize[0]; p.K1 = ksize[1]; p.K2 = ksize[2];
    p.S0 = stride[0]; p.S1 = stride[1]; p.S2 = stride[2];
    // kernelStart = floor(-K/2 + 1) (ConvolutionKernelMap.cu:114-116)
    p.st0 = (int32_t)floor(-ksize[0] / 2.0 + 1.0);
    p.st1 = (int32_t)floor(-ksize[1] / 2.0 + 1.0);
    p.st2 = (int32_t)floor(-ksize[2] / 2.0 + 1.0);
    p.K = (int32_t)K;
    p.ld = ld;
    p.kmap = kmap;
    p.nbsizes = nbsizes;
    p.tile_mask = tile_mask;
    // The source-leaf window of a target leaf has the same extent for every leaf (leaf origins
    // are multiples of 8, so origin*stride is too): size shared memory to it.
    auto span = [](int32_t s, int32_t st, int32_t k) { return ((7 * s + st + k - 1) >> 3) - (st >> 3) + 1; };
    const int64_t W = (int64_t)span(p.S2, p.st2, p.K2) * span(p.S1, p.st1, p.K1) * span(p.S0, p.st0, p.K0);
    p.window = W <= kMaxWindow ? (int32_t)W : 0;
    const int nk_smem = nbsizes ? (int)std::min<int64_t>(K, kMaxKSmem) : 0;
    p.disp_table = (K <= kMaxKSmem && ksize[0] <= 511 && ksize[1] <= 511 && ksize[2] <= 511) ? 1 : 0;
    if (p.window > 0 && p.window <= kMaxWindowWarp && K <= 32) {
        // one warp per target leaf (the common case: 3^3, 2^3, ... kernels)
        const size_t wb = ((size_t)p.window * sizeof(WinLeaf) + 512 * sizeof(uint16_t) + 32 * (size_t)(K | 1) * 4 +
                           8 * 4 + (nbsizes ? (size_t)K * 4 : 0) + 15) & ~(size_t)15;
        const unsigned blocks = (unsigned)ceil_div(tgt->num_leaves, (int64_t)kWarpLeaves);
        const size_t smem = wb * kWarpLeaves;
        const bool cube = ksize[0] == ksize[1] && ksize[1] == ksize[2];
        if (cube && ksize[0] == 3)
            kmap_warp_kernel<3><<<blocks, 32 * kWarpLeaves, smem, as_stream(stream)>>>(p, (int32_t)wb);
        else if (cube && ksize[0] == 2)
            kmap_warp_kernel<2><<<blocks, 32 * kWarpLeaves, smem, as_stream(stream)>>>(p, (int32_t)wb);
        else
            kmap_warp_kernel<0><<<blocks, 32 * kWarpLeaves, smem, as_stream(stream)>>>(p, (int32_t)wb);
        count_launches(1);
        return launch_status();
    }
    const size_t smem = (size_t)p.window * sizeof(WinLeaf) + 512 * sizeof(uint16_t) + nk_smem * 4 + 8 * 4 +
                        (p.disp_table ? (size_t)K * 4 : 0);
    kmap_leaf_kernel<<<(unsigned)tgt->num_leaves, kKmapThreads, smem, as_stream(stream)>>>(p);
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_kmap_transpose(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *mapT,
                                   int64_t n_in, int64_t ldT, fvgb_stream_t stream) {
    if (K < 1 || ld < K || ldT < K || n_out < 0 || n_in < 0) return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    if (n_in > 0) fill_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n_in * ldT, 256), 65535 * 8), 256, 0, s>>>(mapT, n_in * ldT, -1);
    if (n_out > 0)
        transpose_kernel<<<(unsigned)ceil_div(n_out * K, 256), 256, 0, s>>>(kmap, n_out, K, ld, mapT, n_in, ldT);
    count_launches((n_in > 0) + (n_out > 0));
    return launch_status();
}

extern "C" int fvgb_nbmap_workspace(int64_t n_out, int32_t K, size_t *bytes) {
    if (!bytes || n_out < 0 || K < 1) return FVGB_EINVAL;
    const int64_t nblk = ceil_div(n_out > 0 ? n_out : 1, kNbRows);
    const int64_t m = nblk * K + 1;
    size_t c = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, c, (int32_t *)nullptr, (int32_t *)nullptr, m);
    *bytes = c + (size_t)m * 4 * 2 + 1024;
    return FVGB_OK;
}

extern "C" int fvgb_nbmap_build(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *nbmap,
                                int64_t *nboffsets, void *workspace, size_t workspace_bytes,
                                fvgb_stream_t stream) {
    if (K < 1 || ld < K || n_out < 0 || !nboffsets) return FVGB_EINVAL;
    size_t need = 0;
    fvgb_nbmap_workspace(n_out, K, &need);
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    cudaStream_t s = as_stream(stream);
    const int64_t nblk = ceil_div(n_out > 0 ? n_out : 1, kNbRows);
    const int64_t m = nblk * K + 1;
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    int32_t *counts = reinterpret_cast<int32_t *>(base);
    int32_t *offs = counts + ((m + 63) / 64 * 64);
    void *tmp = offs + ((m + 63) / 64 * 64);
    size_t tb = need - 1024 - (size_t)m * 8;
    cudaMemsetAsync(counts, 0, sizeof(int32_t) * m, s);
    if (n_out > 0) nb_count_kernel<<<(unsigned)nblk, 256, 0, s>>>(kmap, n_out, K, ld, nblk, counts);
    cub::DeviceScan::ExclusiveSum(tmp, tb, counts, offs, m, s);
    if (n_out > 0) nb_write_kernel<<<(unsigned)nblk, 256, 0, s>>>(kmap, n_out, K, ld, nblk, offs, nbmap);
    nb_offsets_kernel<<<(unsigned)ceil_div(K + 1, 128), 128, 0, s>>>(offs, K, nblk, nboffsets);
    count_launches(n_out > 0 ? 3 : 1);
    return launch_status();
}

extern "C" int fvgb_kmap_masks(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, uint32_t *row_mask,
                               uint32_t *tile_mask, fvgb_stream_t stream) {
    if (K < 1 || K > 32 || ld < K || n_out < 0) return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    masks_kernel<<<(unsigned)ceil_div(n_out, 128), 128, 0, as_stream(stream)>>>(kmap, n_out, K, ld, row_mask,
                                                                               tile_mask);
    count_launches(1);
    return launch_status();
}
