// Device grid builder: jagged ijk -> sorted unique voxels in NanoVDB order -> leaf table
// + leaf hash.  No host synchronisation inside any entry point; sizes that the caller
// must allocate from (unique count, leaf count) are left in device memory.
//
// Reference behaviour replaced: dispatchCreateNanoGridFromIJK<kCUDA>
// (src/fvdb/detail/ops/BuildGridFromIjk.cu:26-83), which loops over the grids on the
// host and calls nanovdb::tools::cuda::voxelsToGrid per grid.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cub/cub.cuh>

#include "common.cuh"

namespace fvgb {
namespace {

struct SortWs {
    uint64_t *keys_a, *keys_b;
    int32_t *bidx_a, *bidx_b;
    int32_t *flags;  // n+1
    void *cub_tmp;
    size_t cub_bytes;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

size_t cub_sort_bytes(int64_t n) {
    size_t a = 0, b = 0, c = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (uint64_t *)nullptr, (uint64_t *)nullptr,
                                    (int32_t *)nullptr, (int32_t *)nullptr, n, 0, 63);
    cub::DeviceRadixSort::SortPairs(nullptr, b, (int32_t *)nullptr, (int32_t *)nullptr,
                                    (uint64_t *)nullptr, (uint64_t *)nullptr, n, 0, 32);
    cub::DeviceScan::ExclusiveSum(nullptr, c, (int32_t *)nullptr, (int32_t *)nullptr, n + 1);
    size_t m = a > b ? a : b;
    return m > c ? m : c;
}

size_t sort_ws_layout(int64_t n, SortWs *ws, char *base) {
    size_t off = 0;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off = align_up(off + bytes, 256);
        return p;
    };
    SortWs w;
    w.keys_a = (uint64_t *)take(nn * 8);
    w.keys_b = (uint64_t *)take(nn * 8);
    w.bidx_a = (int32_t *)take(nn * 4);
    w.bidx_b = (int32_t *)take(nn * 4);
    w.flags = (int32_t *)take((nn + 1) * 4);
    w.cub_bytes = cub_sort_bytes(n);
    w.cub_tmp = take(w.cub_bytes);
    if (ws) *ws = w;
    return off;
}

// box_lo/box_hi: bounds every coordinate must lie in (the whole coordinate range when the
// caller promises none); a coordinate outside raises FVGB_ERANGE.
// fold > 0: every key agrees above bit `fold` (coordinates inside a box), so the grid index
// replaces those bits and one radix sort orders by (grid, key).
__global__ void keys_kernel(const int32_t *__restrict__ ijk, const int64_t *__restrict__ joff,
                            int32_t B, int64_t n, int3 box_lo, int3 box_hi, int32_t fold,
                            uint64_t *__restrict__ keys, int32_t *__restrict__ bidx, int32_t *__restrict__ err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t x = ijk[3 * i], y = ijk[3 * i + 1], z = ijk[3 * i + 2];
    if (!coord_in_range(x) || !coord_in_range(y) || !coord_in_range(z) || x < box_lo.x || x > box_hi.x ||
        y < box_lo.y || y > box_hi.y || z < box_lo.z || z > box_hi.z)
        atomicExch(err, FVGB_ERANGE);
    const int32_t b = batch_of(joff, B, i);
    uint64_t k = order_key(x, y, z);
    if (fold > 0) k = (k & ((1ull << fold) - 1ull)) | ((uint64_t)b << fold);
    keys[i] = k;
    bidx[i] = b;
}

// One past the highest order_key bit that can differ between coordinates in [lo, hi] (per
// axis): coordinate bits above the highest bit where lo and hi differ are shared by the whole
// box.  Coordinate bit c of x lands on key bit 6+c (leaf), 14+c (lower node), 24+c (upper node)
// or 42+c (root); y sits 3, 4, 5 or 9 positions below x in those fields and z twice as far.
// Within an axis a higher coordinate bit always maps to a higher key bit, so all keys of the
// box agree above the returned bit and sorting only the bits below it orders them exactly as a
// full 63-bit sort.
int order_key_end_bit(const int32_t lo[3], const int32_t hi[3]) {
    static const int kBase[3] = {6, 3, 0};  // x, y, z offset of the leaf field
    int end = 1;
    for (int a = 0; a < 3; ++a) {
        if (lo[a] > hi[a]) continue;
        const uint32_t d = (uint32_t)lo[a] ^ (uint32_t)hi[a];
        if (!d) continue;
        int h = 31;
        while (!((d >> h) & 1u)) --h;
        int kb;
        if (h < 3)
            kb = kBase[a] + h;                    // leaf: bits 0..8
        else if (h < 7)
            kb = 9 + 4 * (2 - a) + (h - 3);       // lower node: x 17..20, y 13..16, z 9..12
        else if (h < 12)
            kb = 21 + 5 * (2 - a) + (h - 7);      // upper node: x 31..35, y 26..30, z 21..25
        else if (h < 21)
            kb = 36 + 9 * (2 - a) + (h - 12);     // root: x 54..62, y 45..53, z 36..44
        else
            return 63;
        if (kb + 1 > end) end = kb + 1;
    }
    return end;
}

__global__ void unique_flags_kernel(const uint64_t *__restrict__ keys,
                                    const int32_t *__restrict__ bidx, int64_t n,
                                    int32_t *__restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { flags[i] = 0; return; }
    flags[i] = (i == 0 || keys[i] != keys[i - 1] || bidx[i] != bidx[i - 1]) ? 1 : 0;
}

// low_mask / high: a folded key keeps the order key's bits under low_mask; the bits above are
// `high` for every voxel (no folding: low_mask all ones, high zero).
__global__ void unique_write_kernel(const uint64_t *__restrict__ keys,
                                    const int32_t *__restrict__ bidx,
                                    const int32_t *__restrict__ pos, int64_t n, uint64_t low_mask,
                                    uint64_t high, int32_t *__restrict__ out_ijk) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool first = (i == 0 || keys[i] != keys[i - 1] || bidx[i] != bidx[i - 1]);
    if (!first) return;
    int32_t x, y, z;
    key_to_coord((keys[i] & low_mask) | high, x, y, z);
    const int64_t p = pos[i];
    out_ijk[3 * p] = x;
    out_ijk[3 * p + 1] = y;
    out_ijk[3 * p + 2] = z;
}

// out_joff[b] = number of unique voxels in grids < b  (bidx sorted ascending)
__global__ void offsets_kernel(const int32_t *__restrict__ bidx, const int32_t *__restrict__ pos,
                               int64_t n, int32_t B, int64_t *__restrict__ out_joff) {
    const int32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > B) return;
    int64_t lo = 0, hi = n;  // first i with bidx[i] >= b
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (bidx[mid] < b) lo = mid + 1; else hi = mid;
    }
    out_joff[b] = pos[lo];  // pos has n+1 entries; pos[n] = total
}

__global__ void leaf_flags_kernel(const int32_t *__restrict__ ijk, const int64_t *__restrict__ joff,
                                  int32_t B, int64_t n, int32_t *__restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i >= joff[B]) {  // n is a capacity; the voxel count lives on the device
        flags[i] = 0;
        return;
    }
    int32_t f = 1;
    if (i > 0) {
        const int32_t b0 = batch_of(joff, B, i - 1), b1 = batch_of(joff, B, i);
        f = (b0 != b1 || (ijk[3 * i] >> 3) != (ijk[3 * i - 3] >> 3) ||
             (ijk[3 * i + 1] >> 3) != (ijk[3 * i - 2] >> 3) ||
             (ijk[3 * i + 2] >> 3) != (ijk[3 * i - 1] >> 3)) ? 1 : 0;
    }
    flags[i] = f;
}

__global__ void leaf_count_kernel(const int32_t *__restrict__ ids, const int64_t *__restrict__ joff, int32_t B,
                                  int64_t *__restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int64_t n = joff[B];
    out[0] = n > 0 ? (int64_t)ids[n - 1] : 0;  // inclusive scan
    out[1] = n;
}

__global__ void leaf_fill_kernel(const int32_t *__restrict__ ijk, const int64_t *__restrict__ joff,
                                 int32_t B, int64_t n, const int32_t *__restrict__ leaf_ids,
                                 FvgbLeaf *__restrict__ leaves) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t id = leaf_ids[i] - 1;  // inclusive scan
    const int32_t x = ijk[3 * i], y = ijk[3 * i + 1], z = ijk[3 * i + 2];
    FvgbLeaf &L = leaves[id];
    const bool first = (i == 0) || leaf_ids[i - 1] != leaf_ids[i];
    if (first) {
        L.origin[0] = x & ~7;
        L.origin[1] = y & ~7;
        L.origin[2] = z & ~7;
        L.batch = batch_of(joff, B, i);
        L.base = i;
    }
    const uint32_t bit = leaf_bit(x, y, z);
    atomicOr(reinterpret_cast<unsigned long long *>(&L.mask[bit >> 6]), 1ull << (bit & 63));
}

__global__ void leaf_finish_kernel(FvgbLeaf *__restrict__ leaves, int64_t L, int32_t *__restrict__ slots,
                                   int64_t cap) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= L) return;
    FvgbLeaf &lf = leaves[id];
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        lf.prefix[w] = (uint16_t)run;
        run += __popcll(lf.mask[w]);
    }
    const uint64_t cap_mask = (uint64_t)cap - 1;
    uint64_t h = leaf_hash(lf.batch, lf.origin[0] >> 3, lf.origin[1] >> 3, lf.origin[2] >> 3) & cap_mask;
    for (int64_t probe = 0; probe < cap; ++probe) {
        const int32_t prev = atomicCAS(slots + h, -1, (int32_t)id);
        if (prev == -1) break;
        h = (h + 1) & cap_mask;
    }
}

// One coordinate of VoxelCoordTransform(1/w, -o/w).apply(p).round() in the arithmetic type T
// that the reference uses for the points' dtype (opmath: double for FP64 points, float for
// FP32/FP16/BF16): scale and translation are the double quotients rounded once to T, the
// transform is one fused multiply-add in T, and round() is floor(v + 1/2) in T
// (src/fvdb/detail/VoxelCoordTransform.h:86-110,230-330, BuildGridFromPoints.cu:27-43).
template <typename T>
__device__ __forceinline__ int32_t voxelise(T p, double w, double o);
template <>
__device__ __forceinline__ int32_t voxelise<float>(float p, double w, double o) {
    const float s = (float)(1.0 / w), t = (float)(-o / w);
    return (int32_t)floorf(__fadd_rn(__fmaf_rn(p, s, t), 0.5f));
}
template <>
__device__ __forceinline__ int32_t voxelise<double>(double p, double w, double o) {
    const double s = 1.0 / w, t = -o / w;
    return (int32_t)floor(__dadd_rn(__fma_rn(p, s, t), 0.5));
}

template <typename P>
__device__ __forceinline__ float point_as_float(P v) { return (float)v; }
template <>
__device__ __forceinline__ float point_as_float<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ float point_as_float<__half>(__half v) { return __half2float(v); }

// P: storage type of the points; T: arithmetic type (double for FP64 points, else float).
template <typename P, typename T>
__global__ void points_kernel(const P *__restrict__ pts, const int64_t *__restrict__ joff, int32_t B, int64_t n,
                              const double *__restrict__ vs, const double *__restrict__ org,
                              int32_t *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t b = batch_of(joff, B, i);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T v;
        if constexpr (sizeof(T) == 8) v = (T)pts[3 * i + a];
        else v = point_as_float<P>(pts[3 * i + a]);
        out[3 * i + a] = voxelise<T>(v, vs[3 * b + a], org[3 * b + a]);
    }
}

__global__ void conv_candidates_kernel(FvgbGrid g, int3 ks, int3 st, int coarse, int32_t kc,
                                       int32_t *__restrict__ out, uint8_t *__restrict__ valid) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.num_voxels) return;
    const int32_t x = g.ijk[3 * i], y = g.ijk[3 * i + 1], z = g.ijk[3 * i + 2];
    if (coarse) {
        // floor(ijk / stride) with the stride Coord applied x<->s0 (CoarseIjkForFineGrid.cu:34-35),
        // in integer arithmetic (exact for int32 inputs; avoids FP64 on the device)
        auto fdiv = [](int32_t a, int32_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
        out[3 * i] = fdiv(x, st.x);
        out[3 * i + 1] = fdiv(y, st.y);
        out[3 * i + 2] = fdiv(z, st.z);
        valid[i] = 1;
        return;
    }
    const int lo0 = (ks.x % 2 == 0) ? 0 : -(ks.x - 1) / 2, hi0 = (ks.x % 2 == 0) ? ks.x - 1 : (ks.x - 1) / 2;
    const int lo1 = (ks.y % 2 == 0) ? 0 : -(ks.y - 1) / 2, hi1 = (ks.y % 2 == 0) ? ks.y - 1 : (ks.y - 1) / 2;
    const int lo2 = (ks.z % 2 == 0) ? 0 : -(ks.z - 1) / 2, hi2 = (ks.z % 2 == 0) ? ks.z - 1 : (ks.z - 1) / 2;
    int64_t c = i * kc;
    // BuildGridForConv.cu:99-121: di over k0 moves z, dk over k2 moves x; C remainder
    for (int di = lo0; di <= hi0; ++di)
        for (int dj = lo1; dj <= hi1; ++dj)
            for (int dk = lo2; dk <= hi2; ++dk, ++c) {
                const int32_t dx = x + dk, dy = y + dj, dz = z + di;
                const bool ok = (dx % st.z == 0) && (dy % st.y == 0) && (dz % st.x == 0);
                valid[c] = ok ? 1 : 0;
                out[3 * c] = ok ? dx / st.z : 0;
                out[3 * c + 1] = ok ? dy / st.y : 0;
                out[3 * c + 2] = ok ? dz / st.x : 0;
            }
}

__global__ void compact_flags_kernel(const uint8_t *__restrict__ valid, int64_t n, int32_t *__restrict__ f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    f[i] = (i < n && valid[i]) ? 1 : 0;
}

__global__ void compact_write_kernel(const int32_t *__restrict__ ijk, const uint8_t *__restrict__ valid,
                                     const int32_t *__restrict__ pos, int64_t n, int32_t *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !valid[i]) return;
    const int64_t p = pos[i];
    out[3 * p] = ijk[3 * i];
    out[3 * p + 1] = ijk[3 * i + 1];
    out[3 * p + 2] = ijk[3 * i + 2];
}

__global__ void compact_offsets_kernel(const int64_t *__restrict__ src_joff, int32_t B, int64_t per,
                                       const int32_t *__restrict__ pos, int64_t *__restrict__ out) {
    const int32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > B) return;
    out[b] = pos[src_joff[b] * per];
}

constexpr int kThreads = 256;
inline unsigned blocks_for(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, kThreads); }

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_ijk_sort_unique_workspace(int64_t n, int32_t num_grids, size_t *bytes) {
    if (!bytes || n < 0 || num_grids < 1) return FVGB_EINVAL;
    *bytes = sort_ws_layout(n, nullptr, nullptr) + 256;
    return FVGB_OK;
}

namespace fvgb {
namespace {
int sort_unique(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids, int64_t n, const int32_t *box_lo,
                const int32_t *box_hi, int32_t *out_ijk, int64_t *out_joffsets, int32_t *err_dev, void *workspace,
                size_t workspace_bytes, fvgb_stream_t stream) {
    if (n < 0 || num_grids < 1 || !joffsets || !out_joffsets || !err_dev) return FVGB_EINVAL;
    if (n > 0 && (!ijk || !out_ijk)) return FVGB_EINVAL;
    if (n >= (int64_t)INT32_MAX) return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    SortWs w;
    const size_t need = sort_ws_layout(n, &w, base);
    if (!workspace || need + 256 > workspace_bytes) return FVGB_ENOSPACE;
    if (n == 0) {
        if (cudaMemsetAsync(out_joffsets, 0, sizeof(int64_t) * (num_grids + 1), s) != cudaSuccess)
            return launch_status();
        return launch_status();
    }
    int3 lo = make_int3(INT32_MIN, INT32_MIN, INT32_MIN), hi = make_int3(INT32_MAX, INT32_MAX, INT32_MAX);
    int end_bit = 63;
    if (box_lo && box_hi) {
        for (int a = 0; a < 3; ++a)
            if (box_lo[a] > box_hi[a]) return FVGB_EINVAL;
        lo = make_int3(box_lo[0], box_lo[1], box_lo[2]);
        hi = make_int3(box_hi[0], box_hi[1], box_hi[2]);
        end_bit = order_key_end_bit(box_lo, box_hi);
    }
    int grid_bits = 0;
    while ((1ll << grid_bits) < num_grids) ++grid_bits;
    // inside a box the keys agree above end_bit: the grid index takes those bits (one sort)
    const int fold = (box_lo && box_hi && num_grids > 1 && end_bit + grid_bits <= 63) ? end_bit : 0;
    uint64_t low_mask = ~0ull, high = 0;
    if (fold) {
        low_mask = (1ull << fold) - 1ull;
        high = order_key(box_lo[0], box_lo[1], box_lo[2]) & ~low_mask;
    }
    keys_kernel<<<blocks_for(n), kThreads, 0, s>>>(ijk, joffsets, num_grids, n, lo, hi, fold, w.keys_a, w.bidx_a,
                                                   err_dev);
    size_t tb = w.cub_bytes;
    // 1) sort by voxel key (stable radix, only the bits that can differ), 2) stable sort by grid
    //    index -- or one sort when the grid index is folded into the key: grids stay contiguous
    //    and every grid's voxels stay in key order.
    cub::DeviceRadixSort::SortPairs(w.cub_tmp, tb, w.keys_a, w.keys_b, w.bidx_a, w.bidx_b, n, 0,
                                    fold ? fold + grid_bits : end_bit, s);
    const uint64_t *keys = w.keys_b;
    const int32_t *bidx = w.bidx_b;
    if (num_grids > 1 && !fold) {
        tb = w.cub_bytes;
        cub::DeviceRadixSort::SortPairs(w.cub_tmp, tb, w.bidx_b, w.bidx_a, w.keys_b, w.keys_a, n, 0, grid_bits, s);
        keys = w.keys_a;
        bidx = w.bidx_a;
    }
    unique_flags_kernel<<<blocks_for(n + 1), kThreads, 0, s>>>(keys, bidx, n, w.flags);
    tb = w.cub_bytes;
    // exclusive scan in place over n+1 flags: pos[n] = unique count
    int32_t *pos = reinterpret_cast<int32_t *>(w.keys_a == keys ? (void *)w.keys_b : (void *)w.keys_a);
    cub::DeviceScan::ExclusiveSum(w.cub_tmp, tb, w.flags, pos, n + 1, s);
    unique_write_kernel<<<blocks_for(n), kThreads, 0, s>>>(keys, bidx, pos, n, low_mask, high, out_ijk);
    offsets_kernel<<<(unsigned)ceil_div(num_grids + 1, kThreads), kThreads, 0, s>>>(bidx, pos, n, num_grids,
                                                                                    out_joffsets);
    count_launches(4);
    return launch_status();
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_ijk_sort_unique(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids,
                                    int64_t n, int32_t *out_ijk, int64_t *out_joffsets,
                                    int32_t *err_dev, void *workspace, size_t workspace_bytes,
                                    fvgb_stream_t stream) {
    return fvgb::sort_unique(ijk, joffsets, num_grids, n, nullptr, nullptr, out_ijk, out_joffsets, err_dev,
                             workspace, workspace_bytes, stream);
}

extern "C" int fvgb_ijk_sort_unique_in_box(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids,
                                           int64_t n, const int32_t *box_lo, const int32_t *box_hi,
                                           int32_t *out_ijk, int64_t *out_joffsets, int32_t *err_dev,
                                           void *workspace, size_t workspace_bytes, fvgb_stream_t stream) {
    if (!box_lo || !box_hi) return FVGB_EINVAL;
    return fvgb::sort_unique(ijk, joffsets, num_grids, n, box_lo, box_hi, out_ijk, out_joffsets, err_dev,
                             workspace, workspace_bytes, stream);
}

extern "C" int fvgb_scan_workspace(int64_t n, size_t *bytes) {
    if (!bytes || n < 0) return FVGB_EINVAL;
    size_t c = 0;
    cub::DeviceScan::InclusiveSum(nullptr, c, (int32_t *)nullptr, (int32_t *)nullptr, n + 1);
    size_t c2 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, c2, (int32_t *)nullptr, (int32_t *)nullptr, n + 1);
    if (c2 > c) c = c2;
    *bytes = c + (size_t)(n + 2) * 4 + 512;
    return FVGB_OK;
}

extern "C" int fvgb_grid_leaf_scan(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids,
                                   int64_t n, int32_t *leaf_ids, int64_t *num_leaves_dev,
                                   void *workspace, size_t workspace_bytes, fvgb_stream_t stream) {
    if (n < 0 || num_grids < 1 || !num_leaves_dev || (n > 0 && (!ijk || !leaf_ids))) return FVGB_EINVAL;
    size_t need = 0;
    fvgb_scan_workspace(n, &need);
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    cudaStream_t s = as_stream(stream);
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    int32_t *flags = reinterpret_cast<int32_t *>(base);
    void *tmp = base + ((size_t)(n + 2) * 4 + 255) / 256 * 256;
    size_t tb = need - ((size_t)(n + 2) * 4 + 255) / 256 * 256 - 256;
    if (n > 0) {
        leaf_flags_kernel<<<blocks_for(n), kThreads, 0, s>>>(ijk, joffsets, num_grids, n, flags);
        cub::DeviceScan::InclusiveSum(tmp, tb, flags, leaf_ids, n, s);
    }
    leaf_count_kernel<<<1, 32, 0, s>>>(leaf_ids, joffsets, num_grids, num_leaves_dev);
    count_launches(n > 0 ? 2 : 1);
    return launch_status();
}

extern "C" int fvgb_grid_index_build(const FvgbGrid *g, const int32_t *leaf_ids, fvgb_stream_t stream) {
    if (!g || g->num_voxels < 0 || g->num_leaves < 0) return FVGB_EINVAL;
    if (g->hash_capacity < 2 * g->num_leaves || (g->hash_capacity & (g->hash_capacity - 1)) != 0)
        return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    FvgbLeaf *leaves = const_cast<FvgbLeaf *>(g->leaves);
    int32_t *slots = const_cast<int32_t *>(g->hash_slots);
    if (g->hash_capacity > 0 && cudaMemsetAsync(slots, 0xff, sizeof(int32_t) * g->hash_capacity, s) != cudaSuccess)
        return launch_status();
    if (g->num_leaves > 0 && cudaMemsetAsync(leaves, 0, sizeof(FvgbLeaf) * g->num_leaves, s) != cudaSuccess)
        return launch_status();
    if (g->num_voxels > 0) {
        leaf_fill_kernel<<<blocks_for(g->num_voxels), kThreads, 0, s>>>(g->ijk, g->voxel_offsets, g->num_grids,
                                                                       g->num_voxels, leaf_ids, leaves);
        leaf_finish_kernel<<<blocks_for(g->num_leaves), kThreads, 0, s>>>(leaves, g->num_leaves, slots,
                                                                         g->hash_capacity);
        count_launches(2);
    }
    return launch_status();
}

extern "C" int fvgb_points_to_ijk(int32_t dtype, const void *points, const int64_t *joffsets, int32_t num_grids,
                                  int64_t n, const double *voxel_sizes, const double *origins,
                                  int32_t *out_ijk, fvgb_stream_t stream) {
    if (dtype != FVGB_F32 && dtype != FVGB_F64 && dtype != FVGB_F16 && dtype != FVGB_BF16) return FVGB_ETYPE;
    if (n < 0 || num_grids < 1 || (n > 0 && (!points || !out_ijk || !voxel_sizes || !origins || !joffsets)))
        return FVGB_EINVAL;
    if (n == 0) return FVGB_OK;
    cudaStream_t s = as_stream(stream);
    switch (dtype) {
        case FVGB_F64:
            points_kernel<double, double><<<blocks_for(n), kThreads, 0, s>>>(
                (const double *)points, joffsets, num_grids, n, voxel_sizes, origins, out_ijk);
            break;
        case FVGB_F16:
            points_kernel<__half, float><<<blocks_for(n), kThreads, 0, s>>>(
                (const __half *)points, joffsets, num_grids, n, voxel_sizes, origins, out_ijk);
            break;
        case FVGB_BF16:
            points_kernel<__nv_bfloat16, float><<<blocks_for(n), kThreads, 0, s>>>(
                (const __nv_bfloat16 *)points, joffsets, num_grids, n, voxel_sizes, origins, out_ijk);
            break;
        default:
            points_kernel<float, float><<<blocks_for(n), kThreads, 0, s>>>(
                (const float *)points, joffsets, num_grids, n, voxel_sizes, origins, out_ijk);
    }
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_conv_grid_candidates(const FvgbGrid *g, const int32_t ksize[3], const int32_t stride[3],
                                         int32_t *out_ijk, uint8_t *out_valid, fvgb_stream_t stream) {
    if (!g || !ksize || !stride) return FVGB_EINVAL;
    for (int a = 0; a < 3; ++a)
        if (ksize[a] < 1 || stride[a] < 1) return FVGB_EINVAL;
    if (g->num_voxels == 0) return FVGB_OK;
    const int coarse = (stride[0] == 1 && stride[1] == 1 && stride[2] == 1) ||
                       (stride[0] == ksize[0] && stride[1] == ksize[1] && stride[2] == ksize[2]);
    const int32_t kc = coarse ? 1 : ksize[0] * ksize[1] * ksize[2];
    conv_candidates_kernel<<<blocks_for(g->num_voxels), kThreads, 0, as_stream(stream)>>>(
        *g, make_int3(ksize[0], ksize[1], ksize[2]), make_int3(stride[0], stride[1], stride[2]), coarse, kc,
        out_ijk, out_valid);
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_compact_ijk(const int32_t *ijk, const uint8_t *valid, const int64_t *src_joffsets,
                                int32_t num_grids, int64_t per_voxel, int64_t n, int32_t *out_ijk,
                                int64_t *out_joffsets, void *workspace, size_t workspace_bytes,
                                fvgb_stream_t stream) {
    if (n < 0 || num_grids < 1 || per_voxel < 1 || !src_joffsets || !out_joffsets) return FVGB_EINVAL;
    size_t need = 0;
    fvgb_scan_workspace(n, &need);
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    cudaStream_t s = as_stream(stream);
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    int32_t *flags = reinterpret_cast<int32_t *>(base);
    const size_t head = ((size_t)(n + 2) * 4 + 255) / 256 * 256;
    void *tmp = base + head;
    size_t tb = need - head - 256;
    compact_flags_kernel<<<blocks_for(n + 1), kThreads, 0, s>>>(valid, n, flags);
    cub::DeviceScan::ExclusiveSum(tmp, tb, flags, flags, n + 1, s);  // in place: flags -> positions
    compact_write_kernel<<<blocks_for(n), kThreads, 0, s>>>(ijk, valid, flags, n, out_ijk);
    compact_offsets_kernel<<<(unsigned)ceil_div(num_grids + 1, kThreads), kThreads, 0, s>>>(
        src_joffsets, num_grids, per_voxel, flags, out_joffsets);
    count_launches(3);
    return launch_status();
}

namespace fvgb {
namespace {
__global__ void ijk_to_index_kernel(FvgbGrid g, const int32_t *__restrict__ q, const int64_t *__restrict__ qoff,
                                    int64_t n, int32_t cumulative, int64_t *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t b = batch_of(qoff, g.num_grids, i);
    const int32_t x = q[3 * i], y = q[3 * i + 1], z = q[3 * i + 2];
    int64_t idx = -1;
    const int32_t id = find_leaf(g, b, x >> 3, y >> 3, z >> 3);
    if (id >= 0) idx = leaf_voxel_index(g.leaves[id], leaf_bit(x, y, z));
    if (idx >= 0 && !cumulative) idx -= g.voxel_offsets[b];
    out[i] = idx;
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_ijk_to_index(const FvgbGrid *grid, const int32_t *ijk, const int64_t *joffsets, int64_t n,
                                 int32_t cumulative, int64_t *out, fvgb_stream_t stream) {
    if (!grid || n < 0 || !joffsets || (n > 0 && (!ijk || !out))) return FVGB_EINVAL;
    if (n == 0) return FVGB_OK;
    ijk_to_index_kernel<<<blocks_for(n), kThreads, 0, as_stream(stream)>>>(*grid, ijk, joffsets, n, cumulative, out);
    count_launches(1);
    return launch_status();
}

// ---------------------------------------------------------------------------------------------
// Coarse grid of floor(ijk / f) built leaf by leaf, for power-of-two factors f <= 8 per axis: a
// fine leaf (8^3 voxels) falls inside one coarse leaf, so the fine leaves are grouped by coarse
// leaf (a radix sort of one key per fine leaf, not per voxel), each coarse leaf's occupancy mask
// is the OR of its fine leaves' voxels mapped down, and the coarse voxels are written leaf by
// leaf in bit order.  Coarse leaves sorted by (grid, order key) and voxels by bit within a leaf
// is the NanoVDB index order: the result is identical to sorting floor(ijk / f) voxel by voxel.
namespace fvgb {
namespace {

constexpr int kCoarseMaxGrids = 1024;  // the grid index takes the key's top 10 bits

struct CoarseWs {
    uint64_t *keys_a, *keys_b, *cmask;
    int32_t *vals_a, *vals_b, *cid, *count, *base;
    int4 *corig;
    void *cub_tmp;
    size_t cub_bytes;
};

size_t coarse_ws_layout(int64_t nl, CoarseWs *w, char *base) {
    size_t cub_bytes = 0, c = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, c, (uint64_t *)nullptr, (uint64_t *)nullptr, (int32_t *)nullptr,
                                    (int32_t *)nullptr, (int)nl, 0, 64);
    cub_bytes = c;
    cub::DeviceRadixSort::SortPairs(nullptr, c, (uint32_t *)nullptr, (uint32_t *)nullptr, (int32_t *)nullptr,
                                    (int32_t *)nullptr, (int)nl, 0, 32);
    if (c > cub_bytes) cub_bytes = c;
    cub::DeviceScan::InclusiveSum(nullptr, c, (int32_t *)nullptr, (int32_t *)nullptr, (int)nl);
    if (c > cub_bytes) cub_bytes = c;
    cub::DeviceScan::ExclusiveSum(nullptr, c, (int32_t *)nullptr, (int32_t *)nullptr, (int)nl + 1);
    if (c > cub_bytes) cub_bytes = c;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    const size_t n = (size_t)nl;
    char *ka = take(n * 8), *kb = take(n * 8), *cm = take(n * 64), *va = take(n * 4), *vb = take(n * 4),
         *ci = take((n + 1) * 4), *co = take((n + 1) * 4), *ba = take((n + 1) * 4), *og = take(n * 16),
         *tmp = take(cub_bytes);
    if (w) {
        w->keys_a = (uint64_t *)ka, w->keys_b = (uint64_t *)kb, w->cmask = (uint64_t *)cm;
        w->vals_a = (int32_t *)va, w->vals_b = (int32_t *)vb, w->cid = (int32_t *)ci, w->count = (int32_t *)co;
        w->base = (int32_t *)ba, w->corig = (int4 *)og, w->cub_tmp = tmp, w->cub_bytes = cub_bytes;
    }
    return off;
}

// key of fine leaf l: (grid << vb) | ((order key of its coarse leaf's origin & low_mask) >> 9); the
// bits above low_mask agree for every coarse voxel of the bounding box, so dropping them keeps the
// order and shortens the sort
__global__ void coarse_keys_kernel(const FvgbLeaf *__restrict__ leaves, int64_t nl, int3 sh, uint64_t low_mask,
                                   int vb, uint64_t *__restrict__ keys, int32_t *__restrict__ vals) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    const FvgbLeaf &lf = leaves[l];
    const int32_t cx = (lf.origin[0] >> (sh.x + 3)) << 3, cy = (lf.origin[1] >> (sh.y + 3)) << 3,
                  cz = (lf.origin[2] >> (sh.z + 3)) << 3;
    keys[l] = ((uint64_t)lf.batch << vb) | ((order_key(cx, cy, cz) & low_mask) >> 9);
    vals[l] = (int32_t)l;
}

template <typename Key>
__global__ void coarse_flags_kernel(const Key *__restrict__ keys, int64_t nl, int32_t *__restrict__ flags) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nl) return;
    flags[p] = (p == 0 || keys[p] != keys[p - 1]) ? 1 : 0;
}

// keys that fit 32 bits, narrowed for a sort with half the traffic and a smaller footprint
__global__ void narrow_keys_kernel(const uint64_t *__restrict__ k64, int64_t nl, uint32_t *__restrict__ k32) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nl) k32[p] = (uint32_t)k64[p];
}

// warp per sorted fine leaf: OR its voxels, mapped down, into its coarse leaf's mask
__global__ void coarse_mask_kernel(const FvgbLeaf *__restrict__ leaves, int64_t nl, int3 sh,
                                   const int32_t *__restrict__ vals, const int32_t *__restrict__ cid,
                                   uint64_t *__restrict__ cmask, int4 *__restrict__ corig) {
    __shared__ unsigned long long wm[8][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t p = (int64_t)blockIdx.x * 8 + warp;
    if (p >= nl) return;  // whole warps leave together
    const FvgbLeaf &lf = leaves[vals[p]];
    const int32_t c = cid[p] - 1;
    if (lane < 8) wm[warp][lane] = 0ull;
    __syncwarp();
    const uint64_t word = lf.mask[lane >> 2];
    const int sub = (lane & 3) * 16;
    for (int i = 0; i < 16; ++i) {
        if (!((word >> (sub + i)) & 1ull)) continue;
        const int b = (lane >> 2) * 64 + sub + i;
        const int32_t gx = lf.origin[0] + (b >> 6), gy = lf.origin[1] + ((b >> 3) & 7), gz = lf.origin[2] + (b & 7);
        const uint32_t cb = leaf_bit(gx >> sh.x, gy >> sh.y, gz >> sh.z);
        atomicOr(&wm[warp][cb >> 6], 1ull << (cb & 63));
    }
    __syncwarp();
    if (lane < 8) {
        const unsigned long long m = wm[warp][lane];
        if (m) atomicOr(reinterpret_cast<unsigned long long *>(cmask) + (int64_t)c * 8 + lane, m);
    }
    if (lane == 0)  // every fine leaf of coarse leaf c writes the same origin
        corig[c] = make_int4((lf.origin[0] >> (sh.x + 3)) << 3, (lf.origin[1] >> (sh.y + 3)) << 3,
                             (lf.origin[2] >> (sh.z + 3)) << 3, lf.batch);
}

// voxels per coarse leaf (zero past the coarse-leaf count, for the exclusive scan over nl + 1)
__global__ void coarse_count_kernel(const uint64_t *__restrict__ cmask, const int32_t *__restrict__ cid, int64_t nl,
                                    int32_t *__restrict__ count) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > nl) return;
    const int64_t lc = cid[nl - 1];
    int32_t n = 0;
    if (c < lc)
#pragma unroll
        for (int w = 0; w < 8; ++w) n += __popcll(cmask[c * 8 + w]);
    count[c] = n;
}

// warp per coarse leaf: its voxels in bit order, and their leaf ids (1-based)
__global__ void coarse_emit_kernel(const uint64_t *__restrict__ cmask, const int4 *__restrict__ corig,
                                   const int32_t *__restrict__ cid, const int32_t *__restrict__ base, int64_t nl,
                                   int32_t *__restrict__ out_ijk, int32_t *__restrict__ leaf_ids) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = (int64_t)blockIdx.x * 8 + warp;
    if (c >= nl || c >= cid[nl - 1]) return;
    const int w = lane >> 2, sub = (lane & 3) * 16;
    int32_t rank = base[c];
    for (int v = 0; v < w; ++v) rank += __popcll(cmask[c * 8 + v]);
    const uint64_t word = cmask[c * 8 + w];
    rank += __popcll(sub ? (word & ((1ull << sub) - 1ull)) : 0ull);
    const int4 o = corig[c];
    for (int i = 0; i < 16; ++i) {
        if (!((word >> (sub + i)) & 1ull)) continue;
        const int b = w * 64 + sub + i;
        out_ijk[3 * (int64_t)rank] = o.x + (b >> 6);
        out_ijk[3 * (int64_t)rank + 1] = o.y + ((b >> 3) & 7);
        out_ijk[3 * (int64_t)rank + 2] = o.z + (b & 7);
        leaf_ids[rank] = (int32_t)c + 1;
        ++rank;
    }
}

// meta[b] = first voxel of grid b (b <= B), meta[B+1] = coarse leaves, meta[B+2] = voxels
__global__ void coarse_offsets_kernel(const int4 *__restrict__ corig, const int32_t *__restrict__ cid,
                                      const int32_t *__restrict__ base, int64_t nl, int32_t B,
                                      int64_t *__restrict__ meta) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > B) return;
    const int64_t lc = cid[nl - 1];
    int64_t lo = 0, hi = lc;  // first coarse leaf with grid >= b
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (corig[mid].w < b) lo = mid + 1; else hi = mid;
    }
    meta[b] = base[lo];
    if (b == 0) {
        meta[B + 1] = lc;
        meta[B + 2] = base[lc];
    }
}

}  // namespace
}  // namespace fvgb

extern "C" int fvgb_coarse_grid_workspace(int64_t num_fine_leaves, size_t *bytes) {
    if (!bytes || num_fine_leaves < 0 || num_fine_leaves >= INT32_MAX) return FVGB_EINVAL;
    *bytes = fvgb::coarse_ws_layout(std::max<int64_t>(num_fine_leaves, 1), nullptr, nullptr) + 256;
    return FVGB_OK;
}

extern "C" int fvgb_coarse_grid_build(const FvgbGrid *fine, const int32_t factor[3], const int32_t *box_lo,
                                      const int32_t *box_hi, int32_t *out_ijk, int64_t *meta, int32_t *leaf_ids,
                                      void *workspace, size_t workspace_bytes, fvgb_stream_t stream) {
    if (!fine || !factor || !meta) return FVGB_EINVAL;
    if (fine->num_grids < 1 || fine->num_grids > kCoarseMaxGrids) return FVGB_EINVAL;
    int sh[3];
    for (int a = 0; a < 3; ++a) {
        const int f = factor[a];
        if (f != 1 && f != 2 && f != 4 && f != 8) return FVGB_EINVAL;
        sh[a] = f == 1 ? 0 : (f == 2 ? 1 : (f == 4 ? 2 : 3));
    }
    const int64_t nl = fine->num_leaves;
    if (nl == 0) return FVGB_EINVAL;  // callers handle empty grids themselves
    if (!out_ijk || !leaf_ids || !fine->leaves) return FVGB_EINVAL;
    size_t need = 0;
    int st = fvgb_coarse_grid_workspace(nl, &need);
    if (st) return st;
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    cudaStream_t s = as_stream(stream);
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    CoarseWs w;
    coarse_ws_layout(nl, &w, base);
    const int3 shv = make_int3(sh[0], sh[1], sh[2]);
    // key bits: the order-key bits that vary inside the coarse bounding box (all 63 without one),
    // less the 9 leaf bits, under the grid index
    int end_bit = 63;
    if (box_lo && box_hi) {
        for (int a = 0; a < 3; ++a)
            if (box_lo[a] > box_hi[a]) return FVGB_EINVAL;
        end_bit = order_key_end_bit(box_lo, box_hi);
    }
    const int vb = end_bit > 9 ? end_bit - 9 : 0;
    const uint64_t low_mask = end_bit >= 63 ? ~0ull : ((1ull << end_bit) - 1ull);
    int grid_bits = 0;
    while ((1 << grid_bits) < fine->num_grids) ++grid_bits;
    const int sort_bits = std::max(1, vb + grid_bits);
    if (cudaMemsetAsync(w.cmask, 0, (size_t)nl * 64, s) != cudaSuccess) return launch_status();
    coarse_keys_kernel<<<blocks_for(nl), kThreads, 0, s>>>(fine->leaves, nl, shv, low_mask, vb, w.keys_a, w.vals_a);
    size_t tb = w.cub_bytes;
    int launched = 6;  // keys, flags, mask, count, emit, offsets (+ narrow)
    if (sort_bits <= 32) {
        // 32-bit keys: the sort's kernels need less shared memory, so they also fit on SMs that a
        // running convolution kernel occupies
        uint32_t *k32a = reinterpret_cast<uint32_t *>(w.keys_b);  // the narrowed keys
        uint32_t *k32b = reinterpret_cast<uint32_t *>(w.keys_a);  // sorted: keys_a is free once narrowed
        narrow_keys_kernel<<<blocks_for(nl), kThreads, 0, s>>>(w.keys_a, nl, k32a);
        cub::DeviceRadixSort::SortPairs(w.cub_tmp, tb, k32a, k32b, w.vals_a, w.vals_b, (int)nl, 0, sort_bits, s);
        coarse_flags_kernel<uint32_t><<<blocks_for(nl), kThreads, 0, s>>>(k32b, nl, w.count);
        ++launched;
    } else {
        cub::DeviceRadixSort::SortPairs(w.cub_tmp, tb, w.keys_a, w.keys_b, w.vals_a, w.vals_b, (int)nl, 0, sort_bits,
                                        s);
        coarse_flags_kernel<uint64_t><<<blocks_for(nl), kThreads, 0, s>>>(w.keys_b, nl, w.count);
    }
    tb = w.cub_bytes;
    cub::DeviceScan::InclusiveSum(w.cub_tmp, tb, w.count, w.cid, (int)nl, s);
    coarse_mask_kernel<<<(unsigned)ceil_div(nl, 8), 256, 0, s>>>(fine->leaves, nl, shv, w.vals_b, w.cid, w.cmask,
                                                                w.corig);
    coarse_count_kernel<<<blocks_for(nl + 1), kThreads, 0, s>>>(w.cmask, w.cid, nl, w.count);
    tb = w.cub_bytes;
    cub::DeviceScan::ExclusiveSum(w.cub_tmp, tb, w.count, w.base, (int)nl + 1, s);
    coarse_emit_kernel<<<(unsigned)ceil_div(nl, 8), 256, 0, s>>>(w.cmask, w.corig, w.cid, w.base, nl, out_ijk,
                                                                leaf_ids);
    coarse_offsets_kernel<<<(unsigned)ceil_div(fine->num_grids + 1, kThreads), kThreads, 0, s>>>(
        w.corig, w.cid, w.base, nl, fine->num_grids, meta);
    count_launches(launched);  // CUB's own launches are not counted
    return launch_status();
}
