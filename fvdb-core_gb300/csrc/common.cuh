// Shared helpers of libfvdb_gb300: status plumbing, the voxel-order key, leaf lookup.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <utility>

#include "../../include/fvdb_gb300.h"

namespace fvgb {

// Records the CUDA error (if any) for fvgb_last_error and maps it to a status code.
int record_cuda(cudaError_t e);
// Records a library error message for fvgb_last_error (host).
void record_message(const char *msg);
// Status of the last launch on this thread.
inline int launch_status() { return record_cuda(cudaGetLastError()); }
// Adds n to the process-wide count of kernels launched by this library (CUB's
// library kernels are not counted).
void count_launches(int n);

inline cudaStream_t as_stream(fvgb_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }
// Streaming multiprocessors of the current device (cached per device).
int device_sm_count();

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device) and size: the
// attribute persists, and setting it before every launch costs host time on the launch path.
template <typename F>
inline cudaError_t set_dynamic_smem(F kern, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    const auto key = std::make_pair(reinterpret_cast<const void *>(kern), dev);
    std::lock_guard<std::mutex> lock(mu);
    auto it = done.find(key);
    if (it != done.end() && it->second >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done[key] = bytes;
    return e;
}

constexpr int kLeafDim = 8;
// find_leaf reads (origin, batch) of a leaf as one 16-byte load: leaves must stay 128 bytes.
static_assert(sizeof(FvgbLeaf) == 128, "FvgbLeaf must be exactly 128 bytes");

// ---------------------------------------------------------------------------------------
// Voxel order key.  NanoVDB numbers the voxels of an OnIndex tree depth-first: root tiles
// (4096^3) by root key, then the upper-node child (x,y,z bits 11..7), lower-node child
// (bits 6..3), leaf voxel (bits 2..0).  The CUDA builder's root key sorts
// (uint32(c) >> 12) per axis as unsigned, i.e. non-negative tiles before negative ones.
// With coordinates limited to [-2^20, 2^20) the tile index fits 9 bits per axis and the
// whole order packs into 63 bits:
//   [rx:9][ry:9][rz:9][upper:15][lower:12][leaf:9]
// (rx = (x >> 12) & 511 keeps the unsigned tile order: 0..255 then -256..-1).
// ---------------------------------------------------------------------------------------
__host__ __device__ inline bool coord_in_range(int32_t c) {
    return c >= -FVGB_COORD_LIMIT && c < FVGB_COORD_LIMIT;
}

__host__ __device__ inline uint64_t order_key(int32_t x, int32_t y, int32_t z) {
    const uint64_t rx = (uint64_t)((x >> 12) & 511), ry = (uint64_t)((y >> 12) & 511),
                   rz = (uint64_t)((z >> 12) & 511);
    const uint64_t up = ((uint64_t)((x >> 7) & 31) << 10) | ((uint64_t)((y >> 7) & 31) << 5) |
                        (uint64_t)((z >> 7) & 31);
    const uint64_t lw = ((uint64_t)((x >> 3) & 15) << 8) | ((uint64_t)((y >> 3) & 15) << 4) |
                        (uint64_t)((z >> 3) & 15);
    const uint64_t lf = ((uint64_t)(x & 7) << 6) | ((uint64_t)(y & 7) << 3) | (uint64_t)(z & 7);
    return (rx << 54) | (ry << 45) | (rz << 36) | (up << 21) | (lw << 9) | lf;
}

__host__ __device__ inline int32_t sext9(uint64_t v) { return (int32_t)((v ^ 256u) & 511u) - 256; }

__host__ __device__ inline void key_to_coord(uint64_t k, int32_t &x, int32_t &y, int32_t &z) {
    const int32_t rx = sext9(k >> 54), ry = sext9(k >> 45), rz = sext9(k >> 36);
    const uint32_t up = (uint32_t)((k >> 21) & 0x7fff), lw = (uint32_t)((k >> 9) & 0xfff),
                   lf = (uint32_t)(k & 0x1ff);
    x = (int32_t)((uint32_t)rx << 12 | ((up >> 10) & 31) << 7 | ((lw >> 8) & 15) << 3 | ((lf >> 6) & 7));
    y = (int32_t)((uint32_t)ry << 12 | ((up >> 5) & 31) << 7 | ((lw >> 4) & 15) << 3 | ((lf >> 3) & 7));
    z = (int32_t)((uint32_t)rz << 12 | (up & 31) << 7 | (lw & 15) << 3 | (lf & 7));
}

// Leaf bit of a voxel inside its 8^3 leaf (x-major, as NanoVDB LeafNode::CoordToOffset).
__host__ __device__ inline uint32_t leaf_bit(int32_t x, int32_t y, int32_t z) {
    return ((uint32_t)(x & 7) << 6) | ((uint32_t)(y & 7) << 3) | (uint32_t)(z & 7);
}

// Hash of a leaf (batch, leaf coordinates = origin >> 3).
__host__ __device__ inline uint64_t leaf_hash(int32_t b, int32_t lx, int32_t ly, int32_t lz) {
    uint64_t h = (uint64_t)(uint32_t)lx * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)(uint32_t)ly * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
    h ^= (uint64_t)(uint32_t)lz * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
    h ^= (uint64_t)(uint32_t)b * 0x27D4EB2F165667C5ull + (h << 6) + (h >> 2);
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    return h;
}

// Leaf id of (b, lx, ly, lz) in the grid's hash, or -1.  Probes are bounded by the
// capacity, so a full table cannot loop forever.
__device__ inline int32_t find_leaf(const FvgbGrid &g, int32_t b, int32_t lx, int32_t ly, int32_t lz) {
    if (g.hash_capacity == 0) return -1;
    const uint64_t cap_mask = (uint64_t)g.hash_capacity - 1;
    uint64_t h = leaf_hash(b, lx, ly, lz) & cap_mask;
    for (int64_t probe = 0; probe < g.hash_capacity; ++probe) {
        const int32_t id = __ldg(g.hash_slots + h);
        if (id < 0) return -1;
        const int4 o = __ldg(reinterpret_cast<const int4 *>(g.leaves + id));
        if (o.x == lx * 8 && o.y == ly * 8 && o.z == lz * 8 && o.w == b) return id;
        h = (h + 1) & cap_mask;
    }
    return -1;
}

// Global index of an active voxel given its leaf and bit, or -1 when inactive.
__device__ inline int64_t leaf_voxel_index(const FvgbLeaf &leaf, uint32_t bit) {
    const uint32_t w = bit >> 6;
    const uint64_t m = leaf.mask[w];
    const uint64_t below = (bit & 63) ? (m & ((1ull << (bit & 63)) - 1ull)) : 0ull;
    if (!((m >> (bit & 63)) & 1ull)) return -1;
    return leaf.base + leaf.prefix[w] + __popcll(below);
}

// Grid of a global row given the jagged offsets (binary search, B+1 entries).
__device__ inline int32_t batch_of(const int64_t *offsets, int32_t num_grids, int64_t row) {
    int32_t lo = 0, hi = num_grids;  // find largest b with offsets[b] <= row
    while (hi - lo > 1) {
        const int32_t mid = (lo + hi) >> 1;
        if (__ldg(offsets + mid) <= row) lo = mid; else hi = mid;
    }
    return lo;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace fvgb
