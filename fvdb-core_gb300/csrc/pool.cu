// Pooling between a fine and a coarse grid and nearest-neighbour upsampling (the neighbours of
// sparse convolutions in a sparse UNet: fvdb.nn.MaxPool / AvgPool / UpsamplingNearest).
//
// Semantics follow the reference kernels:
//   * pooling: coarse voxel c reads the window of fine voxels c*stride + (i, j, k), i < p0, j < p1,
//     k < p2 (axis a of the window <-> ijk axis a), visited i-outer / k-inner; max starts at -inf
//     (an empty window stays -inf), average = (sum of the window's active voxels in the
//     accumulation type, rounded to the data type) * (1 / (p0 p1 p2) rounded to the data type)
//     (src/fvdb/detail/ops/DownsampleGridMaxPool.cu:19-69, DownsampleGridAvgPool.cu:19-64,144);
//   * max-pool gradient: each window's gradient goes to its first strict maximum;
//     average gradient: fine voxel f gets grad(c) * (1 / (p0 p1 p2)) from the window c holding it
//     (DownsampleGridMaxPool.cu:71-126, DownsampleGridAvgPool.cu:68-112);
//   * upsampling: fine voxel f copies coarse voxel floor(f / factor); its gradient sums the
//     children (src/fvdb/detail/ops/UpsampleGridNearest.cu:19-110).
// Differences, each on inputs where the reference's result is undefined or racy: the coarse
// coordinate of upsampling is an exact integer floor (the reference divides in the data type,
// inexact for 16-bit data beyond |ijk| = 256), a fine voxel without a coarse parent reads zero
// (the reference reads the row before its grid's first), and gradients of overlapping windows
// (stride < pool factor) add up (the reference's concurrent assignments keep one of them).
//
// Lookups go through the grids' leaf hash; one warp per output voxel gathers the window's
// indices (lanes over window positions) into shared memory and then reduces channels (lanes over
// channels, coalesced rows).  All of these kernels are bound by HBM and hash-probe latency.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace fvgb {
namespace {

constexpr int kPoolWarps = 8;
constexpr int kMaxWindow = 512;  // pool factor / upsampling factor volume (8x8x8)

__device__ __forceinline__ int64_t voxel_at(const FvgbGrid &g, int32_t b, int32_t x, int32_t y, int32_t z) {
    const int32_t lid = find_leaf(g, b, x >> 3, y >> 3, z >> 3);
    if (lid < 0) return -1;
    return leaf_voxel_index(g.leaves[lid], leaf_bit(x, y, z));
}

template <typename T>
struct Num;
template <>
struct Num<float> {
    using Acc = float;
    __device__ static float to(float v) { return v; }
    __device__ static float from(float v) { return v; }
};
template <>
struct Num<double> {
    using Acc = double;
    __device__ static double to(double v) { return v; }
    __device__ static double from(double v) { return v; }
};
template <>
struct Num<__half> {
    using Acc = float;
    __device__ static float to(__half v) { return __half2float(v); }
    __device__ static __half from(float v) { return __float2half_rn(v); }
};
template <>
struct Num<__nv_bfloat16> {
    using Acc = float;
    __device__ static float to(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static __nv_bfloat16 from(float v) { return __float2bfloat16_rn(v); }
};

// x * y in the data type's arithmetic: both rounded to T, multiplied in the accumulation type,
// the product rounded to T (c10::Half / BFloat16 multiply through float).
template <typename T>
__device__ __forceinline__ T mul_in(T a, double b) {
    using A = typename Num<T>::Acc;
    return Num<T>::from(Num<T>::to(a) * Num<T>::to(Num<T>::from((A)b)));
}

// Window indices of one output voxel into the warp's shared array (window order i-outer,
// k-inner); returns nothing, lanes fill positions lane, lane+32, ...
__device__ __forceinline__ void window_indices(const FvgbGrid &g, int32_t b, int3 base, int3 ext, int32_t *idx,
                                               int lane) {
    const int W = ext.x * ext.y * ext.z;
    for (int w = lane; w < W; w += 32) {
        const int i = w / (ext.y * ext.z), j = (w / ext.z) % ext.y, k = w % ext.z;
        const int64_t v = voxel_at(g, b, base.x + i, base.y + j, base.z + k);
        idx[w] = (int32_t)v;
    }
    __syncwarp();
}

template <typename T, bool MAX>
__global__ void __launch_bounds__(kPoolWarps * 32) pool_fwd_kernel(FvgbGrid fine, FvgbGrid coarse, int3 pf, int3 st,
                                                                   const T *__restrict__ x, int64_t ldx, int32_t C,
                                                                   T *__restrict__ y, int64_t ldy, double avg) {
    using A = typename Num<T>::Acc;
    __shared__ int32_t widx[kPoolWarps][kMaxWindow];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = pf.x * pf.y * pf.z;
    for (int64_t c = (int64_t)blockIdx.x * kPoolWarps + warp; c < coarse.num_voxels;
         c += (int64_t)gridDim.x * kPoolWarps) {
        const int32_t b = batch_of(coarse.voxel_offsets, coarse.num_grids, c);
        const int3 base = make_int3(coarse.ijk[3 * c] * st.x, coarse.ijk[3 * c + 1] * st.y, coarse.ijk[3 * c + 2] * st.z);
        window_indices(fine, b, base, pf, widx[warp], lane);
        for (int ch = lane; ch < C; ch += 32) {
            A acc = MAX ? (A)(-INFINITY) : (A)0;
            for (int w = 0; w < W; ++w) {
                const int32_t f = widx[warp][w];
                if (f < 0) continue;
                const A v = Num<T>::to(x[(int64_t)f * ldx + ch]);
                acc = MAX ? (A)fmax((double)v, (double)acc) : acc + v;
            }
            y[c * ldy + ch] = MAX ? Num<T>::from(acc) : mul_in<T>(Num<T>::from(acc), avg);
        }
        __syncwarp();
    }
}

// Max-pool gradient: per window and channel, grad to the first strict maximum, added into the
// accumulation buffer dx (zero-initialised by the caller).
template <typename T>
__global__ void __launch_bounds__(kPoolWarps * 32) maxpool_bwd_kernel(FvgbGrid fine, FvgbGrid coarse, int3 pf, int3 st,
                                                                      const T *__restrict__ x, int64_t ldx, int32_t C,
                                                                      const T *__restrict__ dy, int64_t lddy,
                                                                      typename Num<T>::Acc *__restrict__ dx) {
    using A = typename Num<T>::Acc;
    __shared__ int32_t widx[kPoolWarps][kMaxWindow];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = pf.x * pf.y * pf.z;
    for (int64_t c = (int64_t)blockIdx.x * kPoolWarps + warp; c < coarse.num_voxels;
         c += (int64_t)gridDim.x * kPoolWarps) {
        const int32_t b = batch_of(coarse.voxel_offsets, coarse.num_grids, c);
        const int3 base = make_int3(coarse.ijk[3 * c] * st.x, coarse.ijk[3 * c + 1] * st.y, coarse.ijk[3 * c + 2] * st.z);
        window_indices(fine, b, base, pf, widx[warp], lane);
        for (int ch = lane; ch < C; ch += 32) {
            A best = (A)(-INFINITY);
            int32_t arg = -1;
            for (int w = 0; w < W; ++w) {
                const int32_t f = widx[warp][w];
                if (f < 0) continue;
                const A v = Num<T>::to(x[(int64_t)f * ldx + ch]);
                if (v > best) {
                    best = v;
                    arg = f;
                }
            }
            if (arg >= 0) atomicAdd(dx + (int64_t)arg * C + ch, Num<T>::to(dy[c * lddy + ch]));
        }
        __syncwarp();
    }
}

// Average-pool gradient, gathered per fine voxel: the coarse voxels whose window holds fine
// voxel f are c with c*s <= f < c*s + p per axis.
template <typename T>
__global__ void __launch_bounds__(kPoolWarps * 32) avgpool_bwd_kernel(FvgbGrid fine, FvgbGrid coarse, int3 pf, int3 st,
                                                                      int32_t C, const T *__restrict__ dy,
                                                                      int64_t lddy, T *__restrict__ dx, int64_t lddx,
                                                                      double avg) {
    using A = typename Num<T>::Acc;
    __shared__ int32_t widx[kPoolWarps][kMaxWindow];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto fdiv = [](int32_t a, int32_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
    for (int64_t f = (int64_t)blockIdx.x * kPoolWarps + warp; f < fine.num_voxels; f += (int64_t)gridDim.x * kPoolWarps) {
        const int32_t b = batch_of(fine.voxel_offsets, fine.num_grids, f);
        const int32_t fx = fine.ijk[3 * f], fy = fine.ijk[3 * f + 1], fz = fine.ijk[3 * f + 2];
        // candidate coarse range per axis: [ceil((f - p + 1) / s), floor(f / s)]
        const int3 lo = make_int3(-fdiv(-(fx - pf.x + 1), st.x), -fdiv(-(fy - pf.y + 1), st.y), -fdiv(-(fz - pf.z + 1), st.z));
        const int3 hi = make_int3(fdiv(fx, st.x), fdiv(fy, st.y), fdiv(fz, st.z));
        const int3 ext = make_int3(max(hi.x - lo.x + 1, 0), max(hi.y - lo.y + 1, 0), max(hi.z - lo.z + 1, 0));
        const int W = ext.x * ext.y * ext.z;  // <= p0 p1 p2
        window_indices(coarse, b, lo, ext, widx[warp], lane);
        for (int ch = lane; ch < C; ch += 32) {
            bool any = false;
            A acc = (A)0;
            for (int w = 0; w < W; ++w) {
                const int32_t c = widx[warp][w];
                if (c < 0) continue;
                const T g = mul_in<T>(dy[(int64_t)c * lddy + ch], avg);
                acc = any ? acc + Num<T>::to(g) : Num<T>::to(g);
                any = true;
            }
            dx[f * lddx + ch] = Num<T>::from(acc);
        }
        __syncwarp();
    }
}

// Nearest upsampling: fine voxel f copies coarse voxel floor(f / factor) (zero without one).
template <typename T>
__global__ void __launch_bounds__(kPoolWarps * 32) upsample_fwd_kernel(FvgbGrid coarse, FvgbGrid fine, int3 fac,
                                                                       const T *__restrict__ x, int64_t ldx, int32_t C,
                                                                       T *__restrict__ y, int64_t ldy) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto fdiv = [](int32_t a, int32_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
    for (int64_t f = (int64_t)blockIdx.x * kPoolWarps + warp; f < fine.num_voxels; f += (int64_t)gridDim.x * kPoolWarps) {
        int64_t c = -1;
        if (lane == 0) {
            const int32_t b = batch_of(fine.voxel_offsets, fine.num_grids, f);
            c = voxel_at(coarse, b, fdiv(fine.ijk[3 * f], fac.x), fdiv(fine.ijk[3 * f + 1], fac.y),
                         fdiv(fine.ijk[3 * f + 2], fac.z));
        }
        c = __shfl_sync(0xffffffffu, c, 0);
        for (int ch = lane; ch < C; ch += 32)
            y[f * ldy + ch] = c >= 0 ? x[c * ldx + ch] : Num<T>::from(0.0f);
    }
}

// Upsampling gradient: coarse voxel c sums its children c*factor + (i, j, k) (window order).
template <typename T>
__global__ void __launch_bounds__(kPoolWarps * 32) upsample_bwd_kernel(FvgbGrid coarse, FvgbGrid fine, int3 fac,
                                                                       const T *__restrict__ dy, int64_t lddy, int32_t C,
                                                                       T *__restrict__ dx, int64_t lddx) {
    using A = typename Num<T>::Acc;
    __shared__ int32_t widx[kPoolWarps][kMaxWindow];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = fac.x * fac.y * fac.z;
    for (int64_t c = (int64_t)blockIdx.x * kPoolWarps + warp; c < coarse.num_voxels;
         c += (int64_t)gridDim.x * kPoolWarps) {
        const int32_t b = batch_of(coarse.voxel_offsets, coarse.num_grids, c);
        const int3 base = make_int3(coarse.ijk[3 * c] * fac.x, coarse.ijk[3 * c + 1] * fac.y, coarse.ijk[3 * c + 2] * fac.z);
        window_indices(fine, b, base, fac, widx[warp], lane);
        for (int ch = lane; ch < C; ch += 32) {
            A acc = (A)0;
            for (int w = 0; w < W; ++w) {
                const int32_t f = widx[warp][w];
                if (f >= 0) acc += Num<T>::to(dy[(int64_t)f * lddy + ch]);
            }
            dx[c * lddx + ch] = Num<T>::from(acc);
        }
        __syncwarp();
    }
}

// Candidates of the subdivided grid: coarse voxel c (where mask[c] != 0, or every voxel without a
// mask) yields c*factor + (i, j, k); out_valid marks the kept ones.
__global__ void subdivide_candidates_kernel(FvgbGrid coarse, int3 fac, const uint8_t *__restrict__ mask,
                                            int32_t *__restrict__ out, uint8_t *__restrict__ valid) {
    const int W = fac.x * fac.y * fac.z;
    const int64_t total = coarse.num_voxels * W;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / W;
        const int w = (int)(e % W);
        const int i = w / (fac.y * fac.z), j = (w / fac.z) % fac.y, k = w % fac.z;
        out[3 * e] = coarse.ijk[3 * c] * fac.x + i;
        out[3 * e + 1] = coarse.ijk[3 * c + 1] * fac.y + j;
        out[3 * e + 2] = coarse.ijk[3 * c + 2] * fac.z + k;
        valid[e] = mask ? (uint8_t)(mask[c] != 0) : (uint8_t)1;
    }
}

unsigned pool_blocks(int64_t items) {
    const int64_t b = ceil_div(items, kPoolWarps);
    return (unsigned)std::min<int64_t>(std::max<int64_t>(b, 1), 65535 * 16);
}

bool vec_ok(const int32_t *v, int max_volume) {
    if (!v || v[0] < 1 || v[1] < 1 || v[2] < 1) return false;
    return (int64_t)v[0] * v[1] * v[2] <= max_volume;
}

template <template <typename> class F, typename... Args>
int dispatch_dtype(int32_t dtype, Args &&...args) {
    switch (dtype) {
        case FVGB_F32: F<float>::run(args...); break;
        case FVGB_F64: F<double>::run(args...); break;
        case FVGB_F16: F<__half>::run(args...); break;
        case FVGB_BF16: F<__nv_bfloat16>::run(args...); break;
        default: return FVGB_ETYPE;
    }
    count_launches(1);
    return launch_status();
}

template <typename T>
struct PoolFwd {
    static void run(int mode, const FvgbGrid &f, const FvgbGrid &c, int3 pf, int3 st, const void *x, int64_t ldx,
                    int32_t C, void *y, int64_t ldy, cudaStream_t s) {
        const double avg = 1.0 / ((double)pf.x * pf.y * pf.z);
        if (mode == FVGB_POOL_MAX)
            pool_fwd_kernel<T, true><<<pool_blocks(c.num_voxels), kPoolWarps * 32, 0, s>>>(
                f, c, pf, st, (const T *)x, ldx, C, (T *)y, ldy, avg);
        else
            pool_fwd_kernel<T, false><<<pool_blocks(c.num_voxels), kPoolWarps * 32, 0, s>>>(
                f, c, pf, st, (const T *)x, ldx, C, (T *)y, ldy, avg);
    }
};
template <typename T>
struct MaxPoolBwd {
    static void run(const FvgbGrid &f, const FvgbGrid &c, int3 pf, int3 st, const void *x, int64_t ldx, int32_t C,
                    const void *dy, int64_t lddy, void *dx_acc, cudaStream_t s) {
        maxpool_bwd_kernel<T><<<pool_blocks(c.num_voxels), kPoolWarps * 32, 0, s>>>(
            f, c, pf, st, (const T *)x, ldx, C, (const T *)dy, lddy, (typename Num<T>::Acc *)dx_acc);
    }
};
template <typename T>
struct AvgPoolBwd {
    static void run(const FvgbGrid &f, const FvgbGrid &c, int3 pf, int3 st, int32_t C, const void *dy, int64_t lddy,
                    void *dx, int64_t lddx, cudaStream_t s) {
        const double avg = 1.0 / ((double)pf.x * pf.y * pf.z);
        avgpool_bwd_kernel<T><<<pool_blocks(f.num_voxels), kPoolWarps * 32, 0, s>>>(f, c, pf, st, C, (const T *)dy,
                                                                                      lddy, (T *)dx, lddx, avg);
    }
};
template <typename T>
struct UpFwd {
    static void run(const FvgbGrid &c, const FvgbGrid &f, int3 fac, const void *x, int64_t ldx, int32_t C, void *y,
                    int64_t ldy, cudaStream_t s) {
        upsample_fwd_kernel<T><<<pool_blocks(f.num_voxels), kPoolWarps * 32, 0, s>>>(c, f, fac, (const T *)x, ldx, C,
                                                                                      (T *)y, ldy);
    }
};
template <typename T>
struct UpBwd {
    static void run(const FvgbGrid &c, const FvgbGrid &f, int3 fac, const void *dy, int64_t lddy, int32_t C, void *dx,
                    int64_t lddx, cudaStream_t s) {
        upsample_bwd_kernel<T><<<pool_blocks(c.num_voxels), kPoolWarps * 32, 0, s>>>(c, f, fac, (const T *)dy, lddy, C,
                                                                                      (T *)dx, lddx);
    }
};

bool grids_ok(const FvgbGrid *a, const FvgbGrid *b) {
    return a && b && a->num_grids == b->num_grids && a->num_voxels >= 0 && b->num_voxels >= 0;
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_pool_forward(int32_t mode, int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse,
                                 const int32_t pool[3], const int32_t stride[3], const void *x, int64_t ldx,
                                 int32_t C, void *y, int64_t ldy, fvgb_stream_t stream) {
    if ((mode != FVGB_POOL_MAX && mode != FVGB_POOL_AVG) || !grids_ok(fine, coarse) || !vec_ok(pool, kMaxWindow) ||
        !vec_ok(stride, 1 << 30) || C < 1 || ldx < C || ldy < C)
        return FVGB_EINVAL;
    if (coarse->num_voxels == 0) return FVGB_OK;
    if (!y || (fine->num_voxels > 0 && !x)) return FVGB_EINVAL;
    return dispatch_dtype<PoolFwd>(dtype, mode, *fine, *coarse, make_int3(pool[0], pool[1], pool[2]),
                                   make_int3(stride[0], stride[1], stride[2]), x, ldx, C, y, ldy, as_stream(stream));
}

extern "C" int fvgb_maxpool_backward(int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse, const int32_t pool[3],
                                     const int32_t stride[3], const void *x, int64_t ldx, int32_t C, const void *dy,
                                     int64_t lddy, void *dx_acc, fvgb_stream_t stream) {
    if (!grids_ok(fine, coarse) || !vec_ok(pool, kMaxWindow) || !vec_ok(stride, 1 << 30) || C < 1 || ldx < C ||
        lddy < C)
        return FVGB_EINVAL;
    if (coarse->num_voxels == 0 || fine->num_voxels == 0) return FVGB_OK;
    if (!x || !dy || !dx_acc) return FVGB_EINVAL;
    return dispatch_dtype<MaxPoolBwd>(dtype, *fine, *coarse, make_int3(pool[0], pool[1], pool[2]),
                                      make_int3(stride[0], stride[1], stride[2]), x, ldx, C, dy, lddy, dx_acc,
                                      as_stream(stream));
}

extern "C" int fvgb_avgpool_backward(int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse, const int32_t pool[3],
                                     const int32_t stride[3], int32_t C, const void *dy, int64_t lddy, void *dx,
                                     int64_t lddx, fvgb_stream_t stream) {
    if (!grids_ok(fine, coarse) || !vec_ok(pool, kMaxWindow) || !vec_ok(stride, 1 << 30) || C < 1 || lddy < C ||
        lddx < C)
        return FVGB_EINVAL;
    if (fine->num_voxels == 0) return FVGB_OK;
    if (!dx || (coarse->num_voxels > 0 && !dy)) return FVGB_EINVAL;
    return dispatch_dtype<AvgPoolBwd>(dtype, *fine, *coarse, make_int3(pool[0], pool[1], pool[2]),
                                      make_int3(stride[0], stride[1], stride[2]), C, dy, lddy, dx, lddx,
                                      as_stream(stream));
}

extern "C" int fvgb_upsample_forward(int32_t dtype, const FvgbGrid *coarse, const FvgbGrid *fine, const int32_t factor[3],
                                     const void *x, int64_t ldx, int32_t C, void *y, int64_t ldy,
                                     fvgb_stream_t stream) {
    if (!grids_ok(fine, coarse) || !vec_ok(factor, kMaxWindow) || C < 1 || ldx < C || ldy < C) return FVGB_EINVAL;
    if (fine->num_voxels == 0) return FVGB_OK;
    if (!y || (coarse->num_voxels > 0 && !x)) return FVGB_EINVAL;
    return dispatch_dtype<UpFwd>(dtype, *coarse, *fine, make_int3(factor[0], factor[1], factor[2]), x, ldx, C, y, ldy,
                                 as_stream(stream));
}

extern "C" int fvgb_upsample_backward(int32_t dtype, const FvgbGrid *coarse, const FvgbGrid *fine,
                                      const int32_t factor[3], const void *dy, int64_t lddy, int32_t C, void *dx,
                                      int64_t lddx, fvgb_stream_t stream) {
    if (!grids_ok(fine, coarse) || !vec_ok(factor, kMaxWindow) || C < 1 || lddy < C || lddx < C) return FVGB_EINVAL;
    if (coarse->num_voxels == 0) return FVGB_OK;
    if (!dx || (fine->num_voxels > 0 && !dy)) return FVGB_EINVAL;
    return dispatch_dtype<UpBwd>(dtype, *coarse, *fine, make_int3(factor[0], factor[1], factor[2]), dy, lddy, C, dx,
                                 lddx, as_stream(stream));
}

extern "C" int fvgb_subdivide_candidates(const FvgbGrid *coarse, const int32_t factor[3], const uint8_t *mask,
                                         int32_t *out_ijk, uint8_t *out_valid, fvgb_stream_t stream) {
    if (!coarse || !vec_ok(factor, kMaxWindow)) return FVGB_EINVAL;
    const int64_t total = coarse->num_voxels * factor[0] * factor[1] * factor[2];
    if (total == 0) return FVGB_OK;
    if (!out_ijk || !out_valid) return FVGB_EINVAL;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(total, 256), 65535 * 16);
    subdivide_candidates_kernel<<<blocks, 256, 0, as_stream(stream)>>>(*coarse, make_int3(factor[0], factor[1], factor[2]),
                                                                      mask, out_ijk, out_valid);
    count_launches(1);
    return launch_status();
}
