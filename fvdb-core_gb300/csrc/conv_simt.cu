// CUDA-core contractions: the plain FP32 form (no TF32) and the FP64 form.
//
// Forward:  y[m,:] (+)= sum_k x[map[m,k],:] . W[k]   (one CTA owns a 128x64 output tile; every
//           output element is written exactly once, no atomics).  Offsets whose 128 map entries
//           are all -1 are skipped.  With the transposed map and W^T strides the same kernel is
//           the data gradient.
// Wgrad:    dW[k,ci,co] = sum_m x[map[m,k],ci] * dy[m,co] with per-CTA partials and a
//           fixed-order FP64 reduction across CTAs.
//
// Replaces the gather -> torch::mm_out -> scatter loop of
// src/fvdb/detail/ops/convolution/backend/SparseConvolutionKernelMap.cu:116-415.
#include "common.cuh"

namespace fvgb {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;  // wgrad tile
constexpr int FM = 128, FN = 64;                    // forward tile: 128 rows x 64 channels, 8 x 4 per thread

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    __device__ static void load(const float *p, float (&v)[4]) {
        const float4 q = *reinterpret_cast<const float4 *>(p);
        v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
    }
};
template <>
struct Vec4<double> {
    __device__ static void load(const double *p, double (&v)[4]) {
        const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
        v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
    }
};

// One CTA per 128-row x 64-channel output tile, 256 threads of 8 rows x 4 channels.  Per
// offset with any present row and per 16-channel slice (8 for FP64), the gathered rows (transposed, so a
// thread's 8 rows are two vector loads) and the weight slice go through shared memory; the
// slice after is loaded into registers while this one is multiplied, so one barrier per slice
// separates the two shared-memory buffers.
template <typename T>
__global__ void __launch_bounds__(NT) conv_fwd_simt_kernel(const T *__restrict__ x, int64_t n_x, int32_t cin,
                                                           int64_t ldx, const int32_t *__restrict__ map,
                                                           int64_t n_out, int32_t K, int64_t ldm,
                                                           const T *__restrict__ w, int64_t wsk, int64_t wsci,
                                                           int64_t wsco, T *__restrict__ y, int32_t cout,
                                                           int64_t ldy, int32_t accumulate,
                                                           const int32_t *__restrict__ out_rows) {
    // map row m (m < n_out) computes output row out_rows[m] (m itself when out_rows is null)
    constexpr int FK = sizeof(T) == 8 ? 8 : 16;  // channels per slice (static shared memory < 48 KB)
    constexpr int QA = FM * FK / NT, QB = FK * FN / NT;
    __shared__ int32_t rows[2][FM];
    __shared__ __align__(16) T As[2][FK][FM + 4];
    __shared__ __align__(16) T Bs[2][FK][FN + 4];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t m0 = (int64_t)blockIdx.x * FM;
    const int32_t n0 = blockIdx.y * FN;
    T acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);

    // rows of offset k into rows[rb]; true if any is present (a CTA-wide vote)
    auto load_rows = [&](int32_t k, int rb) -> bool {
        int valid = 0;
        if (tid < FM) {
            const int64_t r = m0 + tid;
            int32_t v = r < n_out ? map[r * ldm + k] : -1;
            if (v >= n_x) v = -1;
            rows[rb][tid] = v;
            valid = v >= 0;
        }
        return __syncthreads_or(valid) != 0;
    };
    // per thread: A elements e = tid + 256 q (q < QA) -> (row e / FK, channel e % FK); B elements
    // e = tid + 256 q (q < QB) -> (channel e / 64, column e % 64)
    T ra[QA], rb4[QB];
    auto fetch = [&](int32_t k, int32_t c0, int rbuf) {
#pragma unroll
        for (int q = 0; q < QA; ++q) {
            const int e = tid + q * NT, r = e / FK, c = e % FK;
            const int32_t src = rows[rbuf][r];
            ra[q] = (src >= 0 && c0 + c < cin) ? x[(int64_t)src * ldx + c0 + c] : T(0);
        }
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int e = tid + q * NT, c = e >> 6, n = e & 63;
            rb4[q] = (c0 + c < cin && n0 + n < cout)
                         ? w[k * wsk + (int64_t)(c0 + c) * wsci + (int64_t)(n0 + n) * wsco]
                         : T(0);
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < QA; ++q) {
            const int e = tid + q * NT;
            As[buf][e % FK][e / FK] = ra[q];
        }
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int e = tid + q * NT;
            Bs[buf][e >> 6][e & 63] = rb4[q];
        }
    };

    // walk (offset, channel slice) pairs, skipping offsets with no present row
    int32_t k = 0;
    int rbuf = 0;
    while (k < K && !load_rows(k, rbuf)) ++k;
    if (k < K) {
        int32_t c0 = 0;
        fetch(k, c0, rbuf);
        store(0);
        __syncthreads();
        int buf = 0;
        while (true) {
            // the next (offset, slice)
            int32_t kn = k, cn = c0 + FK;
            int rn = rbuf;
            if (cn >= cin) {
                cn = 0;
                rn = rbuf ^ 1;
                ++kn;
                while (kn < K && !load_rows(kn, rn)) ++kn;
            }
            const bool more = kn < K;
            if (more) fetch(kn, cn, rn);
#pragma unroll
            for (int c = 0; c < FK; ++c) {
                T a[8], b[4];
                T a0[4], a1[4];
                Vec4<T>::load(&As[buf][c][ty * 8], a0);
                Vec4<T>::load(&As[buf][c][ty * 8 + 4], a1);
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = a0[i], a[i + 4] = a1[i];
                Vec4<T>::load(&Bs[buf][c][tx * 4], b);
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
            if (!more) break;
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
            k = kn, c0 = cn, rbuf = rn;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int64_t t = m0 + ty * 8 + i;
        if (t >= n_out) continue;
        const int64_t r = out_rows ? (int64_t)out_rows[t] : t;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int32_t n = n0 + tx * 4 + j;
            if (n >= cout) continue;
            T *dst = y + r * ldy + n;
            *dst = accumulate ? (T)(*dst + acc[i][j]) : acc[i][j];
        }
    }
}

// Rows per wgrad chunk so that the grid has enough CTAs; deterministic in the sizes only.
struct WgradPlan {
    int64_t chunks, rows_per_chunk;
    int32_t tiles_ci, tiles_co;
};

WgradPlan wgrad_plan(int64_t n_out, int32_t K, int32_t cin, int32_t cout) {
    WgradPlan p;
    p.tiles_ci = (int32_t)ceil_div(cin, BM);
    p.tiles_co = (int32_t)ceil_div(cout, BN);
    const int64_t per_chunk_ctas = (int64_t)K * p.tiles_ci * p.tiles_co;
    int64_t chunks = ceil_div(2048, per_chunk_ctas);
    const int64_t max_chunks = ceil_div(n_out > 0 ? n_out : 1, 256);
    if (chunks > max_chunks) chunks = max_chunks;
    if (chunks < 1) chunks = 1;
    p.rows_per_chunk = ceil_div(ceil_div(n_out > 0 ? n_out : 1, chunks), BK) * BK;
    p.chunks = ceil_div(n_out > 0 ? n_out : 1, p.rows_per_chunk);
    return p;
}

template <typename T, typename AccT>
__global__ void __launch_bounds__(NT) wgrad_simt_kernel(const T *__restrict__ x, int64_t n_x, int32_t cin,
                                                        int64_t ldx, const int32_t *__restrict__ map,
                                                        int64_t n_out, int32_t K, int64_t ldm,
                                                        const T *__restrict__ dy, int32_t cout, int64_t lddy,
                                                        int64_t rows_per_chunk, int32_t tiles_co,
                                                        AccT *__restrict__ partials) {
    __shared__ int32_t rows[BK];
    __shared__ AccT Xs[BK][BM + 4];
    __shared__ AccT Ds[BK][BN + 4];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t chunk = blockIdx.x;
    const int32_t k = blockIdx.y;
    const int32_t ci0 = (blockIdx.z / tiles_co) * BM, co0 = (blockIdx.z % tiles_co) * BN;
    const int64_t r_begin = chunk * rows_per_chunk;
    int64_t r_end = r_begin + rows_per_chunk;
    if (r_end > n_out) r_end = n_out;
    AccT acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = AccT(0);
    for (int64_t r0 = r_begin; r0 < r_end; r0 += BK) {
        int valid = 0;
        if (tid < BK) {
            const int64_t r = r0 + tid;
            int32_t v = r < r_end ? map[r * ldm + k] : -1;
            if (v >= n_x) v = -1;
            rows[tid] = v;
            valid = v >= 0;
        }
        if (!__syncthreads_or(valid)) continue;
#pragma unroll
        for (int q = 0; q < (BK * BM) / NT; ++q) {
            const int e = tid + q * NT, r = e / BM, c = e % BM;
            const int32_t src = rows[r];
            Xs[r][c] = (src >= 0 && ci0 + c < cin) ? (AccT)x[(int64_t)src * ldx + ci0 + c] : AccT(0);
            Ds[r][c] = (src >= 0 && co0 + c < cout) ? (AccT)dy[(r0 + r) * lddy + co0 + c] : AccT(0);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < BK; ++r) {
            AccT a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = Xs[r][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Ds[r][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
        }
        __syncthreads();
    }
    AccT *dst = partials + ((chunk * K + k) * (int64_t)cin) * cout;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int32_t ci = ci0 + ty * 4 + i;
        if (ci >= cin) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int32_t co = co0 + tx * 4 + j;
            if (co < cout) dst[(int64_t)ci * cout + co] = acc[i][j];
        }
    }
}

// dW[e] = sum over chunks (ascending) of partials[chunk][e], accumulated in FP64.
template <typename AccT, typename OutT>
__global__ void wgrad_reduce_kernel(const AccT *__restrict__ partials, int64_t chunks, int64_t per_chunk,
                                    OutT *__restrict__ dw) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per_chunk) return;
    double s = 0.0;
    for (int64_t c = 0; c < chunks; ++c) s += (double)partials[c * per_chunk + e];
    dw[e] = (OutT)s;
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_conv_fwd_simt(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                  const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const void *w,
                                  int64_t wsk, int64_t wsci, int64_t wsco, void *y, int32_t c_out, int64_t ldy,
                                  int32_t accumulate, fvgb_stream_t stream) {
    return fvgb_conv_fwd_simt_rows(dtype, x, n_x, c_in, ldx, map, n_out, K, ldm, nullptr, w, wsk, wsci, wsco, y, c_out,
                                   ldy, accumulate, stream);
}

extern "C" int fvgb_conv_fwd_simt_rows(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                       const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const int32_t *rows,
                                       const void *w, int64_t wsk, int64_t wsci, int64_t wsco, void *y, int32_t c_out,
                                       int64_t ldy, int32_t accumulate, fvgb_stream_t stream) {
    if (c_in < 1 || c_out < 1 || K < 1 || n_out < 0 || n_x < 0 || ldm < K || ldx < c_in || ldy < c_out)
        return FVGB_EINVAL;
    if (n_out == 0) return FVGB_OK;
    if (!map || !w || !y || (n_x > 0 && !x)) return FVGB_EINVAL;
    const dim3 grid((unsigned)ceil_div(n_out, FM), (unsigned)ceil_div(c_out, FN));
    if (grid.y > 65535) return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    if (dtype == FVGB_F32) {
        conv_fwd_simt_kernel<float><<<grid, NT, 0, s>>>((const float *)x, n_x, c_in, ldx, map, n_out, K, ldm,
                                                        (const float *)w, wsk, wsci, wsco, (float *)y, c_out, ldy,
                                                        accumulate, rows);
    } else if (dtype == FVGB_F64) {
        conv_fwd_simt_kernel<double><<<grid, NT, 0, s>>>((const double *)x, n_x, c_in, ldx, map, n_out, K, ldm,
                                                         (const double *)w, wsk, wsci, wsco, (double *)y, c_out,
                                                         ldy, accumulate, rows);
    } else {
        return FVGB_ETYPE;
    }
    count_launches(1);
    return launch_status();
}

extern "C" int fvgb_wgrad_workspace(int32_t dtype, int64_t n_out, int32_t K, int32_t c_in, int32_t c_out,
                                    size_t *bytes) {
    if (!bytes || K < 1 || c_in < 1 || c_out < 1 || n_out < 0) return FVGB_EINVAL;
    const WgradPlan p = wgrad_plan(n_out, K, c_in, c_out);
    const size_t elem = dtype == FVGB_F64 ? 8 : 4;
    *bytes = (size_t)p.chunks * K * c_in * c_out * elem + 256;
    return FVGB_OK;
}

extern "C" int fvgb_conv_wgrad_simt(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                    const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const void *dy,
                                    int32_t c_out, int64_t lddy, void *dw, void *workspace,
                                    size_t workspace_bytes, fvgb_stream_t stream) {
    if (c_in < 1 || c_out < 1 || K < 1 || n_out < 0 || n_x < 0 || ldm < K || ldx < c_in || lddy < c_out || !dw)
        return FVGB_EINVAL;
    size_t need = 0;
    fvgb_wgrad_workspace(dtype, n_out, K, c_in, c_out, &need);
    if (!workspace || workspace_bytes < need) return FVGB_ENOSPACE;
    const WgradPlan p = wgrad_plan(n_out, K, c_in, c_out);
    cudaStream_t s = as_stream(stream);
    const int64_t per_chunk = (int64_t)K * c_in * c_out;
    const dim3 grid((unsigned)p.chunks, (unsigned)K, (unsigned)(p.tiles_ci * p.tiles_co));
    if (grid.y > 65535 || grid.z > 65535) return FVGB_EINVAL;
    char *base = reinterpret_cast<char *>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    if (dtype == FVGB_F32) {
        float *part = reinterpret_cast<float *>(base);
        if (n_out > 0)
            wgrad_simt_kernel<float, float><<<grid, NT, 0, s>>>((const float *)x, n_x, c_in, ldx, map, n_out, K,
                                                               ldm, (const float *)dy, c_out, lddy,
                                                               p.rows_per_chunk, p.tiles_co, part);
        wgrad_reduce_kernel<float, float><<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>(
            part, n_out > 0 ? p.chunks : 0, per_chunk, (float *)dw);
    } else if (dtype == FVGB_F64) {
        double *part = reinterpret_cast<double *>(base);
        if (n_out > 0)
            wgrad_simt_kernel<double, double><<<grid, NT, 0, s>>>((const double *)x, n_x, c_in, ldx, map, n_out,
                                                                 K, ldm, (const double *)dy, c_out, lddy,
                                                                 p.rows_per_chunk, p.tiles_co, part);
        wgrad_reduce_kernel<double, double><<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>(
            part, n_out > 0 ? p.chunks : 0, per_chunk, (double *)dw);
    } else {
        return FVGB_ETYPE;
    }
    count_launches(n_out > 0 ? 2 : 1);
    return launch_status();
}

// ---------------------------------------------------------------------------------------------
// Weight gradient that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a weight gradient:
// plugins running inside a host runtime that plans every device buffer ahead of time and
// forbids allocation during execution, and latency-bound serving code that must not risk the
// implicit device synchronisation or the out-of-memory failure of cudaMalloc / cudaFree in the
// middle of a request.  fvgb_conv_wgrad_simt needs a caller-provided partials workspace; this
// variant keeps its per-CTA partials in a fixed device array of this file instead (4 MiB per
// device, held by every GPU that loads the library until the process exits).
//
// * The device address of the array is looked up once per device, with that device current,
//   by the first call on that device (cudaGetSymbolAddress); make that first call before any
//   stream capture.
// * Every call shares the one array and it keeps the previous call's contents.  Each call
//   overwrites every partial it later reads (no clearing needed), so consecutive calls are
//   independent -- but calls that overlap on the GPU (different streams, or concurrent host
//   threads) race on the array and must be serialised by the caller.
// * Sizes whose partials of one row chunk (K * c_in * c_out elements) exceed the array are
//   rejected with FVGB_ENOSPACE before any launch.
// ---------------------------------------------------------------------------------------------
#include <mutex>

static constexpr size_t kWgradScratchBytes = size_t(4) << 20;
static __device__ __align__(256) double fvgb_wgrad_scratch[kWgradScratchBytes / sizeof(double)];

namespace fvgb {
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of fvgb_wgrad_scratch on the current device (looked up once per device).
int wgrad_scratch_address(void **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_cuda(e);
    if (dev < 0 || dev >= kMaxDevices) return FVGB_EINVAL;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, fvgb_wgrad_scratch);
        if (e != cudaSuccess) return record_cuda(e);
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return FVGB_OK;
}
}  // namespace
}  // namespace fvgb

extern "C" int fvgb_conv_wgrad_simt_noalloc(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                            const int32_t *map, int64_t n_out, int32_t K, int64_t ldm,
                                            const void *dy, int32_t c_out, int64_t lddy, void *dw,
                                            fvgb_stream_t stream) {
    if (c_in < 1 || c_out < 1 || K < 1 || n_out < 0 || n_x < 0 || ldm < K || ldx < c_in || lddy < c_out || !dw)
        return FVGB_EINVAL;
    if (dtype != FVGB_F32 && dtype != FVGB_F64) return FVGB_ETYPE;
    if (K > 65535) return FVGB_EINVAL;  // one grid row per kernel offset
    const size_t elem = dtype == FVGB_F64 ? 8 : 4;
    // K*c_in*c_out*elem <= the array, compared without overflow: K*c_in < 2^47 fits int64, and
    // for integers a*b > c  <=>  a > floor(c / b)
    const int64_t kc = (int64_t)K * c_in;
    if (kc > (int64_t)(kWgradScratchBytes / ((size_t)c_out * elem))) {
        record_message("fvgb_conv_wgrad_simt_noalloc: K*c_in*c_out partials exceed the 4 MiB scratch array");
        return FVGB_ENOSPACE;
    }
    const size_t per_chunk_bytes = (size_t)kc * (size_t)c_out * elem;
    const int64_t cap_chunks = (int64_t)(kWgradScratchBytes / per_chunk_bytes);
    void *scratch = nullptr;
    const int st = wgrad_scratch_address(&scratch);
    if (st != FVGB_OK) return st;
    WgradPlan p = wgrad_plan(n_out, K, c_in, c_out);
    if (p.chunks > cap_chunks) {
        p.rows_per_chunk = ceil_div(ceil_div(n_out > 0 ? n_out : 1, cap_chunks), BK) * BK;
        p.chunks = ceil_div(n_out > 0 ? n_out : 1, p.rows_per_chunk);
    }
    cudaStream_t s = as_stream(stream);
    const int64_t per_chunk = (int64_t)K * c_in * c_out;
    const dim3 grid((unsigned)p.chunks, (unsigned)K, (unsigned)(p.tiles_ci * p.tiles_co));
    if (grid.y > 65535 || grid.z > 65535) return FVGB_EINVAL;
    if (dtype == FVGB_F32) {
        float *part = reinterpret_cast<float *>(scratch);
        if (n_out > 0)
            wgrad_simt_kernel<float, float><<<grid, NT, 0, s>>>((const float *)x, n_x, c_in, ldx, map, n_out, K,
                                                               ldm, (const float *)dy, c_out, lddy,
                                                               p.rows_per_chunk, p.tiles_co, part);
        wgrad_reduce_kernel<float, float><<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>(
            part, n_out > 0 ? p.chunks : 0, per_chunk, (float *)dw);
    } else {
        double *part = reinterpret_cast<double *>(scratch);
        if (n_out > 0)
            wgrad_simt_kernel<double, double><<<grid, NT, 0, s>>>((const double *)x, n_x, c_in, ldx, map, n_out,
                                                                 K, ldm, (const double *)dy, c_out, lddy,
                                                                 p.rows_per_chunk, p.tiles_co, part);
        wgrad_reduce_kernel<double, double><<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>(
            part, n_out > 0 ? p.chunks : 0, per_chunk, (double *)dw);
    }
    count_launches(n_out > 0 ? 2 : 1);
    return launch_status();
}
