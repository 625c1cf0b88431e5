// Leaf-local halo convolution: stride-1 3x3x3 sparse convolution of a grid onto itself without a
// kernel map (GridBatch.sparse_conv_halo).
//
//   y[v] = sum_{k<27} x[v + d_k] . W[k],   d_k = (k/9 - 1, (k/3)%3 - 1, k%3 - 1)
//
// (the kernel map's offset order: ijk axis 0 moves with k/9, i.e. weight dim K2; W = [27, Cin,
// Cout]).  One CTA per leaf stages the leaf's 10x10x10 halo -- the leaf and a one-voxel shell of
// its 26 neighbours -- in shared memory, a chunk of input channels at a time, and computes the
// leaf's active voxels only, so a sparse surface leaf costs its active rows and no [N, 27] map is
// built.  The 27 neighbour leaves are found once per CTA through the grid's leaf hash; a halo
// position's row is then a mask test and a popcount.  The data gradient is the same kernel with
// mirrored offsets and transposed channels (W'[k] = W[26-k]^T); the weight gradient accumulates
// dW[k] = sum_v x[v + d_k]^T dy[v] per (leaf chunk, offset, channel tile) CTA, with the
// neighbour found by the same leaf lookup, and sums the chunks' FP32 partials in FP64 in a fixed
// order (deterministic).
//
// CUDA-core arithmetic (FP32 accumulation for FP32 / BF16 / FP16 data, FP64 for FP64).  Replaces
// the reference's halo backend: stencilConvHaloKernel and its gradient
// (src/fvdb/detail/ops/convolution/backend/SparseConvolutionHalo.cu:22-351,
// SparseConvolutionHaloGrad.cu:161-273, autograd/SparseConvolutionHalo.cpp:17-86).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace fvgb {
namespace {

constexpr int kHT = 256;     // threads per CTA
constexpr int kHalo = 1000;  // 10^3 halo positions
constexpr int kCoTile = 16;  // output channels per pass (two halves of 8)

template <typename T>
struct HNum;
template <>
struct HNum<float> {
    using A = float;
    static constexpr int CC = 16;  // input channels staged per pass
    __device__ static float to(float v) { return v; }
    __device__ static float from(float v) { return v; }
};
template <>
struct HNum<double> {
    using A = double;
    static constexpr int CC = 8;
    __device__ static double to(double v) { return v; }
    __device__ static double from(double v) { return v; }
};
template <>
struct HNum<__nv_bfloat16> {
    using A = float;
    static constexpr int CC = 16;
    __device__ static float to(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static __nv_bfloat16 from(float v) { return __float2bfloat16_rn(v); }
};
template <>
struct HNum<__half> {
    using A = float;
    static constexpr int CC = 16;
    __device__ static float to(__half v) { return __half2float(v); }
    __device__ static __half from(float v) { return __float2half_rn(v); }
};

template <typename T>
constexpr int halo_smem_bytes() {
    using A = typename HNum<T>::A;
    return (kHalo + 1) * (HNum<T>::CC + 1) * (int)sizeof(A) + 27 * HNum<T>::CC * kCoTile * (int)sizeof(A) +
           kHalo * 2 * 4 + 512 * 2 * 4 + 48 * 4;
}

// Halo of leaf `lf`: the active positions among its 1000 (the leaf and a one-voxel shell of its
// 26 neighbours) in position order, hslot[p] = compact slot of position p or -1 and hrow[slot] =
// its voxel row; and the leaf's active voxels (bit and row) in index order.  Returns
// {active voxels, active halo positions}.
__device__ int2 halo_setup(const FvgbGrid &g, int64_t lf, int32_t *hslot, int32_t *hrow, int32_t *act_bit,
                           int32_t *act_row, int32_t *nbr, int32_t *wcnt) {
    const FvgbLeaf &leaf = g.leaves[lf];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int32_t ox = leaf.origin[0], oy = leaf.origin[1], oz = leaf.origin[2], b = leaf.batch;
    if (tid < 27) {
        const int dx = tid / 9 - 1, dy = (tid / 3) % 3 - 1, dz = tid % 3 - 1;
        nbr[tid] = (dx | dy | dz) == 0 ? (int32_t)lf : find_leaf(g, b, (ox >> 3) + dx, (oy >> 3) + dy, (oz >> 3) + dz);
    }
    __syncthreads();
    int n_halo = 0;
    for (int p0 = 0; p0 < kHalo; p0 += kHT) {
        const int p = p0 + tid;
        int32_t row = -1;
        if (p < kHalo) {
            const int a = p / 100 - 1, bb = (p / 10) % 10 - 1, c = p % 10 - 1;  // -1 .. 8 per axis
            const int lx = a < 0 ? -1 : (a > 7 ? 1 : 0), ly = bb < 0 ? -1 : (bb > 7 ? 1 : 0),
                      lz = c < 0 ? -1 : (c > 7 ? 1 : 0);
            const int32_t id = nbr[(lx + 1) * 9 + (ly + 1) * 3 + (lz + 1)];
            if (id >= 0) row = (int32_t)leaf_voxel_index(g.leaves[id], leaf_bit(a & 7, bb & 7, c & 7));
        }
        const uint32_t ball = __ballot_sync(0xffffffffu, row >= 0);
        if (lane == 0) wcnt[warp] = __popc(ball);
        __syncthreads();
        int before = n_halo, total = 0;
#pragma unroll
        for (int w = 0; w < kHT / 32; ++w) {
            if (w < warp) before += wcnt[w];
            total += wcnt[w];
        }
        const int slot = before + __popc(ball & ((1u << lane) - 1u));
        if (p < kHalo) hslot[p] = row >= 0 ? slot : -1;
        if (row >= 0) hrow[slot] = row;
        n_halo += total;
        __syncthreads();
    }
    // active voxels of the leaf, in bit (= index) order: warp w takes bits [64 w, 64 w + 64)
    if (warp < 8) {
        const uint64_t m = leaf.mask[warp];
        const int base = leaf.prefix[warp];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int sh = 32 * h + lane;
            if ((m >> sh) & 1ull) {
                const int r = base + __popcll(m & ((1ull << sh) - 1ull));
                act_bit[r] = 64 * warp + sh;
                act_row[r] = (int32_t)(leaf.base + r);
            }
        }
    }
    __syncthreads();
    int n = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) n += __popcll(leaf.mask[w]);
    return make_int2(n, n_halo);
}

template <typename A>
__device__ __forceinline__ void load8(const A *p, A (&v)[8]);
template <>
__device__ __forceinline__ void load8<float>(const float *p, float (&v)[8]) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
}
template <>
__device__ __forceinline__ void load8<double>(const double *p, double (&v)[8]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double2 q = reinterpret_cast<const double2 *>(p)[i];
        v[2 * i] = q.x, v[2 * i + 1] = q.y;
    }
}

// y = conv(x, W) over the leaves, W [27, Cin, Cout].  mirror != 0 computes the data gradient:
// offset k takes W[26-k]^T, with W given as the forward's [27, Cout_fwd = Cin, Cin_fwd = Cout].
// Per leaf and 16-channel output tile, the CTA loops over input-channel slices of CC: the slice's
// rows of the active halo positions (plus one zero row that absent positions read) and its
// 27 x CC x 16 weights are staged in shared memory (zero-padded channels); thread t accumulates
// 4 active voxels (4 (t/2) ..) x 8 output channels (8 (t%2) ..), so every staged value it loads
// feeds 4 or 8 FMAs.
template <typename T>
__global__ void __launch_bounds__(kHT, 2) halo_fwd_kernel(FvgbGrid g, const T *__restrict__ x, int64_t ldx, int32_t Cin,
                                                       const T *__restrict__ w, int32_t Cout, int32_t mirror,
                                                       T *__restrict__ y, int64_t ldy) {
    using A = typename HNum<T>::A;
    constexpr int CC = HNum<T>::CC;
    constexpr int RS = CC + 1;  // padded row stride of the staged halo (bank spread)
    extern __shared__ __align__(16) uint8_t hsm[];
    A *wsm = reinterpret_cast<A *>(hsm);  // [27][CC][16], 16-byte aligned rows
    A *hbuf = wsm + 27 * CC * kCoTile;    // [active halo rows + 1 zero row][RS]
    int32_t *hslot = reinterpret_cast<int32_t *>(hbuf + (kHalo + 1) * RS);
    int32_t *hrow = hslot + kHalo;
    int32_t *act_bit = hrow + kHalo;
    int32_t *act_row = act_bit + 512;
    int32_t *nbr = act_row + 512;
    int32_t *wcnt = nbr + 32;
    const int tid = threadIdx.x;
    const int vg = tid >> 1, ch = (tid & 1) * 8;
    for (int64_t lf = blockIdx.x; lf < g.num_leaves; lf += gridDim.x) {
        __syncthreads();
        const int2 na = halo_setup(g, lf, hslot, hrow, act_bit, act_row, nbr, wcnt);
        const int n_act = na.x, n_halo = na.y;
        const bool busy = 4 * vg < n_act;
        int hb[4];  // halo position of each of the thread's voxels (offset k adds off_k)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int a = 4 * vg + v;
            const int bit = a < n_act ? act_bit[a] : 0;
            hb[v] = ((bit >> 6) * 10 + ((bit >> 3) & 7)) * 10 + (bit & 7);
        }
        for (int co0 = 0; co0 < Cout; co0 += kCoTile) {
            A acc[4][8];
#pragma unroll
            for (int v = 0; v < 4; ++v)
#pragma unroll
                for (int e = 0; e < 8; ++e) acc[v][e] = (A)0;
            for (int c0 = 0; c0 < Cin; c0 += CC) {
                __syncthreads();
                for (int e = tid; e < (n_halo + 1) * CC; e += kHT) {
                    const int sl = e / CC, ci = e % CC;
                    hbuf[sl * RS + ci] = (sl < n_halo && c0 + ci < Cin)
                                             ? HNum<T>::to(x[(int64_t)hrow[sl] * ldx + c0 + ci])
                                             : (A)0;
                }
                for (int e = tid; e < 27 * CC * kCoTile; e += kHT) {
                    const int k = e / (CC * kCoTile), ci = (e / kCoTile) % CC, j = e % kCoTile;
                    const int c = c0 + ci, o = co0 + j;
                    A v = (A)0;
                    if (c < Cin && o < Cout)
                        v = HNum<T>::to(mirror ? w[((int64_t)(26 - k) * Cout + o) * Cin + c]
                                               : w[((int64_t)k * Cin + c) * Cout + o]);
                    wsm[e] = v;
                }
                __syncthreads();
                if (busy) {
                    for (int k = 0; k < 27; ++k) {
                        const int off = (k / 9) * 100 + ((k / 3) % 3) * 10 + (k % 3);
                        int sl[4];
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            const int q = hslot[hb[v] + off];
                            sl[v] = (q < 0 ? n_halo : q) * RS;
                        }
                        const A *wk = wsm + k * CC * kCoTile + ch;
#pragma unroll
                        for (int ci = 0; ci < CC; ++ci) {
                            A wv[8];
                            load8<A>(wk + ci * kCoTile, wv);
#pragma unroll
                            for (int v = 0; v < 4; ++v) {
                                const A h = hbuf[sl[v] + ci];
#pragma unroll
                                for (int e = 0; e < 8; ++e) acc[v][e] += h * wv[e];
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const int a = 4 * vg + v;
                if (a >= n_act) continue;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int co = co0 + ch + e;
                    if (co < Cout) y[(int64_t)act_row[a] * ldy + co] = HNum<T>::from(acc[v][e]);
                }
            }
        }
    }
}

// dW partials: CTA (chunk, k, tile) sums x[v + d_k]^T dy[v] over the voxels of its leaf chunk for a
// 32 (ci) x 64 (co) tile; part [chunks][27][Cin][Cout] FP32 (FP64 for FP64 data).
template <typename T>
__global__ void __launch_bounds__(kHT) halo_wgrad_kernel(FvgbGrid g, const T *__restrict__ x, int64_t ldx, int32_t Cin,
                                                         const T *__restrict__ dy, int64_t lddy, int32_t Cout,
                                                         int64_t leaves_per_chunk, int32_t tiles_co,
                                                         typename HNum<T>::A *__restrict__ part) {
    using A = typename HNum<T>::A;
    constexpr int VB = sizeof(A) == 8 ? 32 : 64;  // voxels per batch (static shared memory < 48 KB)
    __shared__ A xs[VB][33];
    __shared__ A ds[VB][65];
    __shared__ int32_t nrow[VB], vrow[VB];
    const int tid = threadIdx.x;
    const int k = blockIdx.y;
    const int ci0 = (blockIdx.z / tiles_co) * 32, co0 = (blockIdx.z % tiles_co) * 64;
    const int dx = k / 9 - 1, dyo = (k / 3) % 3 - 1, dz = k % 3 - 1;
    // thread -> outputs (ci = ci0 + tid / 8, co = co0 + (tid % 8) * 8 .. +7)
    const int tci = tid / 8, tco = (tid % 8) * 8;
    A acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = (A)0;
    const int64_t l0 = (int64_t)blockIdx.x * leaves_per_chunk;
    const int64_t l1 = min(g.num_leaves, l0 + leaves_per_chunk);
    if (l0 < l1) {
        const int64_t v0 = g.leaves[l0].base;
        const int64_t v1 = l1 < g.num_leaves ? g.leaves[l1].base : g.num_voxels;
        for (int64_t vb = v0; vb < v1; vb += VB) {
            __syncthreads();
            if (tid < VB) {
                // the voxel's neighbour at offset k through the leaf hash
                const int64_t v = vb + tid;
                int32_t r = -1;
                if (v < v1) {
                    const int32_t b = batch_of(g.voxel_offsets, g.num_grids, v);
                    const int32_t qx = g.ijk[3 * v] + dx, qy = g.ijk[3 * v + 1] + dyo, qz = g.ijk[3 * v + 2] + dz;
                    const int32_t id = find_leaf(g, b, qx >> 3, qy >> 3, qz >> 3);
                    if (id >= 0) r = (int32_t)leaf_voxel_index(g.leaves[id], leaf_bit(qx, qy, qz));
                }
                nrow[tid] = r;
                vrow[tid] = v < v1 ? (int32_t)v : -1;
            }
            __syncthreads();
            for (int e = tid; e < VB * 32; e += kHT) {
                const int i = e / 32, c = e % 32;
                xs[i][c] = (nrow[i] >= 0 && ci0 + c < Cin) ? HNum<T>::to(x[(int64_t)nrow[i] * ldx + ci0 + c]) : (A)0;
            }
            for (int e = tid; e < VB * 64; e += kHT) {
                const int i = e / 64, c = e % 64;
                ds[i][c] = (vrow[i] >= 0 && co0 + c < Cout) ? HNum<T>::to(dy[(int64_t)vrow[i] * lddy + co0 + c]) : (A)0;
            }
            __syncthreads();
#pragma unroll 4
            for (int i = 0; i < VB; ++i) {
                const A xv = xs[i][tci];
#pragma unroll
                for (int e = 0; e < 8; ++e) acc[e] += xv * ds[i][tco + e];
            }
        }
    }
    A *dst = part + (((int64_t)blockIdx.x * 27 + k) * Cin + ci0 + tci) * Cout + co0 + tco;
    if (ci0 + tci < Cin)
#pragma unroll
        for (int e = 0; e < 8; ++e)
            if (co0 + tco + e < Cout) dst[e] = acc[e];
}

template <typename A, typename T>
__global__ void halo_wgrad_reduce_kernel(const A *__restrict__ part, int64_t chunks, int64_t per_chunk,
                                         T *__restrict__ dw) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per_chunk) return;
    double s = 0.0;
    for (int64_t c = 0; c < chunks; ++c) s += (double)part[c * per_chunk + e];
    dw[e] = HNum<T>::from((typename HNum<T>::A)s);
}

int64_t halo_chunks(int64_t leaves, int tiles) {
    const int64_t want = std::max<int64_t>(1, ceil_div(8 * (int64_t)device_sm_count(), 27 * (int64_t)tiles));
    return std::min<int64_t>(std::max<int64_t>(leaves, 1), want);
}

template <typename T>
int launch_halo_fwd(const FvgbGrid &g, const void *x, int64_t ldx, int32_t Cin, const void *w, int32_t Cout,
                    int32_t mirror, void *y, int64_t ldy, cudaStream_t s) {
    constexpr int smem = halo_smem_bytes<T>();
    if (set_dynamic_smem(halo_fwd_kernel<T>, smem) != cudaSuccess)
        return launch_status();
    const unsigned blocks = (unsigned)std::min<int64_t>(g.num_leaves, (int64_t)device_sm_count() * 8);
    halo_fwd_kernel<T><<<blocks, kHT, smem, s>>>(g, (const T *)x, ldx, Cin, (const T *)w, Cout, mirror, (T *)y, ldy);
    count_launches(1);
    return launch_status();
}

template <typename T>
int launch_halo_wgrad(const FvgbGrid &g, const void *x, int64_t ldx, int32_t Cin, const void *dy, int64_t lddy,
                      int32_t Cout, void *dw, void *ws, size_t ws_bytes, cudaStream_t s) {
    using A = typename HNum<T>::A;
    const int64_t tiles_ci = ceil_div(Cin, 32), tiles_co = ceil_div(Cout, 64);
    if (tiles_ci * tiles_co > 65535) return FVGB_EINVAL;  // one grid z slice per channel tile
    const int64_t chunks = halo_chunks(g.num_leaves, (int)(tiles_ci * tiles_co));
    const int64_t per_chunk = 27LL * Cin * Cout;
    if (ws_bytes < (size_t)(chunks * per_chunk) * sizeof(A)) return FVGB_ENOSPACE;
    const int64_t lpc = ceil_div(std::max<int64_t>(g.num_leaves, 1), chunks);
    const dim3 grid((unsigned)chunks, 27, (unsigned)(tiles_ci * tiles_co));
    halo_wgrad_kernel<T><<<grid, kHT, 0, s>>>(g, (const T *)x, ldx, Cin, (const T *)dy, lddy, Cout, lpc,
                                             (int)tiles_co, (A *)ws);
    halo_wgrad_reduce_kernel<A, T><<<(unsigned)ceil_div(per_chunk, 256), 256, 0, s>>>((const A *)ws, chunks, per_chunk,
                                                                                     (T *)dw);
    count_launches(2);
    return launch_status();
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_halo_conv(int32_t dtype, const FvgbGrid *grid, const void *x, int64_t ldx, int32_t c_in,
                              const void *w, int32_t c_out, int32_t mirror, void *y, int64_t ldy,
                              fvgb_stream_t stream) {
    if (!grid || c_in < 1 || c_out < 1 || ldx < c_in || ldy < c_out) return FVGB_EINVAL;
    if (grid->num_voxels == 0) return FVGB_OK;
    if (!x || !w || !y || !grid->leaves) return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    switch (dtype) {
        case FVGB_F32: return launch_halo_fwd<float>(*grid, x, ldx, c_in, w, c_out, mirror, y, ldy, s);
        case FVGB_F64: return launch_halo_fwd<double>(*grid, x, ldx, c_in, w, c_out, mirror, y, ldy, s);
        case FVGB_BF16: return launch_halo_fwd<__nv_bfloat16>(*grid, x, ldx, c_in, w, c_out, mirror, y, ldy, s);
        case FVGB_F16: return launch_halo_fwd<__half>(*grid, x, ldx, c_in, w, c_out, mirror, y, ldy, s);
        default: return FVGB_ETYPE;
    }
}

extern "C" int fvgb_halo_wgrad_workspace(int32_t dtype, const FvgbGrid *grid, int32_t c_in, int32_t c_out,
                                         size_t *bytes) {
    if (!grid || !bytes || c_in < 1 || c_out < 1) return FVGB_EINVAL;
    if (ceil_div(c_in, 32) * ceil_div(c_out, 64) > 65535) return FVGB_EINVAL;
    const int tiles = (int)(ceil_div(c_in, 32) * ceil_div(c_out, 64));
    const size_t elem = dtype == FVGB_F64 ? 8 : 4;
    *bytes = (size_t)halo_chunks(grid->num_leaves, tiles) * 27 * c_in * c_out * elem + 256;
    return FVGB_OK;
}

extern "C" int fvgb_halo_wgrad(int32_t dtype, const FvgbGrid *grid, const void *x, int64_t ldx, int32_t c_in,
                               const void *dy, int64_t lddy, int32_t c_out, void *dw, void *workspace,
                               size_t workspace_bytes, fvgb_stream_t stream) {
    if (!grid || c_in < 1 || c_out < 1 || ldx < c_in || lddy < c_out || !dw || !workspace) return FVGB_EINVAL;
    if (((uintptr_t)workspace & 15)) return FVGB_EINVAL;
    if (grid->num_voxels > 0 && (!x || !dy || !grid->leaves || !grid->ijk)) return FVGB_EINVAL;
    cudaStream_t s = as_stream(stream);
    switch (dtype) {
        case FVGB_F32: return launch_halo_wgrad<float>(*grid, x, ldx, c_in, dy, lddy, c_out, dw, workspace, workspace_bytes, s);
        case FVGB_F64: return launch_halo_wgrad<double>(*grid, x, ldx, c_in, dy, lddy, c_out, dw, workspace, workspace_bytes, s);
        case FVGB_BF16:
            return launch_halo_wgrad<__nv_bfloat16>(*grid, x, ldx, c_in, dy, lddy, c_out, dw, workspace, workspace_bytes, s);
        case FVGB_F16: return launch_halo_wgrad<__half>(*grid, x, ldx, c_in, dy, lddy, c_out, dw, workspace, workspace_bytes, s);
        default: return FVGB_ETYPE;
    }
}
