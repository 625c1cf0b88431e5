/*
 * fvdb_gb300 — C ABI of the GB300 sparse-convolution path (libfvdb_gb300.so).
 *
 * Conventions for every entry point:
 *   - plain C types only; every buffer is caller-allocated device memory unless the
 *     argument says "host"; the library never allocates, frees or keeps a pointer
 *     after returning;
 *   - all device work is enqueued on the `stream` argument (0 = legacy default);
 *   - return value is a status code (FVGB_OK on success); nothing throws.
 *   - counts are int64, map entries are int32 (-1 = no neighbour), exactly as in the
 *     reference's torch tensors.
 *
 * Each declaration names the reference interface it replaces (fvdb-core paths).
 */
#ifndef FVDB_GB300_H
#define FVDB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void *fvgb_stream_t; /* a cudaStream_t */

/* status codes; the host wrapper maps them to ValueError / TypeError / RuntimeError */
enum {
    FVGB_OK = 0,
    FVGB_EINVAL = 1,   /* bad shape / size / argument          -> ValueError   */
    FVGB_ETYPE = 2,    /* unsupported element type or layout  -> TypeError    */
    FVGB_ERANGE = 3,   /* coordinate outside the supported box -> ValueError  */
    FVGB_ECUDA = 4,    /* CUDA launch or runtime failure       -> RuntimeError */
    FVGB_ETIMEOUT = 5, /* a bounded device wait gave up        -> RuntimeError */
    FVGB_ENOSPACE = 6  /* caller workspace too small           -> RuntimeError */
};

/* element types */
enum { FVGB_F32 = 0, FVGB_F64 = 1, FVGB_BF16 = 2, FVGB_F16 = 3, FVGB_E4M3 = 4 };

/* Voxel coordinates must lie in [-2^20, 2^20) on every axis (the sort key packs nine
 * root-tile bits per axis); grids may hold up to 2^31-1 voxels. */
#define FVGB_COORD_LIMIT (1 << 20)

/*
 * One leaf (8x8x8 brick) of an index grid.  Voxels of a leaf are contiguous in the
 * grid's index order; bit b = (x&7)<<6 | (y&7)<<3 | (z&7) of `mask` marks an active
 * voxel, whose index is base + prefix[b>>6] + popcount(mask[b>>6] & ((1<<(b&63))-1)).
 * Replaces nanovdb::OnIndexTree::LeafNodeType as used by GridBatchImpl::Accessor
 * (src/fvdb/detail/GridBatchImpl.h:118-245).  128 bytes, 128-byte aligned.
 */
typedef struct FvgbLeaf {
    int32_t origin[3]; /* coordinate of voxel (0,0,0) of the leaf, multiples of 8 */
    int32_t batch;     /* grid of the batch this leaf belongs to */
    int64_t base;      /* global index of the leaf's first active voxel */
    uint16_t prefix[8];
    uint64_t mask[8];
    int64_t pad[3];
} FvgbLeaf;

/*
 * A batch of index grids (a jagged GridBatch), as a view over caller-owned device
 * memory.  Replaces fvdb::detail::GridBatchImpl's device accessor
 * (src/fvdb/detail/GridBatchImpl.h:118-245) for the convolution path.
 */
typedef struct FvgbGrid {
    int32_t num_grids;
    int32_t reserved;
    int64_t num_voxels;
    int64_t num_leaves;
    int64_t hash_capacity;        /* power of two, >= 2 * num_leaves */
    const int64_t *voxel_offsets; /* [num_grids+1] device, int64 (fvdb joffsets) */
    const int32_t *ijk;           /* [num_voxels,3] device, index order */
    const FvgbLeaf *leaves;       /* [num_leaves] device, index order */
    const int32_t *hash_slots;    /* [hash_capacity] device, leaf id or -1 */
} FvgbGrid;

/* Library version and build info (host). */
const char *fvgb_version(void);
/* Last CUDA error string seen by the library on this thread (host). */
const char *fvgb_last_error(void);
/* Number of kernels this library has launched in this process (host; library kernels of
 * CUB used inside the grid builder are not counted). */
uint64_t fvgb_launch_count(void);

/* ---------------------------------------------------------------- grid build ----- */

/*
 * Bytes of workspace that fvgb_ijk_sort_unique needs for n input coordinates.
 * (host, no device work)
 */
int fvgb_ijk_sort_unique_workspace(int64_t n, int32_t num_grids, size_t *bytes);

/*
 * Sort jagged ijk [n,3] (grid b owns rows joffsets[b]..joffsets[b+1]) into the
 * NanoVDB OnIndex voxel order of each grid and drop duplicates.  Writes out_ijk
 * (capacity n rows) and out_joffsets[num_grids+1] (device); the unique count is
 * out_joffsets[num_grids].  *err_dev (device int32, zeroed by the caller) becomes
 * FVGB_ERANGE if a coordinate is outside FVGB_COORD_LIMIT.
 * Replaces dispatchCreateNanoGridFromIJK<kCUDA> (src/fvdb/detail/ops/BuildGridFromIjk.cu:26-83)
 * and its nanovdb::tools::cuda::voxelsToGrid call, without the per-grid host loop.
 */
int fvgb_ijk_sort_unique(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids, int64_t n,
                         int32_t *out_ijk, int64_t *out_joffsets, int32_t *err_dev, void *workspace,
                         size_t workspace_bytes, fvgb_stream_t stream);

/*
 * fvgb_ijk_sort_unique for callers that know bounds of the coordinates: every ijk lies in
 * [box_lo, box_hi] (host int32[3] each).  The radix sort then covers only the order-key bits
 * that can differ inside the box (e.g. 21 of 63 bits for coordinates in [0,128)^3), with the
 * same result as the full sort; a coordinate outside the box raises FVGB_ERANGE in *err_dev.
 * Same workspace as fvgb_ijk_sort_unique.  Used for conv_grid targets, whose bounds follow
 * from the source grid's (no counterpart in the reference: its builder sorts full keys).
 */
int fvgb_ijk_sort_unique_in_box(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids, int64_t n,
                                const int32_t *box_lo, const int32_t *box_hi, int32_t *out_ijk,
                                int64_t *out_joffsets, int32_t *err_dev, void *workspace,
                                size_t workspace_bytes, fvgb_stream_t stream);

/*
 * Leaf ids of sorted unique ijk: leaf_ids[i] = 1 + id of the leaf of voxel i (inclusive scan
 * of leaf starts).  n is a capacity (>= joffsets[num_grids], the voxel count, read on the
 * device), so this can run straight after fvgb_ijk_sort_unique without a host round trip.
 * num_leaves_dev (device int64[2]) receives {leaf count, voxel count}.
 * workspace: fvgb_scan_workspace(n) bytes.
 */
int fvgb_scan_workspace(int64_t n, size_t *bytes);
int fvgb_grid_leaf_scan(const int32_t *ijk, const int64_t *joffsets, int32_t num_grids, int64_t n,
                        int32_t *leaf_ids, int64_t *num_leaves_dev, void *workspace,
                        size_t workspace_bytes, fvgb_stream_t stream);

/*
 * Fill grid->leaves and grid->hash_slots (both caller-allocated, writable through the
 * casts) from sorted unique ijk and the leaf ids of fvgb_grid_leaf_scan.  Replaces the
 * NanoVDB tree build + PopulateGridMetadata (src/fvdb/detail/ops/PopulateGridMetadata.cu:39-90).
 */
int fvgb_grid_index_build(const FvgbGrid *grid, const int32_t *leaf_ids, fvgb_stream_t stream);

/*
 * Coarse grid of floor(ijk / factor) (factor[a] in {1, 2, 4, 8}; num_grids <= 1024), built leaf by
 * leaf: the fine leaves are grouped by the coarse leaf they fall in (one radix-sort key per fine
 * leaf, not per voxel), each coarse leaf's mask is the OR of its fine leaves' voxels mapped down,
 * and the coarse voxels are written leaf by leaf in bit order -- the same voxels in the same
 * order as fvgb_ijk_sort_unique of floor(ijk / factor).  out_ijk and leaf_ids (capacity: the fine
 * voxel count) receive the sorted voxels and their 1-based leaf ids (as fvgb_grid_leaf_scan);
 * meta (device int64 [num_grids + 3], zeroed) the voxel offsets [0..num_grids], the leaf count and
 * the voxel count.  box_lo/box_hi (optional, host int32[3]): bounds of the coarse voxels, which
 * shorten the sort to the key bits that vary.  The fine grid must have at least one leaf.
 * Replaces the coarse-grid paths of
 * BuildGridForConv (src/fvdb/detail/ops/BuildGridForConv.cu:181-255, CoarseIjkForFineGrid.cu:19-41)
 * and BuildCoarseGridFromFine.
 */
int fvgb_coarse_grid_workspace(int64_t num_fine_leaves, size_t *bytes);
int fvgb_coarse_grid_build(const FvgbGrid *fine, const int32_t factor[3], const int32_t *box_lo, const int32_t *box_hi,
                           int32_t *out_ijk, int64_t *meta, int32_t *leaf_ids, void *workspace, size_t workspace_bytes,
                           fvgb_stream_t stream);

/*
 * Index of each query coordinate (query q belongs to grid b with joffsets[b] <= q <
 * joffsets[b+1]) in `grid`, or -1 where the grid has no voxel; global (cumulative != 0) or
 * per-grid index.  One leaf-hash probe per query.  Replaces GridBatch::ijk_to_index
 * (src/fvdb/GridBatch.cpp, dispatchIjkToIndex) for the convolution path's callers.
 */
int fvgb_ijk_to_index(const FvgbGrid *grid, const int32_t *ijk, const int64_t *joffsets, int64_t n,
                      int32_t cumulative, int64_t *out, fvgb_stream_t stream);

/*
 * ijk of points, per grid: ijk = floor(fma(p, s, t) + 1/2) with s = 1/voxel_size and
 * t = -origin/voxel_size, evaluated in the points' own arithmetic type as the reference does
 * (at::opmath_type: double for FVGB_F64 points; float for FVGB_F32, FVGB_F16 and FVGB_BF16
 * points, with s and t rounded once to float).  points [n,3] of `dtype`; per-grid
 * voxel_size/origin f64 [num_grids,3] (device); the grid of each point from joffsets.
 * Replaces ijkForPoints + VoxelCoordTransform::apply(...).round()
 * (src/fvdb/detail/ops/BuildGridFromPoints.cu:27-43, src/fvdb/detail/VoxelCoordTransform.h:86-110).
 */
int fvgb_points_to_ijk(int32_t dtype, const void *points, const int64_t *joffsets, int32_t num_grids, int64_t n,
                       const double *voxel_sizes, const double *origins, int32_t *out_ijk,
                       fvgb_stream_t stream);

/*
 * Candidate coordinates of conv_grid(kernel, stride) for every voxel of `grid`
 * (k = k0*k1*k2 candidates per voxel, or one when stride==1 or stride==kernel).
 * Writes out_ijk [num_voxels*kc, 3] and out_valid [num_voxels*kc] (uint8); the caller
 * compacts (fvgb_compact_ijk) and sorts (fvgb_ijk_sort_unique).
 * Replaces convIJKForGrid / dispatchCoarseIJKForFineGrid
 * (src/fvdb/detail/ops/BuildGridForConv.cu:66-178, src/fvdb/detail/ops/CoarseIjkForFineGrid.cu:19-75).
 */
int fvgb_conv_grid_candidates(const FvgbGrid *grid, const int32_t ksize[3], const int32_t stride[3],
                              int32_t *out_ijk, uint8_t *out_valid, fvgb_stream_t stream);

/*
 * Stream-compact flagged rows: out_ijk/out_joffsets get the rows of ijk whose flag is
 * non-zero, grouped per grid (row r of the candidates belongs to grid of voxel r/per_voxel).
 * workspace: fvgb_scan_workspace(n) bytes.
 */
int fvgb_compact_ijk(const int32_t *ijk, const uint8_t *valid, const int64_t *src_joffsets,
                     int32_t num_grids, int64_t per_voxel, int64_t n, int32_t *out_ijk,
                     int64_t *out_joffsets, void *workspace, size_t workspace_bytes,
                     fvgb_stream_t stream);

/* ---------------------------------------------------------------- kernel maps ---- */

/*
 * Kernel map: kmap[t*ld + k] = index of the source voxel at
 * (t.x*s2 + dx, t.y*s1 + dy, t.z*s0 + dz) or -1, with the reference's offset order
 * and axis convention (k0 and s0 act on ijk axis 2).  Rows [tgt->num_voxels, ...)
 * are not touched.  If nbsizes (device int32[K]) is non-null, the per-offset count of
 * valid entries is ADDED to it.  If tile_mask (device uint32[ceil(N_tgt/128)], zeroed by the
 * caller; K <= 32) is non-null, bit k of tile_mask[t] is set when any row of the 128-row tile
 * t has a neighbour at offset k (the occupancy mask the contractions use to skip offsets).
 * Replaces dispatchConvolutionKernelMap<kCUDA>
 * (src/fvdb/detail/ops/convolution/pack_info/ConvolutionKernelMap.cu:104-138).
 */
int fvgb_kmap_build(const FvgbGrid *src, const FvgbGrid *tgt, const int32_t ksize[3],
                    const int32_t stride[3], int32_t *kmap, int64_t ld, int32_t *nbsizes,
                    uint32_t *tile_mask, fvgb_stream_t stream);

/*
 * mapT[i*ldT + k] = t where kmap[t*ld + k] == i, else -1 (fills all n_in rows).
 * Replaces dispatchTransposeOutInMap
 * (src/fvdb/detail/ops/convolution/pack_info/IGEMMBitOperations.cu:92-105,164-182).
 */
int fvgb_kmap_transpose(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *mapT,
                        int64_t n_in, int64_t ldT, fvgb_stream_t stream);

/*
 * Gather-scatter neighbour map: nbmap[p] = (in, out) for every valid kmap entry,
 * ordered by offset then by output row; nboffsets[k] = exclusive prefix of nbsizes
 * (device int64[K+1], computed here).  workspace: fvgb_nbmap_workspace bytes.
 * Replaces SparseConvPackInfo::buildGatherScatter (src/fvdb/SparseConvPackInfo.cpp:61-88).
 */
int fvgb_nbmap_workspace(int64_t n_out, int32_t K, size_t *bytes);
int fvgb_nbmap_build(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *nbmap,
                     int64_t *nboffsets, void *workspace, size_t workspace_bytes,
                     fvgb_stream_t stream);

/*
 * Per-row occupancy bitmask (bit k set when kmap[t,k] >= 0) for K <= 32, and the
 * OR-reduced mask of every 128-row tile.  Replaces dispatchBitmaskFromOutInMap and
 * dispatchReduceMask (IGEMMBitOperations.cu:14-36,54-90).
 */
int fvgb_kmap_masks(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, uint32_t *row_mask,
                    uint32_t *tile_mask, fvgb_stream_t stream);

/*
 * Row order for the contractions (K <= 32): the rows of kmap sorted by occupancy mask, descending
 * (a stable radix sort), so that the 128 rows of a contraction tile tend to share their present
 * offsets and the per-tile mask skips more of the reduction.  rows [ceil(n_out/128)*128] receives
 * the order (padding -1), tile_mask [ceil(n_out/128)] the OR of each ordered tile's row masks,
 * and sorted_map (optional, [ceil(n_out/128)*128, K]) the map's rows in that order (-1 rows for
 * padding), which the *_rows contractions read tile by tile.  The sorted-mask / reorder_loc /
 * reordered out_in_map of the reference's sorted implicit GEMM (SparseConvPackInfo.cpp:110-147,
 * IGEMMBitOperations.cu:14-90), computed on the device.
 */
int fvgb_kmap_row_order_workspace(int64_t n_out, int32_t K, size_t *bytes);
int fvgb_kmap_row_order(const int32_t *kmap, int64_t n_out, int32_t K, int64_t ld, int32_t *rows,
                        uint32_t *tile_mask, int32_t *sorted_map, void *workspace, size_t workspace_bytes,
                        fvgb_stream_t stream);

/* ---------------------------------------------------------------- contractions --- */

/*
 * Forward gather-GEMM on CUDA cores, one fused pass, no atomics:
 *   y[m, :] (+)= sum_k x[map[m*ldm + k], :] . W[k]      for m < n_out
 * x [n_x, c_in] rows of length ldx; W element (k, ci, co) at
 * w[k*wsk + ci*wsci + co*wsco]; y [n_out, c_out] rows of length ldy.  dtype FVGB_F32
 * or FVGB_F64 (x, W, y all that type).  accumulate != 0 adds into y.
 * This is the plain FP32 form (no TF32) and the FP64 form.  Together with the maps it
 * replaces the gather -> mm -> scatter loop of dispatchSparseConvolutionKernelMap
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionKernelMap.cu:116-261) and the
 * f32 IGEMM kernels (SparseConvolutionImplicitGEMM.cu:2389-2788).
 * Used for dgrad with the transposed map and W^T strides.
 */
int fvgb_conv_fwd_simt(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                       const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const void *w,
                       int64_t wsk, int64_t wsci, int64_t wsco, void *y, int32_t c_out,
                       int64_t ldy, int32_t accumulate, fvgb_stream_t stream);
/* fvgb_conv_fwd_simt over 128-row tiles of a given row order (map and rows as for
 * fvgb_conv_fwd_tc_rows, padded to a multiple of 128 rows): each output row is computed exactly
 * as in index order; offsets absent from a whole tile are skipped. */
int fvgb_conv_fwd_simt_rows(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map,
                            int64_t n_out, int32_t K, int64_t ldm, const int32_t *rows, const void *w, int64_t wsk,
                            int64_t wsci, int64_t wsco, void *y, int32_t c_out, int64_t ldy, int32_t accumulate,
                            fvgb_stream_t stream);

/*
 * Weight gradient on CUDA cores:  dW[k, ci, co] = sum_m x[map[m,k], ci] * dy[m, co].
 * Per-CTA FP32 (or FP64) partials go to `partials` (fvgb_wgrad_workspace bytes); the
 * final cross-CTA reduction runs in FP64 in a fixed order (deterministic) and writes
 * dW [K, c_in, c_out] contiguous in `dtype_out` (FVGB_F32 or FVGB_F64).
 * Replaces the per-offset torch::mm_out(x_k^T, dy_k) of
 * dispatchSparseConvolutionKernelMapGrad (SparseConvolutionKernelMap.cu:263-415).
 */
int fvgb_wgrad_workspace(int32_t dtype, int64_t n_out, int32_t K, int32_t c_in, int32_t c_out,
                         size_t *bytes);
int fvgb_conv_wgrad_simt(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                         const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const void *dy,
                         int32_t c_out, int64_t lddy, void *dw, void *workspace,
                         size_t workspace_bytes, fvgb_stream_t stream);

/*
 * Weight gradient that allocates nothing -- no counterpart in the reference.
 * Same result as fvgb_conv_wgrad_simt (up to the FP32 rounding of a different chunking),
 * for callers that cannot allocate device memory when they call it: plugins inside runtimes
 * that plan all device memory ahead of time and forbid allocation during execution, and
 * serving code that must not risk cudaMalloc/cudaFree synchronising the device or failing
 * mid-request.  The partials live in a fixed 4 MiB device array of the library (every GPU
 * that loads the library holds it until exit); sizes with K*c_in*c_out*elem > 4 MiB are
 * rejected with FVGB_ENOSPACE before any launch.  The first call on a device looks up the
 * array's device address for that device (make it before any stream capture).  All calls
 * share the array: calls that overlap on the GPU race and must be serialised by the caller.
 * dtype FVGB_F32 or FVGB_F64; dw [K, c_in, c_out] contiguous.
 */
int fvgb_conv_wgrad_simt_noalloc(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                                 const int32_t *map, int64_t n_out, int32_t K, int64_t ldm, const void *dy,
                                 int32_t c_out, int64_t lddy, void *dw, fvgb_stream_t stream);

/* ------------------------------------------------------- tensor-core contractions --- */

/*
 * Bytes of the packed weight image that fvgb_conv_fwd_tc reads for a [K, c_in, c_out]
 * weight in `dtype` (FVGB_BF16 or FVGB_E4M3); c_out <= 256.  (host)
 */
int fvgb_tc_weight_bytes(int32_t dtype, int64_t K, int32_t c_in, int32_t c_out, size_t *bytes);

/*
 * Pack W (element (k, ci, co) at w[k*wsk + ci*wsci + co*wsco], elements of `dtype`) into
 * the tile image of fvgb_conv_fwd_tc: one [N_tile x 128 B] block per 128-byte unit of the
 * reduction, in the 128B-swizzled K-major shared-memory layout, zero padded.  A unit is one
 * (offset, 128-byte channel chunk) when c_in*elem >= 128 bytes, else a group of
 * 128/(c_in*elem) consecutive offsets side by side.  Strides select W or W^T, so the same
 * image format serves forward and data gradient.
 */
int fvgb_tc_pack_weights(int32_t dtype, const void *w, int64_t K, int32_t c_in, int32_t c_out, int64_t wsk,
                         int64_t wsci, int64_t wsco, void *packed, size_t packed_bytes, fvgb_stream_t stream);

/*
 * Tensor-core implicit-GEMM convolution (tcgen05.mma, FP32 accumulators in TMEM):
 *   y[m, :] = out_scale (.) sum_k x[map[m*K + k], :] . W[k]          for m < n_out
 * x: dtype (FVGB_BF16 or FVGB_E4M3) [n_x, c_in], row stride ldx elements (16-byte rows,
 * c_in*elem multiple of 32 bytes); map int32 [n_out, K] (-1 = absent); tile_mask: per
 * 128-row tile the OR of the rows' occupancy bits (fvgb_kmap_masks; may be null, K <= 32
 * only) -- offsets absent from a whole tile are skipped; packed_w from fvgb_tc_pack_weights;
 * y: bf16 [n_out, ldy]; out_scale: per output channel FP32 factor or null.  Every output
 * row is written once (no atomics).  *err_dev (caller-zeroed device int32) becomes
 * FVGB_ETIMEOUT if a bounded in-kernel wait gave up.
 * Replaces the implicit-GEMM forward kernels
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMM.cu:120-3826,
 *  SparseConvolutionImplicitGEMMSorted.cu:115-4639) and, with the transposed map and the
 * W^T image, the data gradient of SparseConvolutionImplicitGEMM::backward
 * (src/fvdb/detail/autograd/SparseConvolutionImplicitGEMM.cpp:165-177).
 */
int fvgb_conv_fwd_tc(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map,
                     int64_t n_out, int32_t K, const uint32_t *tile_mask, const void *packed_w, int32_t c_out,
                     void *y, int64_t ldy, const float *out_scale, int32_t *err_dev, fvgb_stream_t stream);

/*
 * fvgb_conv_fwd_tc with a per-output-channel FP32 bias added in the epilogue (after out_scale,
 * before the BF16 rounding): y[m, :] = out_scale (.) sum_k ... + bias.  bias may be null (then
 * identical to fvgb_conv_fwd_tc).  Rows of tiles without any active offset get the bias alone.
 * No counterpart in the reference, which adds the bias as a separate pass over the output
 * (fvdb/nn/modules.py:399-400).
 */
int fvgb_conv_fwd_tc_bias(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map,
                          int64_t n_out, int32_t K, const uint32_t *tile_mask, const void *packed_w, int32_t c_out,
                          void *y, int64_t ldy, const float *out_scale, const float *bias, int32_t *err_dev,
                          fvgb_stream_t stream);

/*
 * fvgb_conv_fwd_tc_bias with a fused activation: relu != 0 clamps every output at zero after the
 * scale and the bias (NaN passes through), so conv -> ReLU writes its output once.  Rounding to
 * BF16 keeps signs, so the result equals ReLU applied to fvgb_conv_fwd_tc_bias's output.  The
 * reference applies fvdb.nn.ReLU as a separate pass (fvdb/nn/modules.py, torch.nn.ReLU on jdata).
 */
int fvgb_conv_fwd_tc_epilogue(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                              const int32_t *map, int64_t n_out, int32_t K, const uint32_t *tile_mask,
                              const void *packed_w, int32_t c_out, void *y, int64_t ldy, const float *out_scale,
                              const float *bias, int32_t relu, int32_t *err_dev, fvgb_stream_t stream);

/*
 * fvgb_conv_fwd_tc_epilogue over tiles of a given row order: `map` holds the rows in that order
 * (fvgb_kmap_row_order's sorted_map), row 128t + r of it computes output row rows[128t + r]
 * (-1 = none), and tile_mask is that order's.  Each output row is computed exactly as in the
 * index order (same units, same order), so the result is the same; rows are stored one by one.  Replaces the sorted implicit-GEMM forward
 * (SparseConvolutionImplicitGEMMSorted.cu:115-2979, its reorder_loc gather / scatter).
 */
int fvgb_conv_fwd_tc_rows(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map,
                          int64_t n_out, int32_t K, const int32_t *rows, const uint32_t *tile_mask,
                          const void *packed_w, int32_t c_out, void *y, int64_t ldy, const float *out_scale,
                          const float *bias, int32_t relu, int32_t *err_dev, fvgb_stream_t stream);

/*
 * Tile plan of a kernel map for the planned tensor-core convolution: for every 128-row tile of
 * `map` ([ceil(n_rows/128)*128, K] int32, -1 = absent, K <= 32) the distinct source rows it
 * reads (split into phases that fit the kernel's staging buffer, which depends on row_bytes =
 * c_in * element size) and each entry's 16-bit index into its phase's row list.  Built once per
 * kernel map and feature row size; fvgb_tc_plan_bytes gives its size.  No reference counterpart
 * of the plan itself: it is the staging schedule of the kernel that replaces
 * dispatchSparseConvolutionImplicitGEMM[Sorted]<kCUDA> (see fvgb_conv_fwd_tc).
 */
int fvgb_tc_plan_bytes(int64_t n_rows, int32_t K, int32_t row_bytes, size_t *bytes);
int fvgb_tc_plan_build(const int32_t *map, int64_t n_rows, int32_t K, int32_t row_bytes, void *plan,
                       size_t plan_bytes, fvgb_stream_t stream);

/* FVGB_OK when fvgb_conv_fwd_tc_planned takes (dtype, K, c_in, c_out): K <= 32, c_out <= 128,
 * c_in * element size a multiple of 32 bytes up to 256 that tiles 128 bytes when shorter. */
int fvgb_tc_plan_supported(int32_t dtype, int32_t K, int32_t c_in, int32_t c_out);

/*
 * fvgb_conv_fwd_tc_bias over a tile plan of the same map (fvgb_tc_plan_build with
 * row_bytes = c_in * element size): each tile's distinct input rows are staged in shared memory
 * once and the gathered A operand is assembled in tensor memory, so no map entry is gathered
 * from L2 on its own.  Same arguments, weight image, result and error flag as
 * fvgb_conv_fwd_tc_epilogue (the map and tile masks are read from the plan).  Replaces
 * dispatchSparseConvolutionImplicitGEMM[Sorted]<kCUDA>
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMM.cu:2754-3826,
 * SparseConvolutionImplicitGEMMSorted.cu:3101-4641).
 */
int fvgb_conv_fwd_tc_planned(int32_t dtype, const void *x, int64_t n_x, int32_t c_in, int64_t ldx,
                             const void *plan, int64_t n_out, int32_t K, const void *packed_w, int32_t c_out,
                             void *y, int64_t ldy, const float *out_scale, const float *bias, int32_t relu,
                             int32_t *err_dev, fvgb_stream_t stream);

/*
 * Tensor-core weight gradient, BF16 operands:  dw[k, ci, co] = sum_m x[map[m,k], ci] * dy[m, co]
 * (FP32, [K, c_in, c_out] contiguous).  c_in in {32, 64, 128} (128/c_in offsets share one
 * M=128 MMA), c_out in {64, 128, 256}; rows of x and dy 16-byte aligned; map as for
 * fvgb_conv_fwd_tc ([ceil(n_out/128)*128, K], padding rows -1, 16-byte aligned).  dy is read
 * with TMA tile loads (a tensor map is encoded per call).  Per-CTA FP32 partials go to
 * `workspace` (fvgb_tc_wgrad_workspace bytes, which depend on the device's SM count) and are
 * summed across CTAs in FP64 in a fixed order (deterministic).  tile_mask as for
 * fvgb_conv_fwd_tc (may be null).
 * Replaces the split-K implicit-GEMM wgrad
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionImplicitGEMMGrad.cu:115-4101,
 *  SparseConvolutionImplicitGEMMGradSorted.cu:115-4582).
 */
int fvgb_tc_wgrad_workspace(int64_t n_out, int32_t K, int32_t c_in, int32_t c_out, size_t *bytes);
int fvgb_conv_wgrad_tc(const void *x, int64_t n_x, int32_t c_in, int64_t ldx, const int32_t *map, int64_t n_out,
                       int32_t K, const uint32_t *tile_mask, const void *dy, int32_t c_out, int64_t lddy, float *dw,
                       void *workspace, size_t workspace_bytes, int32_t *err_dev, fvgb_stream_t stream);

/*
 * FP8-E4M3 quantisation of features: out[r, c] = e4m3_satfinite(x[r, c] * inv_scale[c]),
 * x FVGB_F32 or FVGB_BF16 [n, c] (row stride ldx), out uint8 [n, ldo].  Per-channel scales
 * of the FP8 convolution (the reference has no FP8 path; its closest interface is the
 * dtype dispatch of SparseConvolutionImplicitGEMM.cu:2788-3826).
 */
int fvgb_quantize_e4m3(int32_t dtype, const void *x, int64_t n, int32_t c, int64_t ldx, const float *inv_scale,
                       void *out, int64_t ldo, fvgb_stream_t stream);

/* ------------------------------------------------------------------- self test --- */

/*
 * Exercises the bounded wait every tensor-core kernel uses (about one second there): one
 * thread waits on an mbarrier phase for at most budget_cycles SM cycles (1..2^32).  With
 * arrive == 0 nothing completes the phase, so the wait gives up and *err_dev (caller-zeroed
 * device int32) becomes FVGB_ETIMEOUT; with arrive != 0 the phase completes first and *err_dev
 * stays 0.  The GPU context stays usable either way.  No counterpart in the reference (its
 * kernels have no in-kernel waits).
 */
int fvgb_selftest_wait_timeout(int32_t *err_dev, int64_t budget_cycles, int32_t arrive, fvgb_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Pooling and nearest upsampling between a fine and a coarse grid of the same batch.
 * Features [n, C] rows in grid index order (ld = row stride in elements), dtype FVGB_F32 /
 * FVGB_F64 / FVGB_F16 / FVGB_BF16.  Window / factor volume at most 512.
 * ------------------------------------------------------------------------------------------ */
enum { FVGB_POOL_MAX = 0, FVGB_POOL_AVG = 1 };

/* y[c] = max (or average) of fine voxels c*stride + (i,j,k), i<pool[0], j<pool[1], k<pool[2]
 * (max of an empty window = -inf; average = window sum * 1/(pool volume), rounded as the
 * reference).  Replaces DownsampleGridMaxPool / DownsampleGridAvgPool
 * (src/fvdb/detail/ops/DownsampleGridMaxPool.cu:19-69,128-230, DownsampleGridAvgPool.cu:19-64,114-201). */
int fvgb_pool_forward(int32_t mode, int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse, const int32_t pool[3],
                      const int32_t stride[3], const void *x, int64_t ldx, int32_t C, void *y, int64_t ldy,
                      fvgb_stream_t stream);
/* Max-pool gradient added into dx_acc [fine n, C] (float for F32/F16/BF16, double for F64;
 * zero it first): each window's gradient goes to its first strict maximum.  Replaces
 * DownsampleGridMaxPoolBackward (DownsampleGridMaxPool.cu:71-126,232-326). */
int fvgb_maxpool_backward(int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse, const int32_t pool[3],
                          const int32_t stride[3], const void *x, int64_t ldx, int32_t C, const void *dy, int64_t lddy,
                          void *dx_acc, fvgb_stream_t stream);
/* Average-pool gradient dx [fine n, C] = sum over the windows holding a fine voxel of
 * dy * 1/(pool volume).  Replaces DownsampleGridAvgPoolBackward (DownsampleGridAvgPool.cu:68-112,203-283). */
int fvgb_avgpool_backward(int32_t dtype, const FvgbGrid *fine, const FvgbGrid *coarse, const int32_t pool[3],
                          const int32_t stride[3], int32_t C, const void *dy, int64_t lddy, void *dx, int64_t lddx,
                          fvgb_stream_t stream);
/* Nearest upsampling y[f] = x[coarse voxel floor(f / factor)] (zero where there is none), and its
 * gradient dx[c] = sum of dy over c's children.  Replaces UpsampleGridNearest[Backward]
 * (src/fvdb/detail/ops/UpsampleGridNearest.cu:19-295). */
int fvgb_upsample_forward(int32_t dtype, const FvgbGrid *coarse, const FvgbGrid *fine, const int32_t factor[3],
                          const void *x, int64_t ldx, int32_t C, void *y, int64_t ldy, fvgb_stream_t stream);
int fvgb_upsample_backward(int32_t dtype, const FvgbGrid *coarse, const FvgbGrid *fine, const int32_t factor[3],
                           const void *dy, int64_t lddy, int32_t C, void *dx, int64_t lddx, fvgb_stream_t stream);
/* Candidates of the subdivided grid: voxel c (mask[c] != 0, or all when mask is NULL) gives
 * c*factor + (i,j,k); out_ijk [n*V, 3], out_valid [n*V] (V = factor volume).  With
 * fvgb_compact_ijk and a grid build this replaces BuildFineGridFromCoarse
 * (src/fvdb/detail/ops/BuildFineGridFromCoarse.cu:66-226,343-352). */
int fvgb_subdivide_candidates(const FvgbGrid *coarse, const int32_t factor[3], const uint8_t *mask, int32_t *out_ijk,
                              uint8_t *out_valid, fvgb_stream_t stream);

/* FP32 FMA rate probe (for reporting the CUDA-core roofline of the plain FP32 form): launches
 * blocks_per_sm x SMs CTAs of 256 threads, each thread 8 independent fma chains of `iters` steps;
 * *flops (host) = FLOPs of the launch, which the caller times on `stream`.  out: device float[2].
 * No counterpart in the reference. */
int fvgb_ffma_probe(float *out, int64_t iters, int32_t blocks_per_sm, double *flops, fvgb_stream_t stream);
/* Row-gather probe (for the design notes: how fast random 128-byte feature rows reach a
 * 128B-swizzled shared-memory stage): one CTA of 256 threads per SM gathers `iters` stages of 128
 * rows (row indices rows[0..nlist), cycled) of x [n_rows, 128 B] into a 4-deep ring; mode 0/1/2:
 * TMA tile::gather4 issued by 1 thread / lane 0 of 8 warps / 32 lanes of one warp, mode 3:
 * cp.async by 8 warps, mode 4: half of each stage by gather4 and half by cp.async.  *bytes (host) = bytes moved by the launch, which the caller times on
 * `stream`; *err_dev (zeroed device int32) becomes FVGB_ETIMEOUT if a bounded wait gave up.  x
 * 128-byte aligned.  No counterpart in the reference. */
int fvgb_row_gather_probe(int32_t mode, const void *x, int64_t n_rows, const int32_t *rows, int32_t nlist,
                          int32_t iters, int32_t *err_dev, int64_t *bytes, fvgb_stream_t stream);

/* ------------------------------------------------------------------------------------------
 * Leaf-halo convolution: stride-1 3x3x3 convolution of a grid onto itself with no kernel map.
 * Offset k = 9*a + 3*b + c reads the voxel at ijk + (a-1, b-1, c-1) (the kernel map's order,
 * weight dims K2, K1, K0 on ijk axes 0, 1, 2).  dtype FVGB_F32 / FVGB_F64 / FVGB_BF16 / FVGB_F16,
 * FP32 accumulation (FP64 for FP64), CUDA cores.
 * ------------------------------------------------------------------------------------------ */
/* y [n, c_out] = sum_k x[v + d_k] . w[k], w [27, c_in, c_out].  mirror != 0: the data gradient,
 * offset k takes w[26-k]^T with w in the forward layout [27, c_out, c_in] (x = dy, y = dx).
 * Replaces stencilConvHaloKernel and the dgrad of its backward
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionHalo.cu:22-351,
 * src/fvdb/detail/autograd/SparseConvolutionHalo.cpp:17-86). */
int fvgb_halo_conv(int32_t dtype, const FvgbGrid *grid, const void *x, int64_t ldx, int32_t c_in, const void *w,
                   int32_t c_out, int32_t mirror, void *y, int64_t ldy, fvgb_stream_t stream);
/* Workspace bytes of fvgb_halo_wgrad. */
int fvgb_halo_wgrad_workspace(int32_t dtype, const FvgbGrid *grid, int32_t c_in, int32_t c_out, size_t *bytes);
/* dw [27, c_in, c_out] = sum_v x[v + d_k]^T dy[v]: per-chunk partials summed in FP64 in a fixed
 * order (deterministic).  Replaces the halo weight gradient
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionHaloGrad.cu:161-273). */
int fvgb_halo_wgrad(int32_t dtype, const FvgbGrid *grid, const void *x, int64_t ldx, int32_t c_in, const void *dy,
                    int64_t lddy, int32_t c_out, void *dw, void *workspace, size_t workspace_bytes,
                    fvgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* FVDB_GB300_H */
