/*
 * CPU oracle for the sparse-convolution index path.  TEST INFRASTRUCTURE ONLY:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library, and only to compare results against.  The product never links or calls it.
 *
 * It restates, in plain C, the integer algorithms of fVDB 0.2.1 (reference paths
 * relative to the fvdb-core source tree):
 *
 *   - voxel index order of a NanoVDB OnIndex grid built from ijk
 *       src/fvdb/detail/ops/BuildGridFromIjk.cu:26-83 (CUDA, nanovdb voxelsToGrid)
 *       src/fvdb/detail/utils/nanovdb/ActiveVoxelIterator.h:109-125 (leaf order)
 *       src/fvdb/detail/ops/PopulateGridMetadata.cu:39-90 (per-grid voxel offsets)
 *     NanoVDB (OpenVDB commit 5f0432b3, not vendored) numbers the voxels of an
 *     OnIndex tree in depth-first node order: root tiles by key, then upper-node
 *     child bit (x,y,z bits 11..7), lower-node child bit (bits 6..3), leaf bit
 *     (bits 2..0).  The root key of the CUDA builder is
 *     (uint32(x)>>12)<<42 | (uint32(y)>>12)<<21 | (uint32(z)>>12), sorted as an
 *     unsigned integer; this file follows that (GPU) order.
 *   - the kernel map  src/fvdb/detail/ops/convolution/pack_info/ConvolutionKernelMap.cu:60-102
 *   - conv_grid       src/fvdb/detail/ops/BuildGridForConv.cu:25-64,190-255
 *                     src/fvdb/detail/ops/CoarseIjkForFineGrid.cu:19-41
 *   - ijk of points   src/fvdb/detail/ops/BuildGridFromPoints.cu:27-43 with
 *                     VoxelCoordTransform::apply(...).round()
 *                     (src/fvdb/detail/VoxelCoordTransform.h:86-110,230-330)
 *
 * Parity of raw map integers against the reference's NanoVDB build is pinned only
 * within one root tile (all coordinates in [0,4096)^3); across root tiles it
 * follows the order stated above.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef struct {
    uint64_t hi;  /* root-tile key */
    uint64_t lo;  /* upper(15) | lower(12) | leaf(9) child offsets */
    int64_t src;  /* position in the caller's input (for stable tie handling) */
    int32_t x, y, z;
} orc_rec;

static uint64_t root_key(int32_t x, int32_t y, int32_t z) {
    /* NanoVDB RootNode::CoordToKey with 21 bits per axis (nanovdb/NanoVDB.h). */
    return ((uint64_t)((uint32_t)x >> 12) << 42) | ((uint64_t)((uint32_t)y >> 12) << 21) |
           (uint64_t)((uint32_t)z >> 12);
}

static uint64_t inner_key(int32_t x, int32_t y, int32_t z) {
    /* UpperNode::CoordToOffset (LOG2DIM 5), LowerNode (LOG2DIM 4), LeafNode (LOG2DIM 3). */
    uint64_t up = ((uint64_t)((x & 4095) >> 7) << 10) | ((uint64_t)((y & 4095) >> 7) << 5) |
                  (uint64_t)((z & 4095) >> 7);
    uint64_t lw = ((uint64_t)((x & 127) >> 3) << 8) | ((uint64_t)((y & 127) >> 3) << 4) |
                  (uint64_t)((z & 127) >> 3);
    uint64_t lf = ((uint64_t)(x & 7) << 6) | ((uint64_t)(y & 7) << 3) | (uint64_t)(z & 7);
    return (up << 21) | (lw << 9) | lf;
}

static int cmp_rec(const void *a, const void *b) {
    const orc_rec *p = (const orc_rec *)a, *q = (const orc_rec *)b;
    if (p->hi != q->hi) return p->hi < q->hi ? -1 : 1;
    if (p->lo != q->lo) return p->lo < q->lo ? -1 : 1;
    if (p->src != q->src) return p->src < q->src ? -1 : 1;
    return 0;
}

/*
 * Build a batch of index grids from jagged ijk.  Duplicates collapse to one voxel.
 * out_ijk must hold joff[B] rows; out_joff has B+1 entries.  Returns the number of
 * unique voxels.  (BuildGridFromIjk.cu:157-207: one grid per batch item, merged in
 * batch order; voxel offsets are the running sum of per-grid counts.)
 */
int64_t orc_grid_build(const int32_t *ijk, const int64_t *joff, int32_t B, int32_t *out_ijk,
                       int64_t *out_joff) {
    int64_t total = 0;
    out_joff[0] = 0;
    for (int32_t b = 0; b < B; ++b) {
        int64_t s = joff[b], e = joff[b + 1], n = e - s;
        orc_rec *r = (orc_rec *)malloc(sizeof(orc_rec) * (size_t)(n > 0 ? n : 1));
        for (int64_t i = 0; i < n; ++i) {
            int32_t x = ijk[3 * (s + i)], y = ijk[3 * (s + i) + 1], z = ijk[3 * (s + i) + 2];
            r[i].hi = root_key(x, y, z);
            r[i].lo = inner_key(x, y, z);
            r[i].src = i;
            r[i].x = x; r[i].y = y; r[i].z = z;
        }
        qsort(r, (size_t)n, sizeof(orc_rec), cmp_rec);
        for (int64_t i = 0; i < n; ++i) {
            if (i > 0 && r[i].hi == r[i - 1].hi && r[i].lo == r[i - 1].lo) continue;
            out_ijk[3 * total] = r[i].x;
            out_ijk[3 * total + 1] = r[i].y;
            out_ijk[3 * total + 2] = r[i].z;
            ++total;
        }
        out_joff[b + 1] = total;
        free(r);
    }
    return total;
}

/* Rank of (x,y,z) inside the sorted voxels [s,e) of one grid, or -1 (NanoVDB isActive/getValue-1). */
static int64_t find_voxel(const uint64_t *hi, const uint64_t *lo, int64_t s, int64_t e, int32_t x,
                          int32_t y, int32_t z) {
    uint64_t h = root_key(x, y, z), l = inner_key(x, y, z);
    int64_t a = s, b = e;
    while (a < b) {
        int64_t m = a + (b - a) / 2;
        if (hi[m] < h || (hi[m] == h && lo[m] < l)) a = m + 1; else b = m;
    }
    if (a < e && hi[a] == h && lo[a] == l) return a;
    return -1;
}

static void keys_of(const int32_t *ijk, int64_t n, uint64_t *hi, uint64_t *lo) {
    for (int64_t i = 0; i < n; ++i) {
        hi[i] = root_key(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
        lo[i] = inner_key(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
    }
}

/*
 * Kernel map, ConvolutionKernelMap.cu:60-102.  ksize/stride are the user's
 * (k0,k1,k2)/(s0,s1,s2); the reference applies stride s2 and kernel extent k2 to
 * ijk axis 0, and k0/s0 to ijk axis 2 (":37-38,43-47").  Both grids must be in
 * index order (as produced by orc_grid_build).  kmap is [n_tgt, k0*k1*k2] row major
 * with leading dimension ld; every entry of the valid rows is written.
 */
void orc_kernel_map(const int32_t *src_ijk, const int64_t *src_joff, const int32_t *tgt_ijk,
                    const int64_t *tgt_joff, int32_t B, const int32_t *ksize, const int32_t *stride,
                    int32_t *kmap, int64_t ld) {
    const int64_t ns = src_joff[B];
    uint64_t *hi = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(ns > 0 ? ns : 1));
    uint64_t *lo = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(ns > 0 ? ns : 1));
    keys_of(src_ijk, ns, hi, lo);
    /* kernelStart = floor(-K/2 + 1) per component (":66-68") */
    int32_t st[3];
    for (int a = 0; a < 3; ++a) st[a] = (int32_t)floor(-ksize[a] / 2.0 + 1.0);
    for (int32_t b = 0; b < B; ++b) {
        for (int64_t t = tgt_joff[b]; t < tgt_joff[b + 1]; ++t) {
            int32_t sx = tgt_ijk[3 * t] * stride[2];
            int32_t sy = tgt_ijk[3 * t + 1] * stride[1];
            int32_t sz = tgt_ijk[3 * t + 2] * stride[0];
            int64_t k = 0;
            for (int32_t kz = st[2]; kz < st[2] + ksize[2]; ++kz)
                for (int32_t ky = st[1]; ky < st[1] + ksize[1]; ++ky)
                    for (int32_t kx = st[0]; kx < st[0] + ksize[0]; ++kx, ++k) {
                        int64_t r = find_voxel(hi, lo, src_joff[b], src_joff[b + 1], sx + kz,
                                               sy + ky, sz + kx);
                        kmap[t * ld + k] = (int32_t)r;
                    }
        }
    }
    free(hi);
    free(lo);
}

static int32_t floordiv(int32_t a, int32_t b) {
    /* (Vec3d(ijk) / Vec3d(f)).floor() of CoarseIjkForFineGrid.cu:34-35 for integer inputs */
    return (int32_t)floor((double)a / (double)b);
}

/*
 * Candidate target coordinates of conv_grid(kernel, stride) before de-duplication
 * (BuildGridForConv.cu:66-124 and CoarseIjkForFineGrid.cu:19-41).  Writes at most
 * n_src*k0*k1*k2 rows into out_ijk with per-grid offsets out_joff; returns the count.
 * The caller then builds the grid (orc_grid_build) from these coordinates.
 */
int64_t orc_conv_grid_candidates(const int32_t *ijk, const int64_t *joff, int32_t B,
                                 const int32_t *ksize, const int32_t *stride, int32_t *out_ijk,
                                 int64_t *out_joff) {
    int64_t n = 0;
    out_joff[0] = 0;
    int coarse = (stride[0] == 1 && stride[1] == 1 && stride[2] == 1) ||
                 (stride[0] == ksize[0] && stride[1] == ksize[1] && stride[2] == ksize[2]);
    int32_t lower[3], upper[3];
    for (int a = 0; a < 3; ++a) {
        if (ksize[a] % 2 == 0) { lower[a] = 0; upper[a] = ksize[a] - 1; }
        else { lower[a] = -(ksize[a] - 1) / 2; upper[a] = (ksize[a] - 1) / 2; }
    }
    for (int32_t b = 0; b < B; ++b) {
        for (int64_t v = joff[b]; v < joff[b + 1]; ++v) {
            int32_t x = ijk[3 * v], y = ijk[3 * v + 1], z = ijk[3 * v + 2];
            if (coarse) {
                /* the coarsening factor is the stride Coord itself, x <-> s0 */
                out_ijk[3 * n] = floordiv(x, stride[0]);
                out_ijk[3 * n + 1] = floordiv(y, stride[1]);
                out_ijk[3 * n + 2] = floordiv(z, stride[2]);
                ++n;
                continue;
            }
            for (int32_t di = lower[0]; di <= upper[0]; ++di)
                for (int32_t dj = lower[1]; dj <= upper[1]; ++dj)
                    for (int32_t dk = lower[2]; dk <= upper[2]; ++dk) {
                        int32_t dx = x + dk, dy = y + dj, dz = z + di;
                        /* C remainder semantics, as in the reference */
                        if (dx % stride[2] != 0 || dy % stride[1] != 0 || dz % stride[0] != 0)
                            continue;
                        out_ijk[3 * n] = dx / stride[2];
                        out_ijk[3 * n + 1] = dy / stride[1];
                        out_ijk[3 * n + 2] = dz / stride[0];
                        ++n;
                    }
        }
        out_joff[b + 1] = n;
    }
    return n;
}

/* Transposed map (IGEMMBitOperations.cu:92-105): mapT[in][k] = out.  mapT pre-filled with -1. */
void orc_transpose_map(const int32_t *kmap, int64_t n_out, int64_t K, int64_t ld, int32_t *mapT,
                       int64_t ldT) {
    for (int64_t o = 0; o < n_out; ++o)
        for (int64_t k = 0; k < K; ++k) {
            int32_t i = kmap[o * ld + k];
            if (i >= 0) mapT[(int64_t)i * ldT + k] = (int32_t)o;
        }
}

/*
 * Gather / scatter-add loops of the reference CPU gather-scatter convolution
 * (src/fvdb/detail/ops/convolution/backend/SparseConvolutionKernelMap.cu:60-100): serial
 * loops over the neighbour pairs, one row of c channels each.  `col` picks the column of
 * the [P,2] neighbour map that indexes the dense side (0 = input row, 1 = output row).
 */
void orc_gather_f32(int64_t n, int64_t c, const float *src, float *buf, const int32_t *nbmap, int col) {
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = nbmap[2 * i + col];
        if (r < 0) continue;
        memcpy(buf + i * c, src + (int64_t)r * c, sizeof(float) * (size_t)c);
    }
}

void orc_scatter_add_f32(int64_t n, int64_t c, const float *buf, float *dst, const int32_t *nbmap, int col) {
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = nbmap[2 * i + col];
        if (r < 0) continue;
        float *d = dst + (int64_t)r * c;
        const float *s = buf + i * c;
        for (int64_t j = 0; j < c; ++j) d[j] += s[j];
    }
}

void orc_gather_f64(int64_t n, int64_t c, const double *src, double *buf, const int32_t *nbmap, int col) {
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = nbmap[2 * i + col];
        if (r < 0) continue;
        memcpy(buf + i * c, src + (int64_t)r * c, sizeof(double) * (size_t)c);
    }
}

void orc_scatter_add_f64(int64_t n, int64_t c, const double *buf, double *dst, const int32_t *nbmap, int col) {
    for (int64_t i = 0; i < n; ++i) {
        int32_t r = nbmap[2 * i + col];
        if (r < 0) continue;
        double *d = dst + (int64_t)r * c;
        const double *s = buf + i * c;
        for (int64_t j = 0; j < c; ++j) d[j] += s[j];
    }
}

/*
 * ijk of points (BuildGridFromPoints.cu:27-43): per axis VoxelCoordTransform(1/w, -o/w)
 * .apply(p).round() in the points' arithmetic type (opmath_type: double for double points,
 * float otherwise).  The transform's float copy holds (float)(1/w) and (float)(-o/w)
 * (VoxelCoordTransform.h:230-240); apply() is p*scale + translate, which nvcc contracts to
 * one fused multiply-add; NanoVDB's Vec3::round() is Floor(v + 0.5) in the same type.
 * points are given as double; the f32 variant first rounds each to float (exact for points
 * that are float, half or bfloat16 values).
 */
void orc_points_to_ijk_f32(const double *pts, const int64_t *joff, int32_t B, const double *vs,
                           const double *org, int32_t *out) {
    for (int32_t b = 0; b < B; ++b)
        for (int64_t i = joff[b]; i < joff[b + 1]; ++i)
            for (int a = 0; a < 3; ++a) {
                const float s = (float)(1.0 / vs[3 * b + a]);
                const float t = (float)(-org[3 * b + a] / vs[3 * b + a]);
                const float v = fmaf((float)pts[3 * i + a], s, t);
                out[3 * i + a] = (int32_t)floorf(v + 0.5f);
            }
}

void orc_points_to_ijk_f64(const double *pts, const int64_t *joff, int32_t B, const double *vs,
                           const double *org, int32_t *out) {
    for (int32_t b = 0; b < B; ++b)
        for (int64_t i = joff[b]; i < joff[b + 1]; ++i)
            for (int a = 0; a < 3; ++a) {
                const double s = 1.0 / vs[3 * b + a];
                const double t = -org[3 * b + a] / vs[3 * b + a];
                const double v = fma(pts[3 * i + a], s, t);
                out[3 * i + a] = (int32_t)floor(v + 0.5);
            }
}
