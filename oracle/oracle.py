"""CPU oracle of the sparse-convolution path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this module,
and only to compare results against / as the timed CPU baseline.  The fvdb_gb300 package never
imports it.

Contents (reference paths relative to the fvdb-core tree):
  grid_from_ijk        voxel index order of BuildGridFromIjk.cu:26-83 (fvdb_oracle.c)
  kernel_map           ConvolutionKernelMap.cu:60-102 (fvdb_oracle.c)
  conv_grid            BuildGridForConv.cu:190-255 + CoarseIjkForFineGrid.cu:19-41
  points_to_ijk        BuildGridFromPoints.cu:27-43 + VoxelCoordTransform.h:86-110 (apply().round()
                       in the points' precision; fvdb_oracle.c)
  transpose_map        IGEMMBitOperations.cu:92-105
  neighbour_map        SparseConvPackInfo.cpp:61-88 (kmap.t(), nonzero, sizes)
  gs_forward/backward  the reference CPU gather -> torch::mm -> scatter path,
                       SparseConvolutionKernelMap.cu:417-615, with the weight permutes of
                       autograd/SparseConvolutionKernelMap.cpp:71-93,171-188
  conv_forward_f64 /
  conv_backward_f64    the same sums in float64 (numpy), the precision oracle
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "libfvdb_oracle.so")
        if not os.path.exists(path):
            import importlib.util

            spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(_HERE, "build.py"))
            m = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(m)
            m.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        L.orc_grid_build.restype = i64
        L.orc_grid_build.argtypes = [P, P, i32, P, P]
        L.orc_kernel_map.restype = None
        L.orc_kernel_map.argtypes = [P, P, P, P, i32, P, P, P, i64]
        L.orc_conv_grid_candidates.restype = i64
        L.orc_conv_grid_candidates.argtypes = [P, P, i32, P, P, P, P]
        L.orc_transpose_map.restype = None
        L.orc_transpose_map.argtypes = [P, i64, i64, i64, P, i64]
        for name in ("orc_points_to_ijk_f32", "orc_points_to_ijk_f64"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [P, P, i32, P, P, P]
        for name in ("orc_gather_f32", "orc_scatter_add_f32", "orc_gather_f64", "orc_scatter_add_f64"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [i64, i64, P, P, P, ctypes.c_int]
        _LIB = L
    return _LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _vec3(v) -> np.ndarray:
    if isinstance(v, int):
        v = (v, v, v)
    return np.ascontiguousarray(np.array(v, dtype=np.int32).reshape(3))


# ----------------------------------------------------------------------- integer path ---
def points_to_ijk(points: np.ndarray, joff, voxel_sizes, origins, precision: str) -> np.ndarray:
    """ijk of points as the reference voxelises them (BuildGridFromPoints.cu:27-43):
    precision "f64" for FP64 point clouds, "f32" for FP32 / FP16 / BF16 ones (values given
    as float64 arrays holding the points' exact values).  voxel_sizes / origins: [B, 3]."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    joff = np.ascontiguousarray(joff, dtype=np.int64)
    B = joff.shape[0] - 1
    vs = np.ascontiguousarray(np.broadcast_to(np.asarray(voxel_sizes, np.float64), (B, 3)))
    org = np.ascontiguousarray(np.broadcast_to(np.asarray(origins, np.float64), (B, 3)))
    out = np.empty((pts.shape[0], 3), dtype=np.int32)
    f = _lib().orc_points_to_ijk_f64 if precision == "f64" else _lib().orc_points_to_ijk_f32
    f(_p(pts), _p(joff), B, _p(vs), _p(org), _p(out))
    return out


def grid_from_ijk(ijk: np.ndarray, joff: np.ndarray):
    """(sorted unique ijk [N,3] int32, offsets [B+1] int64) in NanoVDB voxel order."""
    ijk = np.ascontiguousarray(ijk, dtype=np.int32).reshape(-1, 3)
    joff = np.ascontiguousarray(joff, dtype=np.int64)
    B = joff.size - 1
    out = np.empty((max(ijk.shape[0], 1), 3), dtype=np.int32)
    out_off = np.empty(B + 1, dtype=np.int64)
    n = _lib().orc_grid_build(_p(ijk), _p(joff), B, _p(out), _p(out_off))
    return out[:n].copy(), out_off


def kernel_map(src_ijk, src_off, tgt_ijk, tgt_off, ksize, stride) -> np.ndarray:
    """kmap [N_tgt, k0*k1*k2] int32 (-1 = absent)."""
    src_ijk = np.ascontiguousarray(src_ijk, dtype=np.int32)
    tgt_ijk = np.ascontiguousarray(tgt_ijk, dtype=np.int32)
    src_off = np.ascontiguousarray(src_off, dtype=np.int64)
    tgt_off = np.ascontiguousarray(tgt_off, dtype=np.int64)
    ks, st = _vec3(ksize), _vec3(stride)
    K = int(ks.prod())
    out = np.full((max(tgt_ijk.shape[0], 1), K), -1, dtype=np.int32)
    _lib().orc_kernel_map(_p(src_ijk), _p(src_off), _p(tgt_ijk), _p(tgt_off), src_off.size - 1, _p(ks), _p(st), _p(out), K)
    return out[: tgt_ijk.shape[0]]


def conv_grid(ijk, joff, ksize, stride):
    """Target grid of a strided convolution: (ijk sorted, offsets)."""
    ijk = np.ascontiguousarray(ijk, dtype=np.int32)
    joff = np.ascontiguousarray(joff, dtype=np.int64)
    ks, st = _vec3(ksize), _vec3(stride)
    st = np.where(st == 0, 1, st).astype(np.int32)
    cap = max(ijk.shape[0] * int(ks.prod()), 1)
    cand = np.empty((cap, 3), dtype=np.int32)
    coff = np.empty(joff.size, dtype=np.int64)
    n = _lib().orc_conv_grid_candidates(_p(ijk), _p(joff), joff.size - 1, _p(ks), _p(st), _p(cand), _p(coff))
    return grid_from_ijk(cand[:n], coff)


def transpose_map(kmap: np.ndarray, n_in: int) -> np.ndarray:
    kmap = np.ascontiguousarray(kmap, dtype=np.int32)
    K = kmap.shape[1]
    out = np.full((max(n_in, 1), K), -1, dtype=np.int32)
    _lib().orc_transpose_map(_p(kmap), kmap.shape[0], K, K, _p(out), K)
    return out[:n_in]


def neighbour_map(kmap: np.ndarray):
    """(nbmap [P,2] = (in, out) ordered by (offset, out), nbsizes [K])."""
    kt = kmap.T
    k_idx, o_idx = np.nonzero(kt >= 0)
    nbmap = np.stack([kt[k_idx, o_idx], o_idx.astype(np.int32)], 1).astype(np.int32)
    nbsizes = (kt >= 0).sum(1).astype(np.int32)
    return np.ascontiguousarray(nbmap), nbsizes


def weights_kio(weight: np.ndarray, transposed: bool) -> np.ndarray:
    """[K, Cin, Cout] view of (Do,Di,K0,K1,K2) (or (Di,Do,...) when transposed)."""
    w = np.transpose(weight, (4, 3, 2, 0, 1) if transposed else (4, 3, 2, 1, 0))
    return np.ascontiguousarray(w.reshape(-1, w.shape[3], w.shape[4]))


# ----------------------------------------------------------------------- FP64 oracle ----
def conv_forward_f64(x: np.ndarray, weight: np.ndarray, kmap: np.ndarray, transposed: bool = False, n_src=None):
    """out = sum_k x[map[:,k]] W[k] in float64.  For transposed=True, `kmap` is the
    forward map (target rows) and the output lives on the n_src source rows."""
    x = np.asarray(x, dtype=np.float64)
    W = weights_kio(np.asarray(weight, dtype=np.float64), transposed)
    m = transpose_map(kmap, int(n_src)) if transposed else kmap
    out = np.zeros((m.shape[0], W.shape[2]), dtype=np.float64)
    for k in range(W.shape[0]):
        rows = m[:, k]
        v = rows >= 0
        if v.any():
            out[v] += x[rows[v]] @ W[k]
    return out


def conv_backward_f64(x, weight, kmap, dy, transposed: bool = False, n_src=None):
    """(dx, dW[5-D, same layout as weight]) in float64."""
    x = np.asarray(x, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    W = weights_kio(np.asarray(weight, dtype=np.float64), transposed)
    m = transpose_map(kmap, int(n_src)) if transposed else kmap  # rows of dy
    dx = np.zeros_like(x)
    dW = np.zeros_like(W)
    for k in range(W.shape[0]):
        rows = m[:, k]
        v = rows >= 0
        if v.any():
            np.add.at(dx, rows[v], dy[v] @ W[k].T)
            dW[k] = x[rows[v]].T @ dy[v]
    ks = weight.shape[2:]
    dW5 = dW.reshape(ks[2], ks[1], ks[0], W.shape[1], W.shape[2])
    dW5 = np.transpose(dW5, (3, 4, 2, 1, 0) if transposed else (4, 3, 2, 1, 0))
    return dx, np.ascontiguousarray(dW5)


# ----------------------------------------------------------------------- reference CPU path
def gs_forward(x, weight, nbmap: np.ndarray, nbsizes: np.ndarray, n_out: int, transposed=False, middle=False):
    """The reference CPU gather -> torch.mm -> scatter forward (torch tensors, x's dtype).

    `middle` is the stride-1 centre-offset shortcut of SparseConvolutionKernelMap.cu:438-448
    (out = x @ W[K/2] first, then the other offsets)."""
    import torch

    L = _lib()
    dt = x.dtype
    gather = L.orc_gather_f32 if dt == torch.float32 else L.orc_gather_f64
    scatter = L.orc_scatter_add_f32 if dt == torch.float32 else L.orc_scatter_add_f64
    Wt = weight.permute(4, 3, 2, 0, 1) if transposed else weight.permute(4, 3, 2, 1, 0)
    W = Wt.reshape(-1, Wt.shape[3], Wt.shape[4]).contiguous()
    K, cin, cout = W.shape
    x = x.contiguous()
    out = torch.zeros((n_out, cout), dtype=dt)
    nbmap = np.ascontiguousarray(nbmap, dtype=np.int32)
    sizes = [int(s) for s in nbsizes]
    flag = middle and K % 2 == 1 and n_out == x.shape[0]
    if flag:
        torch.mm(x, W[K // 2], out=out)
    cap = max(max(sizes) if sizes else 1, 1)
    inb = torch.zeros((cap, cin), dtype=dt)
    outb = torch.zeros((cap, cout), dtype=dt)
    cur = 0
    gcol, scol = (1, 0) if transposed else (0, 1)
    for k in range(K):
        n = sizes[k]
        if n == 0 or (flag and k == K // 2):
            cur += n
            continue
        seg = nbmap[cur : cur + n]
        a = inb[:n]
        gather(n, cin, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(a.data_ptr()), _p(seg), gcol)
        o = outb[:n]
        torch.mm(a, W[k], out=o)
        scatter(n, cout, ctypes.c_void_p(o.data_ptr()), ctypes.c_void_p(out.data_ptr()), _p(seg), scol)
        cur += n
    return out


# ----------------------------------------------------------------------- pooling ---------
# Restatement of the reference's pooling / nearest-upsampling loops (src/fvdb/detail/ops/
# DownsampleGridMaxPool.cu:19-126, DownsampleGridAvgPool.cu:19-112,144,
# UpsampleGridNearest.cu:19-110, BuildFineGridFromCoarse.cu:66-226,
# CoarseIjkForFineGrid.cu:19-41) on numpy arrays.  Coordinates must lie in [-2048, 2048).
def _coord_keys(ijk: np.ndarray, joff) -> np.ndarray:
    ijk = np.asarray(ijk, dtype=np.int64).reshape(-1, 3)
    assert ijk.size == 0 or (ijk.min() >= -2048 and ijk.max() < 2048)
    b = np.repeat(np.arange(len(joff) - 1), np.diff(np.asarray(joff)))
    return (b << 36) | ((ijk[:, 0] + 2048) << 24) | ((ijk[:, 1] + 2048) << 12) | (ijk[:, 2] + 2048)


def _lookup(ijk: np.ndarray, joff, q_ijk: np.ndarray, q_batch: np.ndarray) -> np.ndarray:
    """Row of each query coordinate in the grid (ijk, joff), or -1."""
    keys = _coord_keys(ijk, joff)
    order = np.argsort(keys)
    sk = keys[order]
    q = np.asarray(q_ijk, dtype=np.int64)
    ok = np.all((q >= -2048) & (q < 2048), axis=1)
    qk = (q_batch.astype(np.int64) << 36) | ((q[:, 0] + 2048) << 24) | ((q[:, 1] + 2048) << 12) | (q[:, 2] + 2048)
    pos = np.searchsorted(sk, qk)
    pos = np.minimum(pos, max(sk.size - 1, 0))
    hit = ok & (sk.size > 0) & (sk[pos] == qk) if sk.size else np.zeros(qk.shape, bool)
    return np.where(hit, order[pos] if sk.size else 0, -1)


def _batch_of(joff) -> np.ndarray:
    return np.repeat(np.arange(len(joff) - 1), np.diff(np.asarray(joff)))


def coarsened_grid(ijk, joff, factor):
    """floor(ijk / factor) per grid, in index order (CoarseIjkForFineGrid.cu:19-41)."""
    f = np.asarray(_vec3(factor), dtype=np.int64)
    c = np.floor_divide(np.asarray(ijk, dtype=np.int64), f).astype(np.int32)
    return grid_from_ijk(c, np.asarray(joff))


def subdivided_grid(ijk, joff, factor, mask=None):
    """Every (masked) voxel c split into c*factor + (i,j,k) (BuildFineGridFromCoarse.cu:66-226)."""
    f = _vec3(factor).astype(np.int64)
    ijk = np.asarray(ijk, dtype=np.int64)
    keep = np.ones(ijk.shape[0], bool) if mask is None else np.asarray(mask, bool)
    off = np.stack(np.meshgrid(np.arange(f[0]), np.arange(f[1]), np.arange(f[2]), indexing="ij"), -1).reshape(-1, 3)
    parts, counts = [], []
    for b in range(len(joff) - 1):
        sel = ijk[joff[b]:joff[b + 1]][keep[joff[b]:joff[b + 1]]]
        ch = (sel[:, None, :] * f + off[None]).reshape(-1, 3)
        parts.append(ch)
        counts.append(ch.shape[0])
    cand = np.concatenate(parts).astype(np.int32) if parts else np.zeros((0, 3), np.int32)
    return grid_from_ijk(cand, np.concatenate([[0], np.cumsum(counts)]).astype(np.int64))


def _windows(base: np.ndarray, ext):
    for i in range(ext[0]):
        for j in range(ext[1]):
            for k in range(ext[2]):
                yield base + np.array([i, j, k], dtype=np.int64)


def pool_forward(fine_ijk, fine_off, coarse_ijk, coarse_off, x: np.ndarray, pool, stride, mode: str) -> np.ndarray:
    """mode "max": max over the window's active fine voxels (-inf when none); "avg": window sum
    in x's precision (window order i-outer, k-inner) times (1 / pool volume) in that precision."""
    p, s = _vec3(pool).astype(np.int64), _vec3(stride).astype(np.int64)
    s = np.where(s == 0, p, s)
    base = np.asarray(coarse_ijk, dtype=np.int64) * s
    cb = _batch_of(coarse_off)
    dt = x.dtype
    acc = np.full((base.shape[0], x.shape[1]), -np.inf if mode == "max" else 0.0, dtype=dt)
    for q in _windows(base, p):
        r = _lookup(fine_ijk, fine_off, q, cb)
        v = r >= 0
        if mode == "max":
            acc[v] = np.fmax(x[r[v]], acc[v])
        else:
            acc[v] = acc[v] + x[r[v]]
    if mode == "avg":
        acc = acc * dt.type(1.0 / float(np.prod(p)))
    return acc


def pool_backward(fine_ijk, fine_off, coarse_ijk, coarse_off, x: np.ndarray, dy: np.ndarray, pool, stride,
                  mode: str) -> np.ndarray:
    """Max: each window's gradient goes to its first strict maximum; average: dy * (1 / volume)
    to every active voxel of the window (DownsampleGridMaxPool.cu:71-126, DownsampleGridAvgPool.cu:68-112)."""
    p, s = _vec3(pool).astype(np.int64), _vec3(stride).astype(np.int64)
    s = np.where(s == 0, p, s)
    base = np.asarray(coarse_ijk, dtype=np.int64) * s
    cb = _batch_of(coarse_off)
    dx = np.zeros_like(x)
    if mode == "max":
        best = np.full(dy.shape, -np.inf, dtype=x.dtype)
        arg = np.full(dy.shape, -1, dtype=np.int64)
        for q in _windows(base, p):
            r = _lookup(fine_ijk, fine_off, q, cb)
            v = r >= 0
            vals = np.where(v[:, None], x[np.maximum(r, 0)], -np.inf)
            upd = vals > best
            best = np.where(upd, vals, best)
            arg = np.where(upd, r[:, None], arg)
        rows, cols = np.nonzero(arg >= 0)
        np.add.at(dx, (arg[rows, cols], cols), dy[rows, cols])
        return dx
    g = dy * dy.dtype.type(1.0 / float(np.prod(p)))
    for q in _windows(base, p):
        r = _lookup(fine_ijk, fine_off, q, cb)
        v = r >= 0
        np.add.at(dx, r[v], g[v])
    return dx


def upsample_forward(coarse_ijk, coarse_off, fine_ijk, fine_off, x: np.ndarray, factor) -> np.ndarray:
    """Fine voxel f takes coarse voxel floor(f / factor) (zero without one)."""
    f = _vec3(factor).astype(np.int64)
    par = np.floor_divide(np.asarray(fine_ijk, dtype=np.int64), f)
    r = _lookup(coarse_ijk, coarse_off, par, _batch_of(fine_off))
    out = np.zeros((par.shape[0], x.shape[1]), dtype=x.dtype)
    out[r >= 0] = x[r[r >= 0]]
    return out


def upsample_backward(coarse_ijk, coarse_off, fine_ijk, fine_off, dy: np.ndarray, factor) -> np.ndarray:
    """Coarse voxel c sums the gradients of its children c*factor + (i,j,k) in window order."""
    f = _vec3(factor).astype(np.int64)
    base = np.asarray(coarse_ijk, dtype=np.int64) * f
    cb = _batch_of(coarse_off)
    dx = np.zeros((base.shape[0], dy.shape[1]), dtype=dy.dtype)
    for q in _windows(base, f):
        r = _lookup(fine_ijk, fine_off, q, cb)
        v = r >= 0
        dx[v] = dx[v] + dy[r[v]]
    return dx
