"""CPU oracle of the sparse-convolution path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this module,
and only as the checker / the timed CPU baseline.  The fvdb_gb300 package never imports it.

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
