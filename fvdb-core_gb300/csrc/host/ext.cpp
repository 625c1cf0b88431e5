// Host side of fvdb_gb300: the C++ PyTorch extension `fvdb._C`.
//
// It mirrors the reference's L2/L3 layers for the convolution path:
//   GridImpl      <-> fvdb::detail::GridBatchImpl (src/fvdb/detail/GridBatchImpl.h)
//   PackInfo      <-> fvdb::SparseConvPackInfo    (src/fvdb/SparseConvPackInfo.{h,cpp})
//   conv_forward / conv_backward <-> the forward/backward bodies of
//                     fvdb::detail::autograd::SparseConvolutionKernelMap / ImplicitGEMM
//                     (src/fvdb/detail/autograd/SparseConvolution*.cpp); the autograd
//                     Function itself is fvdb/_conv.py
// Torch owns every buffer; all device work goes through the C ABI of libfvdb_gb300.so on the
// current torch stream.  Errors map to ValueError / TypeError / RuntimeError exactly where the
// reference uses TORCH_CHECK_VALUE / TORCH_CHECK_TYPE / TORCH_CHECK.
#include <ATen/cuda/CUDAContext.h>
#include <ATen/cuda/CUDAEvent.h>
#include <c10/cuda/CUDAGuard.h>
#include <torch/extension.h>

#include <atomic>
#include <list>
#include <map>
#include <mutex>
#include <optional>
#include <string>
#include <vector>

#include "../../../include/fvdb_gb300.h"

namespace fvgbh {

using torch::Tensor;

inline fvgb_stream_t cur_stream() { return (fvgb_stream_t)at::cuda::getCurrentCUDAStream().stream(); }

void check_status(int st, const char *what) {
    if (st == FVGB_OK) return;
    std::string msg = std::string(what) + " failed";
    if (st == FVGB_ECUDA) msg += std::string(": ") + fvgb_last_error();
    switch (st) {
        case FVGB_EINVAL: TORCH_CHECK_VALUE(false, msg, " (invalid argument)");
        case FVGB_ERANGE: TORCH_CHECK_VALUE(false, msg, " (coordinate outside [-2^20, 2^20))");
        case FVGB_ETYPE: TORCH_CHECK_TYPE(false, msg, " (unsupported dtype)");
        case FVGB_ETIMEOUT: TORCH_CHECK(false, msg, " (device wait timed out)");
        case FVGB_ENOSPACE: TORCH_CHECK(false, msg, " (workspace too small)");
        default: TORCH_CHECK(false, msg);
    }
}

Tensor workspace(size_t bytes, const torch::Device &dev) {
    return torch::empty({(int64_t)std::max<size_t>(bytes, 256)}, torch::dtype(torch::kUInt8).device(dev));
}

// Pinned host staging for the small device-to-host reads of grid builds (per host thread and
// device, grown on demand): one async copy and one stream sync instead of a torch gather +
// copy.  Per thread, so grid builds of concurrent serving slots never share it.
int64_t *pinned_meta(int dev, size_t count) {
    thread_local std::vector<std::pair<int64_t *, size_t>> bufs(64, {nullptr, 0});
    auto &b = bufs.at(dev);
    if (b.second < count) {
        if (b.first) cudaFreeHost(b.first);
        const size_t cap = std::max<size_t>(count, 512);
        void *p = nullptr;
        TORCH_CHECK(cudaHostAlloc(&p, cap * sizeof(int64_t), cudaHostAllocDefault) == cudaSuccess,
                    "pinned staging allocation failed");
        b = {reinterpret_cast<int64_t *>(p), cap};
    }
    return b.first;
}

int64_t next_pow2(int64_t v) {
    int64_t p = 64;
    while (p < v) p <<= 1;
    return p;
}

struct Vec3 {
    int32_t v[3];
};

Vec3 to_vec3(const std::vector<int64_t> &x, const char *name) {
    TORCH_CHECK_VALUE(x.size() == 3 || x.size() == 1, name, " must have 1 or 3 entries");
    Vec3 r;
    for (int a = 0; a < 3; ++a) r.v[a] = (int32_t)(x.size() == 1 ? x[0] : x[a]);
    return r;
}

// Element type code of a feature or point tensor.
int32_t fvgb_dtype(const Tensor &t) {
    switch (t.scalar_type()) {
        case torch::kFloat32: return FVGB_F32;
        case torch::kFloat64: return FVGB_F64;
        case torch::kBFloat16: return FVGB_BF16;
        case torch::kFloat16: return FVGB_F16;
        default: TORCH_CHECK_TYPE(false, "unsupported feature dtype ", t.scalar_type());
    }
    return -1;
}

// ------------------------------------------------------------------------------------------
struct GridImpl {
    int64_t B = 0, N = 0, L = 0, cap = 0;
    Tensor joffsets;       // int64 [B+1] device
    Tensor joffsets_host;  // int64 [B+1] cpu
    Tensor ijk;            // int32 [N,3] device
    Tensor leaves;         // uint8 [L*128] device
    Tensor hash;           // int32 [cap] device
    Tensor voxel_sizes;    // float64 [B,3] cpu
    Tensor origins;        // float64 [B,3] cpu
    Tensor jidx_cache;
    int32_t box_lo[3] = {0, 0, 0}, box_hi[3] = {-1, -1, -1};  // bounding box of ijk (empty if N == 0)
    // recorded on the building stream after the last kernel of the build: work on another stream
    // that reads the grid waits for this, not for everything queued after it
    std::shared_ptr<at::cuda::CUDAEvent> ready;

    // A grid whose counts are still on their way to the host (a coarse grid built on the build
    // stream): the build is enqueued and resolve() completes the grid at its first use, so the
    // caller's stream can be fed meanwhile (e.g. the next layer's convolution).  Until then N and
    // L are -1, and every accessor of the counts, tensors or view resolves first.
    struct PendingBuild {
        at::cuda::CUDAEvent counted;  // on the build stream, after the counts' copy to the host
        Tensor meta_host;             // pinned int64 [B + 4]
        Tensor out_ijk, leaf_ids, meta;
        // the counts' copy into meta_host must land before the pinned block can be reused
        ~PendingBuild() {
            try {
                counted.synchronize();
            } catch (...) {
            }
        }
    };
    std::unique_ptr<PendingBuild> pending;
    std::atomic<bool> is_pending{false};
    std::mutex resolve_mu;
    void resolve() const;

    FvgbGrid view() const {
        resolve();
        return view_unchecked();
    }
    FvgbGrid view_unchecked() const {
        FvgbGrid g;
        g.num_grids = (int32_t)B;
        g.reserved = 0;
        g.num_voxels = N;
        g.num_leaves = L;
        g.hash_capacity = cap;
        g.voxel_offsets = joffsets.data_ptr<int64_t>();
        g.ijk = N > 0 ? ijk.data_ptr<int32_t>() : nullptr;
        g.leaves = L > 0 ? reinterpret_cast<const FvgbLeaf *>(leaves.data_ptr<uint8_t>()) : nullptr;
        g.hash_slots = cap > 0 ? hash.data_ptr<int32_t>() : nullptr;
        return g;
    }
    torch::Device device() const { return joffsets.device(); }
};
using GridPtr = std::shared_ptr<GridImpl>;

const GridPtr &R(const GridPtr &g) {
    if (g) g->resolve();
    return g;
}

Tensor per_grid_vec(const Tensor &t, int64_t B, const char *name) {
    Tensor v = t.to(torch::kFloat64).cpu();
    if (v.dim() == 0) v = v.reshape({1, 1}).expand({B, 3});
    else if (v.dim() == 1) v = v.reshape({1, -1}).expand({B, 3});
    TORCH_CHECK_VALUE(v.dim() == 2 && v.size(0) == B && v.size(1) == 3, name, " must broadcast to [", B, ", 3]");
    return v.contiguous().clone();
}

// Sorted-unique voxels in index order + leaf table + hash (one host sync for the counts and the
// bounding box).  box_lo/box_hi (optional): bounds the caller knows for ijk, which shorten the
// sort to the order-key bits that can differ.
GridPtr build_grid(const Tensor &ijk_in, const Tensor &joff_in, const Tensor &vs, const Tensor &org,
                   const int32_t *box_lo = nullptr, const int32_t *box_hi = nullptr) {
    TORCH_CHECK(ijk_in.is_cuda(), "fvdb_gb300 grids live on CUDA devices");
    c10::cuda::CUDAGuard guard(ijk_in.device());
    auto dev = ijk_in.device();
    TORCH_CHECK_VALUE(ijk_in.dim() == 2 && ijk_in.size(1) == 3, "ijk must have shape (N, 3)");
    TORCH_CHECK_TYPE(!ijk_in.is_floating_point(), "ijk must have an integer dtype");
    Tensor ijk = ijk_in.to(torch::kInt32).contiguous();
    Tensor joff = joff_in.to(dev, torch::kInt64).contiguous();
    const int64_t B = joff.size(0) - 1;
    TORCH_CHECK_VALUE(B >= 1, "a grid batch needs at least one grid");
    const int64_t n = ijk.size(0);
    auto g = std::make_shared<GridImpl>();
    g->B = B;
    g->voxel_sizes = per_grid_vec(vs, B, "voxel_sizes");
    g->origins = per_grid_vec(org, B, "origins");
    auto i32 = torch::dtype(torch::kInt32).device(dev);
    // Large inputs without known bounds: read their bounding box first (one small reduction and
    // one read) so the radix sort covers only the order-key bits that vary (3 of 8 passes for
    // coordinates in [0, 256)^3).  Small inputs sort the full key instead of paying the read.
    int32_t mlo[3], mhi[3];
    if (!(box_lo && box_hi) && n >= (int64_t)1 << 18) {
        Tensor bx = torch::cat({std::get<0>(ijk.min(0)), std::get<0>(ijk.max(0))}).to(torch::kInt64);
        int64_t *hb = pinned_meta(dev.index(), 6);
        cudaStream_t cs = reinterpret_cast<cudaStream_t>(cur_stream());
        TORCH_CHECK(cudaMemcpyAsync(hb, bx.data_ptr<int64_t>(), 6 * sizeof(int64_t), cudaMemcpyDeviceToHost, cs) ==
                            cudaSuccess &&
                        cudaStreamSynchronize(cs) == cudaSuccess,
                    "grid build: reading the bounds failed");
        for (int a = 0; a < 3; ++a) {
            mlo[a] = (int32_t)hb[a];
            mhi[a] = (int32_t)hb[3 + a];
        }
        box_lo = mlo;
        box_hi = mhi;
    }
    Tensor out_ijk = torch::empty({std::max<int64_t>(n, 1), 3}, i32);
    // device metadata read back in one copy: [0, B] voxel offsets, B+1 leaf count, B+2 voxel
    // count, B+3 error word (the sort's int32 flag in its low half; zero-initialised), then the
    // measured bounding box (lo xyz, hi xyz) when the caller gave none
    const int64_t n_meta = B + 4 + ((box_lo && box_hi) ? 0 : 6);
    Tensor meta = torch::zeros({n_meta}, torch::dtype(torch::kInt64).device(dev));
    Tensor out_joff = meta.narrow(0, 0, B + 1);
    int32_t *err_ptr = reinterpret_cast<int32_t *>(meta.data_ptr<int64_t>() + B + 3);
    static_assert(sizeof(void *) == 8, "64-bit host");
    size_t wsb = 0;
    check_status(fvgb_ijk_sort_unique_workspace(n, (int32_t)B, &wsb), "grid build (workspace)");
    Tensor ws = workspace(wsb, dev);
    auto s = cur_stream();
    if (box_lo && box_hi)
        check_status(fvgb_ijk_sort_unique_in_box(n ? ijk.data_ptr<int32_t>() : nullptr, joff.data_ptr<int64_t>(),
                                                 (int32_t)B, n, box_lo, box_hi, out_ijk.data_ptr<int32_t>(),
                                                 out_joff.data_ptr<int64_t>(), err_ptr, ws.data_ptr(), ws.numel(), s),
                     "grid build (sort)");
    else
        check_status(fvgb_ijk_sort_unique(n ? ijk.data_ptr<int32_t>() : nullptr, joff.data_ptr<int64_t>(), (int32_t)B,
                                          n, out_ijk.data_ptr<int32_t>(), out_joff.data_ptr<int64_t>(), err_ptr,
                                          ws.data_ptr(), ws.numel(), s),
                     "grid build (sort)");
    // leaf ids over the capacity n (the unique count stays on the device), so the unique count,
    // the leaf count and the range check come back to the host in one copy
    Tensor leaf_ids = torch::empty({std::max<int64_t>(n, 1)}, i32);
    size_t sb = 0;
    check_status(fvgb_scan_workspace(n, &sb), "grid build (scan workspace)");
    // the sort's workspace is free again: reuse it for the leaf scan when large enough
    Tensor ws2 = sb <= (size_t)ws.numel() ? ws : workspace(sb, dev);
    check_status(fvgb_grid_leaf_scan(n ? out_ijk.data_ptr<int32_t>() : nullptr, out_joff.data_ptr<int64_t>(), (int32_t)B,
                                     n, leaf_ids.data_ptr<int32_t>(), meta.data_ptr<int64_t>() + B + 1, ws2.data_ptr(),
                                     ws2.numel(), s),
                 "grid build (leaf scan)");
    if (!(box_lo && box_hi) && n > 0)  // the bounding box of the input is that of the unique voxels
        meta.narrow(0, B + 4, 6).copy_(torch::cat({std::get<0>(ijk.min(0)), std::get<0>(ijk.max(0))}));
    int64_t *h = pinned_meta(dev.index(), (size_t)n_meta);
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(s);
    TORCH_CHECK(cudaMemcpyAsync(h, meta.data_ptr<int64_t>(), n_meta * sizeof(int64_t), cudaMemcpyDeviceToHost, cs) ==
                        cudaSuccess &&
                    cudaStreamSynchronize(cs) == cudaSuccess,
                "grid build: reading the counts failed");
    TORCH_CHECK_VALUE(h[B + 3] == 0, box_lo ? "voxel coordinates must lie in [-2^20, 2^20) and inside their bounds"
                                            : "voxel coordinates must lie in [-2^20, 2^20)");
    for (int a = 0; a < 3; ++a) {
        if (box_lo && box_hi) {
            g->box_lo[a] = box_lo[a];
            g->box_hi[a] = box_hi[a];
        } else if (n > 0) {
            g->box_lo[a] = (int32_t)h[B + 4 + a];
            g->box_hi[a] = (int32_t)h[B + 7 + a];
        }
    }
    g->joffsets_host = torch::from_blob(h, {B + 1}, torch::kInt64).clone();
    g->joffsets = out_joff;
    g->N = h[B];
    g->ijk = out_ijk.narrow(0, 0, g->N);
    g->L = h[B + 1];
    g->cap = next_pow2(2 * g->L);
    g->leaves = torch::empty({std::max<int64_t>(g->L, 1) * (int64_t)sizeof(FvgbLeaf)}, torch::dtype(torch::kUInt8).device(dev));
    g->hash = torch::empty({g->cap}, i32);
    FvgbGrid v = g->view();
    check_status(fvgb_grid_index_build(&v, leaf_ids.data_ptr<int32_t>(), s), "grid build (index)");
    g->ready = std::make_shared<at::cuda::CUDAEvent>();
    g->ready->record(at::cuda::getCurrentCUDAStream(dev.index()));
    return g;
}

GridPtr grid_from_ijk(const Tensor &ijk, const Tensor &joffsets, const Tensor &vs, const Tensor &org) {
    return build_grid(ijk, joffsets, vs, org);
}

GridPtr grid_from_points(const Tensor &points, const Tensor &joffsets, const Tensor &vs, const Tensor &org) {
    TORCH_CHECK(points.is_cuda(), "fvdb_gb300 grids live on CUDA devices");
    c10::cuda::CUDAGuard guard(points.device());
    TORCH_CHECK_VALUE(points.dim() == 2 && points.size(1) == 3, "points must have shape (N, 3)");
    TORCH_CHECK_TYPE(points.is_floating_point(), "points must have a floating point dtype");
    const int64_t B = joffsets.size(0) - 1;
    // voxelised in the points' own precision (FP64 in double, the rest in float), as the reference
    Tensor p = points.contiguous();
    Tensor joff = joffsets.to(points.device(), torch::kInt64).contiguous();
    Tensor vsb = per_grid_vec(vs, B, "voxel_sizes"), orb = per_grid_vec(org, B, "origins");
    Tensor vsd = vsb.to(points.device()), ord = orb.to(points.device());
    Tensor ijk = torch::empty({p.size(0), 3}, torch::dtype(torch::kInt32).device(points.device()));
    check_status(fvgb_points_to_ijk(fvgb_dtype(p), p.data_ptr(), joff.data_ptr<int64_t>(), (int32_t)B, p.size(0),
                                    vsd.data_ptr<double>(), ord.data_ptr<double>(), ijk.data_ptr<int32_t>(),
                                    cur_stream()),
                 "points to ijk");
    return build_grid(ijk, joff, vsb, orb);
}

// Coarse grid floor(ijk / f) of a grid, built leaf by leaf (fvgb_coarse_grid_build: one sort
// key per fine leaf instead of one per voxel; the same voxels in the same order as sorting the
// coarsened voxels).  f per axis in {1, 2, 4, 8}; lo/hi: bounds of the coarse voxels.
// A high-priority stream of the library's own per device, for builds whose counts the host must
// read: the host then waits for the build alone, not for the convolutions queued on the caller's
// stream before it, and the build's small CTAs are scheduled into the room the running
// persistent convolution CTAs leave on each SM instead of queueing behind them.
c10::cuda::CUDAStream build_stream(c10::DeviceIndex dev) {
    static std::mutex mu;
    static std::map<int, c10::cuda::CUDAStream> streams;
    std::lock_guard<std::mutex> lock(mu);
    auto it = streams.find(dev);
    if (it == streams.end()) it = streams.emplace(dev, c10::cuda::getStreamFromPool(true, dev)).first;
    return it->second;
}

GridPtr build_coarse_by_leaves(const GridPtr &g, const Vec3 &f, const int32_t lo[3], const int32_t hi[3]) {
    auto dev = g->device();
    const int64_t B = g->B;
    auto c = std::make_shared<GridImpl>();
    c->B = B;
    c->voxel_sizes = g->voxel_sizes.clone();
    c->origins = g->origins.clone();
    for (int a = 0; a < 3; ++a) {
        c->box_lo[a] = lo[a];
        c->box_hi[a] = hi[a];
    }
    auto i32 = torch::dtype(torch::kInt32).device(dev);
    // The build runs on the library's build stream once the fine grid is complete (its ready
    // event), so it does not wait for work queued on the caller's stream (e.g. the previous
    // step's convolutions); the host reads its counts only when the coarse grid is first used.
    // Buffers are allocated for the build stream and handed to the caller's stream.
    auto main = at::cuda::getCurrentCUDAStream(dev.index());
    auto side = build_stream(dev.index());
    if (g->ready) g->ready->block(side);
    else {
        at::cuda::CUDAEvent e;
        e.record(main);
        e.block(side);
    }
    auto pb = std::make_unique<GridImpl::PendingBuild>();
    pb->meta_host = torch::empty({B + 4}, torch::dtype(torch::kInt64).pinned_memory(true));
    {
        c10::cuda::CUDAStreamGuard sg(side);
        pb->out_ijk = torch::empty({std::max<int64_t>(g->N, 1), 3}, i32);
        pb->leaf_ids = torch::empty({std::max<int64_t>(g->N, 1)}, i32);
        pb->meta = torch::zeros({B + 4}, torch::dtype(torch::kInt64).device(dev));
        size_t wsb = 0;
        check_status(fvgb_coarse_grid_workspace(g->L, &wsb), "coarse grid (workspace)");
        Tensor ws = workspace(wsb, dev);
        FvgbGrid fv = g->view();
        cudaStream_t cs = side.stream();
        check_status(fvgb_coarse_grid_build(&fv, f.v, lo, hi, pb->out_ijk.data_ptr<int32_t>(),
                                            pb->meta.data_ptr<int64_t>(), pb->leaf_ids.data_ptr<int32_t>(),
                                            ws.data_ptr(), ws.numel(), cs),
                     "coarse grid");
        TORCH_CHECK(cudaMemcpyAsync(pb->meta_host.data_ptr<int64_t>(), pb->meta.data_ptr<int64_t>(),
                                    (B + 4) * sizeof(int64_t), cudaMemcpyDeviceToHost, cs) == cudaSuccess,
                    "coarse grid: copying the counts failed");
        pb->counted.record(side);
    }
    // the buffers live on in the caller's stream
    pb->out_ijk.record_stream(main);
    pb->leaf_ids.record_stream(main);
    pb->meta.record_stream(main);
    c->joffsets = pb->meta.narrow(0, 0, B + 1);  // the device, for guards; values after resolve()
    c->N = -1;
    c->L = -1;
    c->pending = std::move(pb);
    c->is_pending.store(true, std::memory_order_release);
    return c;
}

void GridImpl::resolve() const {
    if (!is_pending.load(std::memory_order_acquire)) return;
    auto *self = const_cast<GridImpl *>(this);  // grids are created non-const; resolving fills them in
    std::lock_guard<std::mutex> lock(self->resolve_mu);
    if (!self->is_pending.load(std::memory_order_acquire)) return;
    PendingBuild &P = *self->pending;
    const auto dev = P.meta.device();
    c10::cuda::CUDAGuard guard(dev);
    P.counted.synchronize();  // the host waits for the coarse build alone
    const int64_t *h = P.meta_host.data_ptr<int64_t>();
    self->joffsets_host = P.meta_host.narrow(0, 0, B + 1).clone();
    self->joffsets = P.meta.narrow(0, 0, B + 1);
    self->N = h[B + 2];
    self->L = h[B + 1];
    self->ijk = P.out_ijk.narrow(0, 0, self->N);
    self->cap = next_pow2(2 * self->L);
    auto main = at::cuda::getCurrentCUDAStream(dev.index());
    P.counted.block(main);  // the index build follows the coarse build on the device
    auto i32 = torch::dtype(torch::kInt32).device(dev);
    self->leaves = torch::empty({std::max<int64_t>(self->L, 1) * (int64_t)sizeof(FvgbLeaf)},
                                torch::dtype(torch::kUInt8).device(dev));
    self->hash = torch::empty({self->cap}, i32);
    FvgbGrid v = self->view_unchecked();
    check_status(fvgb_grid_index_build(&v, P.leaf_ids.data_ptr<int32_t>(), main.stream()), "coarse grid (index)");
    self->ready = std::make_shared<at::cuda::CUDAEvent>();
    self->ready->record(main);
    self->pending.reset();
    self->is_pending.store(false, std::memory_order_release);
}

// conv_grid: output voxel set of a (strided) convolution (BuildGridForConv.cu:181-255).
GridPtr grid_conv_grid(const GridPtr &g, const std::vector<int64_t> &ks_in, const std::vector<int64_t> &st_in) {
    R(g);
    c10::cuda::CUDAGuard guard(g->device());
    Vec3 ks = to_vec3(ks_in, "kernel_size"), st = to_vec3(st_in, "stride");
    for (int a = 0; a < 3; ++a) {
        TORCH_CHECK_VALUE(ks.v[a] > 0, "kernel_size must be positive");
        TORCH_CHECK_VALUE(st.v[a] >= 0, "stride must be non-negative");
    }
    // stride 0 (the Python default) behaves as 1
    for (int a = 0; a < 3; ++a)
        if (st.v[a] == 0) st.v[a] = 1;
    auto dev = g->device();
    const bool coarse = (st.v[0] == 1 && st.v[1] == 1 && st.v[2] == 1) ||
                        (st.v[0] == ks.v[0] && st.v[1] == ks.v[1] && st.v[2] == ks.v[2]);
    auto fdiv = [](int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
    // the coarse path with power-of-two strides <= 8: built leaf by leaf
    bool pow2 = coarse && g->N > 0 && g->L > 0 && g->B <= 1024;
    for (int a = 0; a < 3; ++a) {
        const int v = st.v[a];
        pow2 = pow2 && (v == 1 || v == 2 || v == 4 || v == 8);
    }
    if (pow2 && !(st.v[0] == 1 && st.v[1] == 1 && st.v[2] == 1)) {
        int32_t lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = (int32_t)fdiv(g->box_lo[a], st.v[a]);
            hi[a] = (int32_t)fdiv(g->box_hi[a], st.v[a]);
        }
        return build_coarse_by_leaves(g, st, lo, hi);
    }
    const int64_t kc = coarse ? 1 : (int64_t)ks.v[0] * ks.v[1] * ks.v[2];
    const int64_t n = g->N * kc;
    auto i32 = torch::dtype(torch::kInt32).device(dev);
    Tensor cand = torch::empty({std::max<int64_t>(n, 1), 3}, i32);
    Tensor valid = torch::empty({std::max<int64_t>(n, 1)}, torch::dtype(torch::kUInt8).device(dev));
    FvgbGrid v = g->view();
    auto s = cur_stream();
    check_status(fvgb_conv_grid_candidates(&v, ks.v, st.v, cand.data_ptr<int32_t>(), valid.data_ptr<uint8_t>(), s),
                 "conv_grid (candidates)");
    Tensor ijk, joff;
    if (coarse) {
        ijk = cand.narrow(0, 0, n);
        joff = g->joffsets;
    } else {
        Tensor out = torch::empty({std::max<int64_t>(n, 1), 3}, i32);
        joff = torch::empty({g->B + 1}, torch::dtype(torch::kInt64).device(dev));
        size_t sb = 0;
        check_status(fvgb_scan_workspace(n, &sb), "conv_grid (workspace)");
        Tensor ws = workspace(sb, dev);
        check_status(fvgb_compact_ijk(cand.data_ptr<int32_t>(), valid.data_ptr<uint8_t>(), g->joffsets.data_ptr<int64_t>(),
                                      (int32_t)g->B, kc, n, out.data_ptr<int32_t>(), joff.data_ptr<int64_t>(),
                                      ws.data_ptr(), ws.numel(), s),
                     "conv_grid (compact)");
        const int64_t m = joff[g->B].item<int64_t>();
        ijk = out.narrow(0, 0, m);
    }
    // bounds of the candidates from the source grid's bounding box: floor(ijk/s) per axis on the
    // coarse path; (ijk + offset)/s over the footprint otherwise (k0 and s0 act on axis 2)
    if (g->N == 0) return build_grid(ijk, joff, g->voxel_sizes, g->origins);
    int32_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        if (coarse) {
            lo[a] = (int32_t)fdiv(g->box_lo[a], st.v[a]);
            hi[a] = (int32_t)fdiv(g->box_hi[a], st.v[a]);
        } else {
            const int64_t k = ks.v[2 - a], s = st.v[2 - a];
            const int64_t dlo = k % 2 == 0 ? 0 : -(k - 1) / 2, dhi = k % 2 == 0 ? k - 1 : (k - 1) / 2;
            lo[a] = (int32_t)fdiv(g->box_lo[a] + dlo, s);
            hi[a] = (int32_t)fdiv(g->box_hi[a] + dhi, s);
        }
    }
    return build_grid(ijk, joff, g->voxel_sizes, g->origins, lo, hi);
}

Tensor grid_ijk_to_index(const GridPtr &g, const Tensor &ijk_in, const Tensor &joff_in, bool cumulative) {
    R(g);
    c10::cuda::CUDAGuard guard(g->device());
    TORCH_CHECK_VALUE(ijk_in.dim() == 2 && ijk_in.size(1) == 3, "ijk must have shape (N, 3)");
    Tensor q = ijk_in.to(g->device(), torch::kInt32).contiguous();
    Tensor qo = joff_in.to(g->device(), torch::kInt64).contiguous();
    TORCH_CHECK_VALUE(qo.size(0) == g->B + 1, "ijk must have one list per grid");
    Tensor out = torch::empty({q.size(0)}, torch::dtype(torch::kInt64).device(g->device()));
    FvgbGrid v = g->view();
    check_status(fvgb_ijk_to_index(&v, q.data_ptr<int32_t>(), qo.data_ptr<int64_t>(), q.size(0), cumulative ? 1 : 0,
                                   out.data_ptr<int64_t>(), cur_stream()),
                 "ijk_to_index");
    return out;
}

Tensor grid_jidx(const GridPtr &g) {
    R(g);
    if (!g->jidx_cache.defined()) {
        Tensor counts = (g->joffsets_host.narrow(0, 1, g->B) - g->joffsets_host.narrow(0, 0, g->B));
        g->jidx_cache = torch::repeat_interleave(torch::arange(g->B, torch::kInt32), counts).to(g->device());
    }
    return g->jidx_cache;
}

// ------------------------------------------------------------------------------------------
// Map tensors of one (kernel, stride, source, target) -- SparseConvPackInfo.
struct PackInfo {
    Vec3 ks, st;
    GridPtr src, tgt;
    int32_t K = 0;
    std::optional<Tensor> out_in_map;      // [ceil(N_tgt/128)*128, K]
    std::optional<Tensor> out_in_map_bwd;  // [ceil(N_src/128)*128, K]
    std::optional<Tensor> nbmap, nbsizes;  // GS form
    std::optional<Tensor> tile_mask, tile_mask_t;  // OR of row occupancy per 128-row tile (K <= 32)
    std::optional<Tensor> reorder_loc, sorted_mask, reorder_out_in_map, reduced_sorted_mask;
    std::optional<Tensor> reorder_loc_bwd, reorder_out_in_map_bwd, sorted_mask_bwd_w, sorted_mask_bwd_d;
    bool use_me = false, use_tf32 = false;
    std::optional<bool> gs_use_me;
    int64_t split_mask_num = 1;
    bool training_built = false;
    // tile plans of the forward (0) / transposed (1) map per feature row size in bytes, and how
    // often each was asked for
    std::map<std::pair<int, int32_t>, Tensor> plans;
    std::map<std::pair<int, int32_t>, int> plan_requests;
    // contraction row order of the forward (0) / transposed (1) map: rows sorted by occupancy
    // mask (padded with -1), the map's rows in that order and the per-tile masks of that order;
    // and how often a tensor-core contraction asked for it
    std::optional<Tensor> order_rows[2], order_mask[2], order_map[2];
    int order_requests[2] = {0, 0};
};
using PackPtr = std::shared_ptr<PackInfo>;

void resolve_pack(const PackPtr &p) {
    if (!p) return;
    R(p->src);
    R(p->tgt);
}

PackPtr make_pack(const std::vector<int64_t> &ks_in, const std::vector<int64_t> &st_in, const GridPtr &src,
                  const std::optional<GridPtr> &tgt) {
    R(src);
    if (tgt) R(*tgt);
    auto p = std::make_shared<PackInfo>();
    p->ks = to_vec3(ks_in, "kernel_size");
    p->st = to_vec3(st_in, "stride");
    for (int a = 0; a < 3; ++a) {
        TORCH_CHECK(p->ks.v[a] > 0, "Expect kernel size to be larger than {0,0,0}");
        TORCH_CHECK(p->st.v[a] > 0, "Expect stride to be larger than 0");
    }
    const bool unit_stride = p->st.v[0] == 1 && p->st.v[1] == 1 && p->st.v[2] == 1;
    const bool unit_kernel = p->ks.v[0] == 1 && p->ks.v[1] == 1 && p->ks.v[2] == 1;
    p->src = src;
    if (tgt.has_value()) p->tgt = *tgt;
    else if (unit_stride) p->tgt = src;
    else p->tgt = grid_conv_grid(src, ks_in, st_in);
    TORCH_CHECK(p->src->device() == p->tgt->device(), "Source and target grids must both be on the same device");
    TORCH_CHECK(!(unit_kernel && unit_stride), "1x1 conv does not need kernel map to be built!");
    p->K = p->ks.v[0] * p->ks.v[1] * p->ks.v[2];
    return p;
}

// Kernel map [ceil(N_tgt/128)*128, K] (padding rows -1); for K <= 32 the per-128-row-tile
// occupancy masks come out of the same pass into *tile_mask.
Tensor build_kmap(const GridPtr &src, const GridPtr &tgt, const Vec3 &ks, const Vec3 &st, int32_t K,
                  Tensor *tile_mask = nullptr) {
    c10::cuda::CUDAGuard guard(tgt->device());
    TORCH_CHECK_VALUE(src->B == tgt->B, "source and target grids must have the same grid count");
    const int64_t npad = (tgt->N + 127) / 128 * 128;
    Tensor kmap = torch::empty({npad, K}, torch::dtype(torch::kInt32).device(tgt->device()));
    if (npad > tgt->N) kmap.narrow(0, tgt->N, npad - tgt->N).fill_(-1);
    uint32_t *tm = nullptr;
    if (tile_mask && K <= 32) {
        *tile_mask = torch::zeros({std::max<int64_t>(npad / 128, 1)}, kmap.options());
        tm = reinterpret_cast<uint32_t *>(tile_mask->data_ptr<int32_t>());
    }
    FvgbGrid s = src->view(), t = tgt->view();
    check_status(fvgb_kmap_build(&s, &t, ks.v, st.v, kmap.data_ptr<int32_t>(), K, nullptr, tm, cur_stream()),
                 "kernel map build");
    return kmap;
}

const Tensor &pack_kmap(PackPtr p) {
    resolve_pack(p);
    if (!p->out_in_map) {
        Tensor tm;
        p->out_in_map = build_kmap(p->src, p->tgt, p->ks, p->st, p->K, &tm);
        if (tm.defined()) p->tile_mask = tm;
    }
    return *p->out_in_map;
}

const Tensor &pack_kmap_t(PackPtr p) {
    resolve_pack(p);
    if (!p->out_in_map_bwd) {
        const Tensor &m = pack_kmap(p);
        const int64_t npad = (p->src->N + 127) / 128 * 128;
        Tensor t = torch::empty({npad, p->K}, m.options());
        check_status(fvgb_kmap_transpose(m.data_ptr<int32_t>(), p->tgt->N, p->K, p->K, t.data_ptr<int32_t>(), npad,
                                         p->K, cur_stream()),
                     "kernel map transpose");
        p->out_in_map_bwd = t;
    }
    return *p->out_in_map_bwd;
}

Tensor tile_masks_of(const Tensor &map, int64_t n_rows, int32_t K) {
    const int64_t tiles = (n_rows + 127) / 128;
    Tensor m = torch::zeros({std::max<int64_t>(tiles, 1)}, map.options());
    if (n_rows > 0)
        check_status(fvgb_kmap_masks(map.data_ptr<int32_t>(), n_rows, K, K, nullptr,
                                     reinterpret_cast<uint32_t *>(m.data_ptr<int32_t>()), cur_stream()),
                     "kernel map tile masks");
    return m;
}

// Per-tile occupancy of the forward map (transposed=false) or of the transposed map.
std::optional<Tensor> pack_tile_mask(PackPtr p, bool transposed) {
    resolve_pack(p);
    if (p->K > 32) return std::nullopt;
    if (!transposed) {
        if (!p->tile_mask) p->tile_mask = tile_masks_of(pack_kmap(p), p->tgt->N, p->K);
        return p->tile_mask;
    }
    if (!p->tile_mask_t) p->tile_mask_t = tile_masks_of(pack_kmap_t(p), p->src->N, p->K);
    return p->tile_mask_t;
}

// Whether a contraction may run over a tile plan (fvgb_conv_fwd_tc_planned) instead of over the
// map directly (fvgb_conv_fwd_tc_bias).  A reused map with 4 <= K <= 32 runs over its row order
// instead (faster still), so plans serve the small kernels (K < 4) only.  Measured on GB300 (1.08M surface voxels, 3x3x3): the
// planned kernel is faster for rows shorter than 128 bytes (32->64 BF16: 0.31 vs 0.37 ms) and
// slower for 128-byte rows (64->64 BF16: 0.73 vs 0.6 ms), where assembling the A operand in
// tensor memory costs more than the gathers it saves; so plans serve short rows only.
bool use_plan(int32_t dtype, int64_t K, int64_t cin, int64_t cout, int64_t elem) {
    return cin * elem < 128 && fvgb_tc_plan_supported(dtype, (int32_t)K, (int32_t)cin, (int32_t)cout) == FVGB_OK;
}

std::optional<Tensor> pack_plan(PackPtr p, bool transposed, int32_t row_bytes);

// Row order of a map for the contractions (fvgb_kmap_row_order): rows sorted by occupancy mask so
// that a 128-row tile's rows share their offsets and the per-tile mask skips more of the
// reduction (3x3x3 on the C2 sphere shells: 25.2 -> 16.9 active offsets per tile; a stride-2
// transposed map, one valid offset of 8 per row: 8 -> ~1).  Built once per pack and direction,
// for 4 <= K <= 32: {rows, tile masks, the map in that order}.
struct RowOrder {
    Tensor rows, mask, map;
};

std::optional<RowOrder> pack_row_order(PackPtr p, bool transposed) {
    resolve_pack(p);
    if (p->K < 4 || p->K > 32) return std::nullopt;
    const int d = transposed ? 1 : 0;
    if (!p->order_rows[d]) {
        const Tensor &m = transposed ? pack_kmap_t(p) : pack_kmap(p);
        const int64_t n = transposed ? p->src->N : p->tgt->N;
        const int64_t tiles = std::max<int64_t>((n + 127) / 128, 1);
        Tensor rows = torch::empty({tiles * 128}, m.options());
        Tensor tmask = torch::zeros({tiles}, m.options());
        Tensor smap = torch::empty({tiles * 128, (int64_t)p->K}, m.options());
        size_t wsb = 0;
        check_status(fvgb_kmap_row_order_workspace(n, p->K, &wsb), "row order workspace");
        Tensor ws = workspace(wsb, m.device());
        check_status(fvgb_kmap_row_order(m.data_ptr<int32_t>(), n, p->K, m.stride(0), rows.data_ptr<int32_t>(),
                                         reinterpret_cast<uint32_t *>(tmask.data_ptr<int32_t>()),
                                         smap.data_ptr<int32_t>(), ws.data_ptr(), ws.numel(), cur_stream()),
                     "row order");
        p->order_rows[d] = rows;
        p->order_mask[d] = tmask;
        p->order_map[d] = smap;
    }
    return RowOrder{*p->order_rows[d], *p->order_mask[d], *p->order_map[d]};
}

// The row order for a tensor-core contraction once it is worth building: building it costs about
// 0.19 ms for 1.08M rows x 27 (a sort and a permuted copy of the map), so the first tensor-core
// contraction over a map runs in index order and the order serves the second and later ones
// (training re-uses every map for forward and data gradient).  The CUDA-core forms use the order
// from the first call on large maps: it saves them far more than it costs (C2 layer 1 FP32:
// 3.1 -> 2.0 ms).
std::optional<RowOrder> pack_row_order_if_reused(PackPtr p, bool transposed) {
    const int d = transposed ? 1 : 0;
    if (!p->order_rows[d] && ++p->order_requests[d] < 2) return std::nullopt;
    return pack_row_order(p, transposed);
}

// The plan of a map and row size once it is worth building: building one costs about 0.7x a
// contraction over the map (0.26 ms for 1.08M rows x 27), and a contraction over it saves about
// 0.2x, so the first contraction on a (map, row size) runs unplanned and the plan is built at the
// second and reused by every later one (layers that share a kernel map, training iterations on a
// cached map).
std::optional<Tensor> pack_plan_if_reused(PackPtr p, bool transposed, int32_t row_bytes) {
    const auto key = std::make_pair(transposed ? 1 : 0, row_bytes);
    if (p->plans.count(key)) return p->plans[key];
    if (++p->plan_requests[key] < 2) return std::nullopt;
    return pack_plan(p, transposed, row_bytes);
}

// Tile plan (staging schedule of the planned tensor-core kernel) of the forward map
// (transposed=false) or of the transposed map, for feature rows of row_bytes bytes; built once
// per pack and row size.  nullopt where the planned kernel does not take the shape.
std::optional<Tensor> pack_plan(PackPtr p, bool transposed, int32_t row_bytes) {
    resolve_pack(p);
    if (p->K > 32) return std::nullopt;
    const auto key = std::make_pair(transposed ? 1 : 0, row_bytes);
    auto it = p->plans.find(key);
    if (it != p->plans.end()) return it->second;
    const Tensor &m = transposed ? pack_kmap_t(p) : pack_kmap(p);
    const int64_t n = transposed ? p->src->N : p->tgt->N;
    size_t bytes = 0;
    if (fvgb_tc_plan_bytes(n, p->K, row_bytes, &bytes) != FVGB_OK) return std::nullopt;
    Tensor plan = torch::empty({(int64_t)std::max<size_t>(bytes, 16)}, m.options().dtype(torch::kUInt8));
    check_status(fvgb_tc_plan_build(m.data_ptr<int32_t>(), n, p->K, row_bytes, plan.data_ptr(), (size_t)plan.numel(),
                                    cur_stream()),
                 "tile plan build");
    p->plans[key] = plan;
    return plan;
}

void pack_build_gather_scatter(PackPtr p, bool use_me) {
    resolve_pack(p);
    if (p->nbmap && p->nbsizes) {
        TORCH_CHECK(p->gs_use_me.value_or(use_me) == use_me, "Gather scatter is already built with different use_me value");
        return;
    }
    c10::cuda::CUDAGuard guard(p->tgt->device());
    const Tensor &m = pack_kmap(p);
    const int64_t n_out = p->tgt->N;
    auto dev = m.device();
    Tensor nboff = torch::empty({p->K + 1}, torch::dtype(torch::kInt64).device(dev));
    size_t wsb = 0;
    check_status(fvgb_nbmap_workspace(n_out, p->K, &wsb), "nbmap workspace");
    Tensor ws = workspace(wsb, dev);
    // the pair count is needed to size nbmap: count first, then write
    Tensor counts = (m.narrow(0, 0, n_out) >= 0).sum(0, false, torch::kInt64);
    const int64_t P = counts.sum().item<int64_t>();
    Tensor nbmap = torch::empty({std::max<int64_t>(P, 1), 2}, torch::dtype(torch::kInt32).device(dev));
    check_status(fvgb_nbmap_build(m.data_ptr<int32_t>(), n_out, p->K, p->K, nbmap.data_ptr<int32_t>(),
                                  nboff.data_ptr<int64_t>(), ws.data_ptr(), ws.numel(), cur_stream()),
                 "nbmap build");
    p->nbmap = nbmap.narrow(0, 0, P);
    p->nbsizes = counts.to(torch::kInt32);
    p->gs_use_me = use_me;
    p->use_me = use_me;
}

// Row masks, descending sort and tile-reduced masks for the sorted implicit-GEMM tensors
// (SparseConvPackInfo.cpp:110-147); computed with torch ops for the drop-in properties.
void sorted_tensors(const Tensor &map, int64_t n_valid, int64_t split, Tensor &sorted_mask, Tensor &reorder_loc,
                    Tensor &reordered) {
    const int64_t K = map.size(1), npad = map.size(0);
    const int64_t len = (K + split - 1) / split;
    std::vector<Tensor> masks;
    Tensor valid = (map >= 0).to(torch::kInt32);
    for (int64_t sidx = 0; sidx < split; ++sidx) {
        const int64_t l = sidx == split - 1 ? K - sidx * len : len;
        Tensor w = torch::pow(2, torch::arange(l, map.options().dtype(torch::kInt64))).to(torch::kInt32);
        Tensor mk = (valid.narrow(1, sidx * len, l) * w).sum(1, false, torch::kInt32);
        if (n_valid < npad) mk.narrow(0, n_valid, npad - n_valid).zero_();
        masks.push_back(mk);
    }
    Tensor bitmask = torch::stack(masks, 0);
    auto r = torch::sort(bitmask, -1, true);
    sorted_mask = std::get<0>(r);
    reorder_loc = std::get<1>(r).to(torch::kInt32);
    std::vector<Tensor> cols;
    for (int64_t k = 0; k < K; ++k) {
        Tensor loc = reorder_loc[k / len].to(torch::kInt64);
        cols.push_back(map.select(1, k).index_select(0, loc));
    }
    reordered = torch::stack(cols, 1).contiguous();
}

Tensor reduce_mask(const Tensor &sorted_mask, int64_t tile) {
    const int64_t S = sorted_mask.size(0), n = sorted_mask.size(1);
    const int64_t nt = (n + tile - 1) / tile;
    Tensor padded = torch::zeros({S, nt * tile}, sorted_mask.options());
    padded.narrow(1, 0, n).copy_(sorted_mask);
    Tensor r = padded.view({S, nt, tile});
    Tensor out = r.select(2, 0).clone();
    for (int64_t i = 1; i < tile; ++i) out.bitwise_or_(r.select(2, i));
    return out;
}

void pack_build_implicit_gemm(PackPtr p, bool sorted, int64_t split, bool training, int64_t split_bwd, bool tf32) {
    resolve_pack(p);
    if (p->reorder_loc && sorted)
        TORCH_CHECK(p->reorder_loc->size(0) == split, "Implicit GEMM is already built with different splitMaskNum value");
    c10::cuda::CUDAGuard guard(p->tgt->device());
    const Tensor &m = pack_kmap(p);
    p->use_tf32 = tf32;
    p->split_mask_num = split;
    if (sorted && !p->reorder_loc) {
        Tensor sm, rl, ro;
        sorted_tensors(m, p->tgt->N, split, sm, rl, ro);
        p->sorted_mask = sm;
        p->reorder_loc = rl;
        p->reorder_out_in_map = ro;
        p->reduced_sorted_mask = reduce_mask(sm, 128);
    }
    if (training && !p->training_built) {
        const Tensor &mt = pack_kmap_t(p);
        Tensor sm, rl, ro;
        sorted_tensors(mt, p->src->N, split_bwd, sm, rl, ro);
        p->reorder_loc_bwd = rl;
        p->reorder_out_in_map_bwd = ro;
        p->sorted_mask_bwd_w = reduce_mask(sm, 64);
        p->sorted_mask_bwd_d = reduce_mask(sm, 128);
        p->training_built = true;
    }
}

// ------------------------------------------------------------------------------------------
// Contractions.  W is viewed as [K, Cin, Cout] (any strides).

// Device flag that the tensor-core kernels raise when a bounded wait gives up: one per (device,
// CUDA stream), so a timeout is reported to the work of the stream it happened on (serving slots
// run on streams of their own).
Tensor &device_error_flag(const torch::Device &dev) {
    static std::mutex mu;
    static std::map<std::pair<int, uintptr_t>, Tensor> flags;
    const uintptr_t stream = reinterpret_cast<uintptr_t>(at::cuda::getCurrentCUDAStream(dev.index()).stream());
    std::lock_guard<std::mutex> lock(mu);
    Tensor &f = flags[{(int)dev.index(), stream}];
    if (!f.defined()) f = torch::zeros({1}, torch::dtype(torch::kInt32).device(dev));
    return f;
}

// Raises if a tensor-core kernel on the current stream of `dev` reported a timeout
// (synchronises with that stream's work).
void check_device_errors(const torch::Device &dev) {
    Tensor &f = device_error_flag(dev);
    const int v = f.item<int>();
    if (v != 0) {
        f.zero_();
        check_status(v, "tensor-core sparse convolution");
    }
}

// Shapes the tcgen05 contraction takes: 32-byte multiples of K per MMA, and rows shorter than
// one 128-byte swizzle row must tile it (c_in 16 or 32 for bf16; any multiple of 16 from 64).
bool use_tensor_cores(const Tensor &x, int64_t cin, int64_t cout) {
    const int64_t row = cin * 2;
    return x.scalar_type() == torch::kBFloat16 && row % 32 == 0 && (row >= 128 || 128 % row == 0) && cout <= 256 &&
           x.stride(0) % 8 == 0;
}

// Derived weight tensors, cached per source tensor: the [K, Cin, Cout] view / copy of a 5-D
// weight (reshaping a permuted weight copies it) and the packed tensor-core image of a
// [K, Cin, Cout] weight.  An entry is valid while its source tensor's storage is alive and its
// version counter unchanged (an in-place update, e.g. an optimizer step, makes a new entry), so
// repeated convolutions with the same weights (inference, layers of a serving stack) skip the
// copy and the packing launch.
struct DerivedKey {
    const void *storage;
    int64_t offset;
    std::vector<int64_t> sizes, strides;
    c10::ScalarType dtype;
    int64_t version;
    int tag;  // what is derived: 0/1 = [K, Cin, Cout] (not transposed / transposed), 2/3 = packed (W / W^T)
    bool operator==(const DerivedKey &o) const {
        return storage == o.storage && offset == o.offset && sizes == o.sizes && strides == o.strides &&
               dtype == o.dtype && version == o.version && tag == o.tag;
    }
};
struct DerivedEntry {
    DerivedKey key;
    c10::weak_intrusive_ptr<c10::StorageImpl> alive;
    Tensor value;
};

DerivedKey derived_key(const Tensor &t, int tag) {
    return DerivedKey{t.storage().unsafeGetStorageImpl(), t.storage_offset(), t.sizes().vec(), t.strides().vec(),
                      t.scalar_type(), (int64_t)t.unsafeGetTensorImpl()->version_counter().current_version(), tag};
}

std::mutex g_derived_mu;
std::list<DerivedEntry> g_derived;  // most recently used first
constexpr size_t kDerivedMax = 64;

std::optional<Tensor> derived_get(const Tensor &src, int tag) {
    const DerivedKey k = derived_key(src, tag);
    std::lock_guard<std::mutex> lock(g_derived_mu);
    for (auto it = g_derived.begin(); it != g_derived.end();) {
        auto live = it->alive.lock();
        if (!live) {  // the source storage is gone: drop the entry
            it = g_derived.erase(it);
            continue;
        }
        if (it->key == k && live.get() == src.storage().unsafeGetStorageImpl()) {
            g_derived.splice(g_derived.begin(), g_derived, it);
            return g_derived.front().value;
        }
        ++it;
    }
    return std::nullopt;
}

void derived_put(const Tensor &src, int tag, const Tensor &value) {
    DerivedEntry e{derived_key(src, tag), c10::weak_intrusive_ptr<c10::StorageImpl>(src.storage().getWeakStorageImpl()),
                   value};
    std::lock_guard<std::mutex> lock(g_derived_mu);
    // an older version of the same source is stale for good: drop it
    g_derived.remove_if([&](const DerivedEntry &o) {
        return o.key.storage == e.key.storage && o.key.offset == e.key.offset && o.key.tag == e.key.tag;
    });
    g_derived.push_front(std::move(e));
    while (g_derived.size() > kDerivedMax) g_derived.pop_back();
}

// y[m] = sum_k x[map[m,k]] W[k]   for the first n_out rows of map
// bias (optional, [cout]): added in the tensor-core epilogue, else after the contraction.
// pack / map_t (optional): the pack info that owns `map` and whether `map` is its transposed map;
// with them, shapes the planned kernel takes run over the pack's cached tile plan.
Tensor gather_gemm(const Tensor &x, const Tensor &map, int64_t n_out, const Tensor &Wkio, bool transpose_w,
                   const std::optional<Tensor> &tile_mask = std::nullopt,
                   const std::optional<Tensor> &bias = std::nullopt, PackPtr pack = nullptr, bool map_t = false,
                   bool relu = false, const std::optional<Tensor> &out_scale = std::nullopt) {
    c10::cuda::CUDAGuard guard(x.device());
    const int64_t K = map.size(1);
    const int64_t cin = transpose_w ? Wkio.size(2) : Wkio.size(1);
    const int64_t cout = transpose_w ? Wkio.size(1) : Wkio.size(2);
    TORCH_CHECK_VALUE(x.size(1) == cin, "channel mismatch");
    Tensor y = torch::empty({n_out, cout}, x.options());
    if (n_out == 0) return y;
    Tensor w = Wkio.to(x.scalar_type());
    const int64_t wsk = w.stride(0), wsci = transpose_w ? w.stride(2) : w.stride(1), wsco = transpose_w ? w.stride(1) : w.stride(2);
    const int32_t dt = fvgb_dtype(x);
    auto s = cur_stream();
    if (use_tensor_cores(x, cin, cout)) {
        const int tag = transpose_w ? 3 : 2;
        std::optional<Tensor> cached = derived_get(Wkio, tag);
        Tensor packed;
        if (cached && cached->device() == x.device()) {
            packed = *cached;
        } else {
            size_t wb = 0;
            check_status(fvgb_tc_weight_bytes(FVGB_BF16, K, (int32_t)cin, (int32_t)cout, &wb), "weight pack size");
            packed = torch::empty({(int64_t)wb}, torch::dtype(torch::kUInt8).device(x.device()));
            check_status(fvgb_tc_pack_weights(FVGB_BF16, w.data_ptr(), K, (int32_t)cin, (int32_t)cout, wsk, wsci,
                                              wsco, packed.data_ptr(), wb, s),
                         "weight pack");
            if (Wkio.scalar_type() == torch::kBFloat16) derived_put(Wkio, tag, packed);
        }
        const uint32_t *tm = tile_mask ? reinterpret_cast<const uint32_t *>(tile_mask->data_ptr<int32_t>()) : nullptr;
        Tensor b32, s32;
        if (bias) b32 = bias->to(torch::kFloat32).contiguous();
        if (out_scale) s32 = out_scale->to(torch::kFloat32).contiguous();
        const float *sp = out_scale ? s32.data_ptr<float>() : nullptr;
        // a map used again runs over its row order (measured faster than a tile plan: C2 layer 1,
        // 32->64: 0.30 ms ordered, 0.32 ms planned, 0.365 ms in index order); the tile plan serves
        // maps that have no row order (K < 4 or K > 32)
        const auto order = pack ? pack_row_order_if_reused(pack, map_t) : std::nullopt;
        std::optional<Tensor> plan;
        if (pack && K < 4 && use_plan(FVGB_BF16, K, cin, cout, 2))
            plan = pack_plan_if_reused(pack, map_t, (int32_t)(cin * 2));
        if (order) {
            check_status(fvgb_conv_fwd_tc_rows(FVGB_BF16, x.data_ptr(), x.size(0), (int32_t)cin, x.stride(0),
                                               order->map.data_ptr<int32_t>(), n_out, (int32_t)K,
                                               order->rows.data_ptr<int32_t>(),
                                               reinterpret_cast<const uint32_t *>(order->mask.data_ptr<int32_t>()),
                                               packed.data_ptr(), (int32_t)cout, y.data_ptr(), y.stride(0), sp,
                                               bias ? b32.data_ptr<float>() : nullptr, relu ? 1 : 0,
                                               device_error_flag(x.device()).data_ptr<int32_t>(), s),
                         "sparse conv forward (tensor cores)");
            return y;
        }
        if (plan) {
            check_status(fvgb_conv_fwd_tc_planned(FVGB_BF16, x.data_ptr(), x.size(0), (int32_t)cin, x.stride(0),
                                                  plan->data_ptr(), n_out, (int32_t)K, packed.data_ptr(),
                                                  (int32_t)cout, y.data_ptr(), y.stride(0), sp,
                                                  bias ? b32.data_ptr<float>() : nullptr, relu ? 1 : 0,
                                                  device_error_flag(x.device()).data_ptr<int32_t>(), s),
                         "sparse conv forward (tensor cores)");
            return y;
        }
        check_status(fvgb_conv_fwd_tc_epilogue(FVGB_BF16, x.data_ptr(), x.size(0), (int32_t)cin, x.stride(0),
                                               map.data_ptr<int32_t>(), n_out, (int32_t)K, tm, packed.data_ptr(),
                                               (int32_t)cout, y.data_ptr(), y.stride(0), sp,
                                               bias ? b32.data_ptr<float>() : nullptr, relu ? 1 : 0,
                                               device_error_flag(x.device()).data_ptr<int32_t>(), s),
                     "sparse conv forward (tensor cores)");
        return y;
    } else if (dt == FVGB_F32 || dt == FVGB_F64) {
        // large maps take the row order at once (C2 layer 1 FP32: 3.1 -> 1.9 ms for a 0.23 ms
        // build); small ones only once reused, where the build's launches would dominate
        const auto order = !pack ? std::nullopt
                                 : (n_out >= (int64_t)1 << 16 ? pack_row_order(pack, map_t)
                                                              : pack_row_order_if_reused(pack, map_t));
        const Tensor &m_used = order ? order->map : map;
        check_status(fvgb_conv_fwd_simt_rows(dt, x.data_ptr(), x.size(0), (int32_t)cin, x.stride(0),
                                             m_used.data_ptr<int32_t>(), n_out, (int32_t)K, m_used.stride(0),
                                             order ? order->rows.data_ptr<int32_t>() : nullptr, w.data_ptr(), wsk,
                                             wsci, wsco, y.data_ptr(), (int32_t)cout, y.stride(0), 0, s),
                     "sparse conv forward");
    } else {
        // 16-bit features of shapes the tensor-core kernel does not take: CUDA cores, FP32
        // accumulate, rounded once at the end.
        Tensor xf = x.to(torch::kFloat32), wf = w.to(torch::kFloat32);
        Tensor yf = torch::empty({n_out, cout}, xf.options());
        check_status(fvgb_conv_fwd_simt(FVGB_F32, xf.data_ptr(), xf.size(0), (int32_t)cin, xf.stride(0),
                                        map.data_ptr<int32_t>(), n_out, (int32_t)K, map.stride(0), wf.data_ptr(),
                                        wf.stride(0), transpose_w ? wf.stride(2) : wf.stride(1),
                                        transpose_w ? wf.stride(1) : wf.stride(2), yf.data_ptr(), (int32_t)cout,
                                        yf.stride(0), 0, s),
                     "sparse conv forward");
        y.copy_(yf);
    }
    if (out_scale) y.mul_(out_scale->to(y.scalar_type()));
    if (bias) y.add_(bias->to(y.scalar_type()));
    if (relu) y.relu_();
    return y;
}

// dW[k] = sum_m x[map[m,k]]^T dy[m]   -> [K, Cin, Cout]
Tensor gather_wgrad(const Tensor &x, const Tensor &map, int64_t n_out, const Tensor &dy, int64_t K,
                    const std::optional<Tensor> &tile_mask = std::nullopt) {
    c10::cuda::CUDAGuard guard(x.device());
    const int64_t cin = x.size(1), cout = dy.size(1);
    if (x.scalar_type() == torch::kBFloat16 && (cin == 32 || cin == 64 || cin == 128) &&
        (cout == 64 || cout == 128 || cout == 256)) {
        // tensor cores: FP32 partials per CTA, FP64 reduction across CTAs
        Tensor xx = x.contiguous(), dd = dy.to(torch::kBFloat16).contiguous();
        Tensor dw = torch::empty({K, cin, cout}, x.options().dtype(torch::kFloat32));
        size_t wsb = 0;
        check_status(fvgb_tc_wgrad_workspace(n_out, (int32_t)K, (int32_t)cin, (int32_t)cout, &wsb), "wgrad workspace");
        Tensor ws = workspace(wsb, x.device());
        const uint32_t *tm = tile_mask ? reinterpret_cast<const uint32_t *>(tile_mask->data_ptr<int32_t>()) : nullptr;
        check_status(fvgb_conv_wgrad_tc(xx.data_ptr(), xx.size(0), (int32_t)cin, xx.stride(0), map.data_ptr<int32_t>(),
                                        n_out, (int32_t)K, tm, dd.data_ptr(), (int32_t)cout, dd.stride(0),
                                        dw.data_ptr<float>(), ws.data_ptr(), ws.numel(),
                                        device_error_flag(x.device()).data_ptr<int32_t>(), cur_stream()),
                     "sparse conv weight gradient (tensor cores)");
        return dw.to(x.scalar_type());
    }
    const bool wide = x.scalar_type() == torch::kFloat64;
    Tensor xx = wide ? x : x.to(torch::kFloat32).contiguous();
    Tensor dd = (wide ? dy : dy.to(torch::kFloat32)).contiguous();
    const int32_t dt = wide ? FVGB_F64 : FVGB_F32;
    Tensor dw = torch::empty({K, cin, cout}, xx.options());
    size_t wsb = 0;
    check_status(fvgb_wgrad_workspace(dt, n_out, (int32_t)K, (int32_t)cin, (int32_t)cout, &wsb), "wgrad workspace");
    Tensor ws = workspace(wsb, x.device());
    check_status(fvgb_conv_wgrad_simt(dt, xx.data_ptr(), xx.size(0), (int32_t)cin, xx.stride(0), map.data_ptr<int32_t>(),
                                      n_out, (int32_t)K, map.stride(0), dd.data_ptr(), (int32_t)cout, dd.stride(0),
                                      dw.data_ptr(), ws.data_ptr(), ws.numel(), cur_stream()),
                 "sparse conv weight gradient");
    return dw.to(x.scalar_type());
}

// ------------------------------------------------------------------------------------------
// Forward / backward of one sparse convolution, called by the Python autograd Function.
// Checks and permutes follow SparseConvolutionKernelMap.cpp:18-191.
// relu: the output is max(conv + bias, 0), fused into the tensor-core epilogue; out_scale
// (optional, [Cout]): the output is conv * out_scale + bias (an inference-mode batch norm folded
// into the layer), also in the epilogue.
std::vector<Tensor> conv_forward(const Tensor &x, const Tensor &weights, PackPtr p, bool transposed,
                                 const std::optional<Tensor> &bias = std::nullopt, bool relu = false,
                                 const std::optional<Tensor> &out_scale = std::nullopt) {
    resolve_pack(p);
    TORCH_CHECK_VALUE(x.is_contiguous(), "features must be contiguous");
    TORCH_CHECK_TYPE(x.is_floating_point(), "features must have a floating point type");
    TORCH_CHECK_VALUE(x.dim() == 2, "Expected features to have 2 dimensions (shape (n, nF)) but got ", x.dim(),
                      " dimensions");
    TORCH_CHECK_TYPE(weights.is_floating_point(), "kernels must have a floating point type");
    for (int64_t i = 0; i < weights.dim(); ++i)
        TORCH_CHECK_VALUE(weights.size(i) != 0, "kernels tensor has zero dimension (dim = ", i, ")");
    TORCH_CHECK_VALUE(weights.dim() == 5, "Expected kernels to have 5 dimensions (shape (out_ch, in_ch, d, h, w)) but got ",
                      weights.dim(), " dimensions");
    TORCH_CHECK_VALUE(x.is_cuda() && weights.is_cuda(), "features and kernels must be CUDA tensors");
    const int64_t n_src = p->src->N, n_tgt = p->tgt->N;
    const int64_t K0 = weights.size(2), K1 = weights.size(3), K2 = weights.size(4);
    TORCH_CHECK_VALUE(K0 == p->ks.v[0] && K1 == p->ks.v[1] && K2 == p->ks.v[2],
                      "kernel spatial shape must match the kernel map's kernel_size");
    int64_t cin, cout;
    Tensor Wkio;
    if (!transposed) {
        TORCH_CHECK_VALUE(x.size(0) == n_src, "The number of input features must match the number of voxels");
        TORCH_CHECK_VALUE(weights.size(1) == x.size(1), "Expected input channels of kernels (", weights.size(1),
                          ") to equal input channels of features: ", x.size(1));
        cout = weights.size(0);
        cin = weights.size(1);
        if (auto c = derived_get(weights, 0)) {
            Wkio = *c;
        } else {
            Wkio = weights.permute({4, 3, 2, 1, 0}).reshape({-1, cin, cout});
            // a copy is worth keeping; a view is free to make again (and must not pin the weights)
            if (!Wkio.is_alias_of(weights)) derived_put(weights, 0, Wkio);
        }
    } else {
        TORCH_CHECK_VALUE(x.size(0) == n_tgt, "The number of input features must match the number of voxels");
        TORCH_CHECK_VALUE(weights.size(0) == x.size(1), "Expected input channels of kernels (", weights.size(0),
                          ") to equal input channels of features: ", x.size(1));
        cin = weights.size(0);
        cout = weights.size(1);
        if (auto c = derived_get(weights, 1)) {
            Wkio = *c;
        } else {
            Wkio = weights.permute({4, 3, 2, 0, 1}).reshape({-1, cin, cout});
            // a copy is worth keeping; a view is free to make again (and must not pin the weights)
            if (!Wkio.is_alias_of(weights)) derived_put(weights, 1, Wkio);
        }
    }
    if (bias) {
        TORCH_CHECK_VALUE(bias->dim() == 1 && bias->size(0) == cout, "bias must have shape (", cout, ",)");
        TORCH_CHECK_VALUE(bias->device() == x.device(), "bias must be on the features' device");
    }
    if (out_scale) {
        TORCH_CHECK_VALUE(out_scale->dim() == 1 && out_scale->size(0) == cout, "out_scale must have shape (", cout,
                          ",)");
        TORCH_CHECK_VALUE(out_scale->device() == x.device(), "out_scale must be on the features' device");
    }
    Tensor y;
    if (!transposed)
        y = n_tgt > 0 ? gather_gemm(x, pack_kmap(p), n_tgt, Wkio, false, pack_tile_mask(p, false), bias, p, false, relu,
                                    out_scale)
                      : torch::empty({0, cout}, x.options());
    else
        y = n_src > 0 ? gather_gemm(x, pack_kmap_t(p), n_src, Wkio, false, pack_tile_mask(p, true), bias, p, true, relu,
                                    out_scale)
                      : torch::empty({0, cout}, x.options());
    return {y, Wkio};
}

// Returns (dx, dW) with dW in the 5-D layout of the forward weights.
std::vector<Tensor> conv_backward(const Tensor &dy_in, const Tensor &x, const Tensor &Wkio, PackPtr p, bool transposed,
                                  bool need_dx, bool need_dw) {
    resolve_pack(p);
    Tensor dy = dy_in.contiguous();
    const int64_t K = Wkio.size(0), cin = Wkio.size(1), cout = Wkio.size(2);
    Tensor dx, dW;
    if (!transposed) {
        // dgrad: dx[i] = sum_k dy[mapT[i,k]] W[k]^T ;  wgrad: dW[k] = sum_m x[map[m,k]]^T dy[m]
        if (need_dx)
            dx = gather_gemm(dy, pack_kmap_t(p), p->src->N, Wkio, true, pack_tile_mask(p, true), std::nullopt, p, true);
        if (need_dw) dW = gather_wgrad(x, pack_kmap(p), p->tgt->N, dy, K, pack_tile_mask(p, false));
    } else {
        if (need_dx)
            dx = gather_gemm(dy, pack_kmap(p), p->tgt->N, Wkio, true, pack_tile_mask(p, false), std::nullopt, p, false);
        if (need_dw) dW = gather_wgrad(x, pack_kmap_t(p), p->src->N, dy, K, pack_tile_mask(p, true));
    }
    if (need_dw) {
        dW = dW.reshape({p->ks.v[2], p->ks.v[1], p->ks.v[0], cin, cout});
        dW = transposed ? dW.permute({3, 4, 2, 1, 0}) : dW.permute({4, 3, 2, 1, 0});
    }
    return {dx, dW};
}

// FP8-E4M3 forward (inference): per-input-channel feature scales s_x (folded into the weights)
// and per-output-channel weight scales s_w (applied in the epilogue), FP32 accumulation:
//   y[m, co] = s_w[co] * sum_k sum_ci e4m3(x[., ci] / s_x[ci]) * e4m3(s_x[ci] W[k, ci, co] / s_w[co])
// Returns (y bf16, s_x, s_w).
std::vector<Tensor> conv_forward_fp8(const Tensor &x, const Tensor &weights, PackPtr p, bool transposed,
                                     bool relu = false) {
    resolve_pack(p);
    TORCH_CHECK_VALUE(x.dim() == 2 && x.is_cuda() && x.is_floating_point(), "features must be a 2-D CUDA float tensor");
    TORCH_CHECK_VALUE(weights.dim() == 5, "Expected kernels to have 5 dimensions");
    c10::cuda::CUDAGuard guard(x.device());
    const int64_t cin = transposed ? weights.size(0) : weights.size(1);
    const int64_t cout = transposed ? weights.size(1) : weights.size(0);
    TORCH_CHECK_VALUE(x.size(1) == cin, "Expected input channels of kernels (", cin, ") to equal input channels of features: ",
                      x.size(1));
    TORCH_CHECK_VALUE(cin % 32 == 0 && cout <= 256, "the FP8 path needs in_channels % 32 == 0 and out_channels <= 256");
    const int64_t n_rows = transposed ? p->src->N : p->tgt->N;
    TORCH_CHECK_VALUE(x.size(0) == (transposed ? p->tgt->N : p->src->N),
                      "The number of input features must match the number of voxels");
    Tensor Wkio = (transposed ? weights.permute({4, 3, 2, 0, 1}) : weights.permute({4, 3, 2, 1, 0}))
                      .reshape({-1, cin, cout})
                      .to(torch::kFloat32);
    const int64_t K = Wkio.size(0);
    Tensor xc = x.scalar_type() == torch::kBFloat16 ? x.contiguous() : x.to(torch::kFloat32).contiguous();
    Tensor s_x = (xc.size(0) > 0 ? xc.abs().amax(0).to(torch::kFloat32) : torch::ones({cin}, Wkio.options()))
                     .clamp_min(1e-12) / 448.0f;
    Tensor wf = Wkio * s_x.view({1, cin, 1});
    Tensor s_w = wf.abs().amax({0, 1}).clamp_min(1e-12) / 448.0f;
    Tensor w8 = (wf / s_w.view({1, 1, cout})).to(at::ScalarType::Float8_e4m3fn).contiguous();
    Tensor x8 = torch::empty({xc.size(0), cin}, x.options().dtype(torch::kUInt8));
    Tensor inv = (1.0f / s_x).contiguous();
    auto s = cur_stream();
    check_status(fvgb_quantize_e4m3(xc.scalar_type() == torch::kBFloat16 ? FVGB_BF16 : FVGB_F32, xc.data_ptr(),
                                    xc.size(0), (int32_t)cin, xc.stride(0), inv.data_ptr<float>(), x8.data_ptr(), cin, s),
                 "fp8 quantisation");
    Tensor y = torch::empty({n_rows, cout}, x.options().dtype(torch::kBFloat16));
    if (n_rows == 0) return {y, s_x, s_w};
    size_t wb = 0;
    check_status(fvgb_tc_weight_bytes(FVGB_E4M3, K, (int32_t)cin, (int32_t)cout, &wb), "weight pack size");
    Tensor packed = torch::empty({(int64_t)wb}, x.options().dtype(torch::kUInt8));
    check_status(fvgb_tc_pack_weights(FVGB_E4M3, w8.data_ptr(), K, (int32_t)cin, (int32_t)cout, cin * cout, cout, 1,
                                      packed.data_ptr(), wb, s),
                 "fp8 weight pack");
    const Tensor &map = transposed ? pack_kmap_t(p) : pack_kmap(p);
    auto tm = pack_tile_mask(p, transposed);
    Tensor sw = s_w.contiguous();
    const auto order = pack_row_order_if_reused(p, transposed);
    std::optional<Tensor> plan;
    if (K < 4 && use_plan(FVGB_E4M3, K, cin, cout, 1)) plan = pack_plan_if_reused(p, transposed, (int32_t)cin);
    if (plan) {
        check_status(fvgb_conv_fwd_tc_planned(FVGB_E4M3, x8.data_ptr(), x8.size(0), (int32_t)cin, cin, plan->data_ptr(),
                                              n_rows, (int32_t)K, packed.data_ptr(), (int32_t)cout, y.data_ptr(),
                                              y.stride(0), sw.data_ptr<float>(), nullptr, relu ? 1 : 0,
                                              device_error_flag(x.device()).data_ptr<int32_t>(), s),
                     "sparse conv forward (fp8 tensor cores)");
        return {y, s_x, s_w};
    }
    const std::optional<Tensor> tmo = order ? std::optional<Tensor>(order->mask) : tm;
    check_status(fvgb_conv_fwd_tc_rows(FVGB_E4M3, x8.data_ptr(), x8.size(0), (int32_t)cin, cin,
                                       (order ? order->map : map).data_ptr<int32_t>(), n_rows, (int32_t)K,
                                       order ? order->rows.data_ptr<int32_t>() : nullptr,
                                       tmo ? reinterpret_cast<const uint32_t *>(tmo->data_ptr<int32_t>()) : nullptr,
                                       packed.data_ptr(), (int32_t)cout, y.data_ptr(), y.stride(0),
                                       sw.data_ptr<float>(), nullptr, relu ? 1 : 0,
                                       device_error_flag(x.device()).data_ptr<int32_t>(), s),
                 "sparse conv forward (fp8 tensor cores)");
    return {y, s_x, s_w};
}

// ------------------------------------------------------------------------------------------
// Pooling / nearest upsampling between grids (GridBatch::max_pool / avg_pool / subdivide,
// src/fvdb/GridBatch.cpp:241-345) and the grids they default to.

// coarsened_grid(f): floor(ijk / f) per axis (GridBatch::coarsened_grid, BuildCoarseGridFromFine.cu:22-82),
// the coarse path of conv_grid with kernel == stride == f.
GridPtr grid_coarsened(const GridPtr &g, const std::vector<int64_t> &f) {
    R(g);
    Vec3 v = to_vec3(f, "coarsening_factor");
    for (int a = 0; a < 3; ++a) TORCH_CHECK_VALUE(v.v[a] > 0, "coarsening_factor must be positive");
    std::vector<int64_t> ff = {v.v[0], v.v[1], v.v[2]};
    GridPtr c = grid_conv_grid(g, ff, ff);
    // coarse transform (GridBatchImpl.cu:645-655): size f*w, origin (f-1)*w*0.5 + o
    Tensor fv = torch::tensor({(double)v.v[0], (double)v.v[1], (double)v.v[2]}, torch::kFloat64);
    c->voxel_sizes = fv * g->voxel_sizes;
    c->origins = (fv - 1.0) * g->voxel_sizes * 0.5 + g->origins;
    return c;
}

// subdivided_grid(f, mask): every (masked) voxel c gives c*f + (i,j,k) (GridBatch::subdivided_grid,
// BuildFineGridFromCoarse.cu:66-226).
GridPtr grid_subdivided(const GridPtr &g, const std::vector<int64_t> &f, const std::optional<Tensor> &mask) {
    R(g);
    c10::cuda::CUDAGuard guard(g->device());
    Vec3 v = to_vec3(f, "subdiv_factor");
    for (int a = 0; a < 3; ++a) TORCH_CHECK_VALUE(v.v[a] > 0, "subdiv_factor must be positive");
    const int64_t V = (int64_t)v.v[0] * v.v[1] * v.v[2];
    TORCH_CHECK_VALUE(V <= 512, "subdiv_factor volume must be at most 512");
    auto dev = g->device();
    Tensor m;
    if (mask) {
        TORCH_CHECK_VALUE(mask->dim() == 1 && mask->size(0) == g->N, "mask must have one entry per voxel");
        m = mask->to(dev, torch::kUInt8).contiguous();
    }
    const int64_t n = g->N * V;
    auto i32 = torch::dtype(torch::kInt32).device(dev);
    Tensor cand = torch::empty({std::max<int64_t>(n, 1), 3}, i32);
    Tensor valid = torch::empty({std::max<int64_t>(n, 1)}, torch::dtype(torch::kUInt8).device(dev));
    FvgbGrid gv = g->view();
    auto s = cur_stream();
    check_status(fvgb_subdivide_candidates(&gv, v.v, mask ? m.data_ptr<uint8_t>() : nullptr, cand.data_ptr<int32_t>(),
                                           valid.data_ptr<uint8_t>(), s),
                 "subdivided_grid (candidates)");
    Tensor out = torch::empty({std::max<int64_t>(n, 1), 3}, i32);
    Tensor joff = torch::empty({g->B + 1}, torch::dtype(torch::kInt64).device(dev));
    size_t sb = 0;
    check_status(fvgb_scan_workspace(n, &sb), "subdivided_grid (workspace)");
    Tensor ws = workspace(sb, dev);
    check_status(fvgb_compact_ijk(cand.data_ptr<int32_t>(), valid.data_ptr<uint8_t>(), g->joffsets.data_ptr<int64_t>(),
                                  (int32_t)g->B, V, n, out.data_ptr<int32_t>(), joff.data_ptr<int64_t>(), ws.data_ptr(),
                                  ws.numel(), s),
                 "subdivided_grid (compact)");
    const int64_t mcount = n > 0 ? joff[g->B].item<int64_t>() : 0;
    // fine transform (GridBatchImpl.cu:633-643): size w/f, origin o - (f-1)*(w/f)*0.5
    Tensor fv = torch::tensor({(double)v.v[0], (double)v.v[1], (double)v.v[2]}, torch::kFloat64);
    Tensor vs = g->voxel_sizes / fv;
    Tensor org = g->origins - (fv - 1.0) * (g->voxel_sizes / fv) * 0.5;
    if (g->N == 0) return build_grid(out.narrow(0, 0, 0), joff, vs, org);
    int32_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = g->box_lo[a] * v.v[a];
        hi[a] = g->box_hi[a] * v.v[a] + v.v[a] - 1;
    }
    return build_grid(out.narrow(0, 0, mcount), joff, vs, org, lo, hi);
}

Tensor flat2d(const Tensor &t) { return t.reshape({t.size(0), -1}).contiguous(); }

// y [coarse N, C] = max / average pooling of x [fine N, *] (mode FVGB_POOL_MAX / FVGB_POOL_AVG)
Tensor pool_forward(int32_t mode, const GridPtr &fine, const GridPtr &coarse, const std::vector<int64_t> &pool,
                    const std::vector<int64_t> &stride, const Tensor &x) {
    R(fine);
    R(coarse);
    c10::cuda::CUDAGuard guard(fine->device());
    TORCH_CHECK_VALUE(x.dim() > 1, "fine_data must have more than one dimension. i.e. have shape (num_voxels, *)");
    TORCH_CHECK_VALUE(x.size(0) == fine->N, "fine_data must have the same number of voxels as fine_grid");
    TORCH_CHECK(fine->device() == coarse->device(), "coarse_grid and fine_grid must be on the same device");
    Vec3 p = to_vec3(pool, "pool_factor"), st = to_vec3(stride, "stride");
    for (int a = 0; a < 3; ++a) {
        TORCH_CHECK_VALUE(p.v[a] > 0, "pooling_factor must be greater than 0");
        TORCH_CHECK_VALUE(st.v[a] >= 0, "stride must be greater than or equal to 0");
        if (st.v[a] == 0) st.v[a] = p.v[a];
    }
    Tensor xf = flat2d(x);
    const int64_t C = xf.size(1);
    std::vector<int64_t> shape = x.sizes().vec();
    shape[0] = coarse->N;
    Tensor y = torch::empty({coarse->N, std::max<int64_t>(C, 1)}, x.options());
    if (C > 0 && coarse->N > 0) {
        FvgbGrid fv = fine->view(), cv = coarse->view();
        check_status(fvgb_pool_forward(mode, fvgb_dtype(x), &fv, &cv, p.v, st.v, fine->N ? xf.data_ptr() : nullptr,
                                       C, (int32_t)C, y.data_ptr(), C, cur_stream()),
                     mode == FVGB_POOL_MAX ? "max_pool" : "avg_pool");
    }
    return y.narrow(1, 0, C).reshape(shape);
}

Tensor pool_backward(int32_t mode, const GridPtr &fine, const GridPtr &coarse, const std::vector<int64_t> &pool,
                     const std::vector<int64_t> &stride, const Tensor &x, const Tensor &dy) {
    R(fine);
    R(coarse);
    c10::cuda::CUDAGuard guard(fine->device());
    Vec3 p = to_vec3(pool, "pool_factor"), st = to_vec3(stride, "stride");
    for (int a = 0; a < 3; ++a)
        if (st.v[a] == 0) st.v[a] = p.v[a];
    Tensor xf = flat2d(x), df = flat2d(dy.to(x.scalar_type()));
    const int64_t C = xf.size(1);
    FvgbGrid fv = fine->view(), cv = coarse->view();
    auto s = cur_stream();
    if (C == 0 || fine->N == 0) return torch::zeros_like(x);
    if (mode == FVGB_POOL_MAX) {
        const auto acc = x.scalar_type() == torch::kFloat64 ? torch::kFloat64 : torch::kFloat32;
        Tensor dacc = torch::zeros({fine->N, C}, x.options().dtype(acc));
        check_status(fvgb_maxpool_backward(fvgb_dtype(x), &fv, &cv, p.v, st.v, xf.data_ptr(), C, (int32_t)C,
                                           coarse->N ? df.data_ptr() : nullptr, C, dacc.data_ptr(), s),
                     "max_pool backward");
        return dacc.to(x.scalar_type()).reshape(x.sizes());
    }
    Tensor dx = torch::empty({fine->N, C}, x.options());
    check_status(fvgb_avgpool_backward(fvgb_dtype(x), &fv, &cv, p.v, st.v, (int32_t)C, coarse->N ? df.data_ptr() : nullptr,
                                       C, dx.data_ptr(), C, s),
                 "avg_pool backward");
    return dx.reshape(x.sizes());
}

// Stride-1 3^3 convolution over the grid without a kernel map: y = sum_k x[v + d_k] W[k] for
// W [27, Cin, Cout] (mirror: the data gradient, W[26-k]^T with W in the forward's layout).
Tensor halo_conv(const GridPtr &g, const Tensor &x, const Tensor &w, bool mirror) {
    R(g);
    c10::cuda::CUDAGuard guard(g->device());
    TORCH_CHECK_VALUE(x.dim() == 2 && x.size(0) == g->N, "features must have shape (num_voxels, channels)");
    TORCH_CHECK_VALUE(w.dim() == 3 && w.size(0) == 27, "halo weights must have shape (27, in, out)");
    TORCH_CHECK_TYPE(w.scalar_type() == x.scalar_type(), "halo weights and features must have the same dtype");
    const int64_t cin = x.size(1), cout = mirror ? w.size(1) : w.size(2);
    TORCH_CHECK_VALUE((mirror ? w.size(2) : w.size(1)) == cin, "halo weights do not match the feature channels");
    Tensor xc = x.contiguous(), wc = w.contiguous();
    Tensor y = torch::empty({g->N, cout}, x.options());
    if (g->N > 0 && cin > 0 && cout > 0) {
        FvgbGrid v = g->view();
        check_status(fvgb_halo_conv(fvgb_dtype(x), &v, xc.data_ptr(), cin, (int32_t)cin, wc.data_ptr(), (int32_t)cout,
                                    mirror ? 1 : 0, y.data_ptr(), cout, cur_stream()),
                     "halo convolution");
    } else if (cout > 0) {
        y.zero_();
    }
    return y;
}

// dW [27, Cin, Cout] = sum_v x[v + d_k]^T dy[v] (fixed-order FP64 sum of per-chunk partials)
Tensor halo_wgrad(const GridPtr &g, const Tensor &x, const Tensor &dy) {
    R(g);
    c10::cuda::CUDAGuard guard(g->device());
    TORCH_CHECK_VALUE(x.dim() == 2 && dy.dim() == 2 && x.size(0) == g->N && dy.size(0) == g->N,
                      "features and gradients must have shape (num_voxels, channels)");
    Tensor xc = x.contiguous(), dc = dy.to(x.scalar_type()).contiguous();
    const int64_t cin = x.size(1), cout = dy.size(1);
    Tensor dw = torch::empty({27, cin, cout}, x.options());
    if (cin == 0 || cout == 0) return dw;
    FvgbGrid v = g->view();
    size_t wsb = 0;
    check_status(fvgb_halo_wgrad_workspace(fvgb_dtype(x), &v, (int32_t)cin, (int32_t)cout, &wsb), "halo wgrad workspace");
    Tensor ws = workspace(wsb, x.device());
    check_status(fvgb_halo_wgrad(fvgb_dtype(x), &v, g->N ? xc.data_ptr() : nullptr, cin, (int32_t)cin,
                                 g->N ? dc.data_ptr() : nullptr, cout, (int32_t)cout, dw.data_ptr(), ws.data_ptr(),
                                 ws.numel(), cur_stream()),
                 "halo weight gradient");
    return dw;
}

// y [fine N, *] = nearest upsampling of x [coarse N, *]
Tensor upsample_forward(const GridPtr &coarse, const GridPtr &fine, const std::vector<int64_t> &factor, const Tensor &x) {
    R(fine);
    R(coarse);
    c10::cuda::CUDAGuard guard(fine->device());
    TORCH_CHECK_VALUE(x.dim() > 1 && x.size(0) == coarse->N, "data must have shape (num_voxels, *) of the coarse grid");
    Vec3 f = to_vec3(factor, "subdiv_factor");
    Tensor xf = flat2d(x);
    const int64_t C = xf.size(1);
    std::vector<int64_t> shape = x.sizes().vec();
    shape[0] = fine->N;
    Tensor y = torch::empty({fine->N, std::max<int64_t>(C, 1)}, x.options());
    if (C > 0 && fine->N > 0) {
        FvgbGrid fv = fine->view(), cv = coarse->view();
        check_status(fvgb_upsample_forward(fvgb_dtype(x), &cv, &fv, f.v, coarse->N ? xf.data_ptr() : nullptr, C,
                                           (int32_t)C, y.data_ptr(), C, cur_stream()),
                     "subdivide");
    }
    return y.narrow(1, 0, C).reshape(shape);
}

Tensor upsample_backward(const GridPtr &coarse, const GridPtr &fine, const std::vector<int64_t> &factor, const Tensor &dy,
                         const Tensor &x) {
    R(fine);
    R(coarse);
    c10::cuda::CUDAGuard guard(fine->device());
    Vec3 f = to_vec3(factor, "subdiv_factor");
    Tensor df = flat2d(dy.to(x.scalar_type()));
    const int64_t C = df.size(1);
    Tensor dx = torch::empty({coarse->N, std::max<int64_t>(C, 1)}, x.options());
    if (C > 0 && coarse->N > 0) {
        FvgbGrid fv = fine->view(), cv = coarse->view();
        check_status(fvgb_upsample_backward(fvgb_dtype(x), &cv, &fv, f.v, fine->N ? df.data_ptr() : nullptr, C,
                                            (int32_t)C, dx.data_ptr(), C, cur_stream()),
                     "subdivide backward");
    }
    return dx.narrow(1, 0, C).reshape(x.sizes());
}

std::optional<Tensor> opt(const std::optional<Tensor> &t) { return t; }

}  // namespace fvgbh

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    using namespace fvgbh;
    namespace py = pybind11;
    m.doc() = "fvdb_gb300 host extension: grids, kernel maps and sparse convolution on GB300";
    m.def("version", []() { return std::string(fvgb_version()); });

    py::class_<GridImpl, GridPtr>(m, "GridImpl")
        .def_static("from_ijk", &grid_from_ijk, py::arg("ijk"), py::arg("joffsets"), py::arg("voxel_sizes"),
                    py::arg("origins"), py::call_guard<py::gil_scoped_release>())
        .def_static("from_points", &grid_from_points, py::arg("points"), py::arg("joffsets"),
                    py::arg("voxel_sizes"), py::arg("origins"), py::call_guard<py::gil_scoped_release>())
        .def("conv_grid", &grid_conv_grid, py::call_guard<py::gil_scoped_release>())
        .def("coarsened_grid", &grid_coarsened, py::call_guard<py::gil_scoped_release>())
        .def("subdivided_grid", &grid_subdivided, py::arg("subdiv_factor"), py::arg("mask") = py::none())
        .def_property_readonly("grid_count", [](const GridImpl &g) { return g.B; })
        .def_property_readonly("total_voxels", [](const GridImpl &g) { g.resolve(); return g.N; })
        .def_property_readonly("total_leaf_nodes", [](const GridImpl &g) { g.resolve(); return g.L; })
        .def_property_readonly("ijk", [](const GridImpl &g) { g.resolve(); return g.ijk; })
        .def_property_readonly("joffsets", [](const GridImpl &g) { g.resolve(); return g.joffsets; })
        .def_property_readonly("joffsets_host", [](const GridImpl &g) { g.resolve(); return g.joffsets_host; })
        .def_property_readonly("voxel_sizes", [](const GridImpl &g) { return g.voxel_sizes; })
        .def_property_readonly("origins", [](const GridImpl &g) { return g.origins; })
        .def_property_readonly("leaves", [](const GridImpl &g) { g.resolve(); return g.leaves; })
        .def_property_readonly("hash", [](const GridImpl &g) { g.resolve(); return g.hash; })
        .def_property_readonly("device", [](const GridImpl &g) { return g.device(); })
        .def("jidx", [](GridPtr g) { return grid_jidx(g); })
        .def("ijk_to_index", &grid_ijk_to_index);

    py::class_<PackInfo, PackPtr>(m, "PackInfoImpl")
        .def(py::init([](std::vector<int64_t> k, std::vector<int64_t> s, GridPtr src, std::optional<GridPtr> tgt) {
                 return make_pack(k, s, src, tgt);
             }),
             py::arg("kernel_size"), py::arg("stride"), py::arg("source_grid"), py::arg("target_grid") = py::none())
        .def("kmap", [](PackPtr p) { return pack_kmap(p); })
        .def("kmap_t", [](PackPtr p) { return pack_kmap_t(p); })
        .def("tile_mask", [](PackPtr p, bool transposed) { return pack_tile_mask(p, transposed); },
             py::arg("transposed") = false)
        .def("tile_plan", [](PackPtr p, bool transposed, int32_t row_bytes) { return pack_plan(p, transposed, row_bytes); },
             py::arg("transposed"), py::arg("row_bytes"))
        .def("build_gather_scatter", &pack_build_gather_scatter)
        .def("build_implicit_gemm", &pack_build_implicit_gemm)
        .def_property_readonly("kernel_size", [](const PackInfo &p) { return py::make_tuple(p.ks.v[0], p.ks.v[1], p.ks.v[2]); })
        .def_property_readonly("stride", [](const PackInfo &p) { return py::make_tuple(p.st.v[0], p.st.v[1], p.st.v[2]); })
        .def_property_readonly("source_grid", [](const PackInfo &p) { return p.src; })
        .def_property_readonly("target_grid", [](const PackInfo &p) { return p.tgt; })
        .def_property_readonly("out_in_map", [](const PackInfo &p) { return opt(p.out_in_map); })
        .def_property_readonly("out_in_map_bwd", [](const PackInfo &p) { return opt(p.out_in_map_bwd); })
        .def_property_readonly("neighborhood_map", [](const PackInfo &p) { return opt(p.nbmap); })
        .def_property_readonly("neighborhood_sizes", [](const PackInfo &p) { return opt(p.nbsizes); })
        .def_property_readonly("reorder_loc", [](const PackInfo &p) { return opt(p.reorder_loc); })
        .def_property_readonly("sorted_mask", [](const PackInfo &p) { return opt(p.sorted_mask); })
        .def_property_readonly("reorder_out_in_map", [](const PackInfo &p) { return opt(p.reorder_out_in_map); })
        .def_property_readonly("reduced_sorted_mask", [](const PackInfo &p) { return opt(p.reduced_sorted_mask); })
        .def_property_readonly("reorder_loc_bwd", [](const PackInfo &p) { return opt(p.reorder_loc_bwd); })
        .def_property_readonly("reorder_out_in_map_bwd", [](const PackInfo &p) { return opt(p.reorder_out_in_map_bwd); })
        .def_property_readonly("sorted_mask_bwd_w", [](const PackInfo &p) { return opt(p.sorted_mask_bwd_w); })
        .def_property_readonly("sorted_mask_bwd_d", [](const PackInfo &p) { return opt(p.sorted_mask_bwd_d); })
        .def_property_readonly("use_me", [](const PackInfo &p) { return p.use_me; })
        .def_property_readonly("use_tf32", [](const PackInfo &p) { return p.use_tf32; });

    // the GIL is released while the native calls run (their grid builds wait for a count read),
    // so host threads of concurrent serving slots do not serialise on it
    m.def("conv_forward", &conv_forward, py::arg("features"), py::arg("weights"), py::arg("pack"),
          py::arg("transposed"), py::arg("bias") = py::none(), py::arg("relu") = false,
          py::arg("out_scale") = py::none(), py::call_guard<py::gil_scoped_release>());
    m.def("conv_forward_fp8", &conv_forward_fp8, py::arg("features"), py::arg("weights"), py::arg("pack"),
          py::arg("transposed"), py::arg("relu") = false, py::call_guard<py::gil_scoped_release>());
    m.def("check_device_errors", [](const torch::Device &d) { check_device_errors(d); },
          py::call_guard<py::gil_scoped_release>());
    m.def("conv_backward", &conv_backward, py::call_guard<py::gil_scoped_release>());
    m.def("halo_conv", &halo_conv, py::call_guard<py::gil_scoped_release>());
    m.def("halo_wgrad", &halo_wgrad, py::call_guard<py::gil_scoped_release>());
    m.def("pool_forward", &pool_forward);
    m.def("pool_backward", &pool_backward);
    m.def("upsample_forward", &upsample_forward);
    m.def("upsample_backward", &upsample_backward);
    m.attr("POOL_MAX") = (int)FVGB_POOL_MAX;
    m.attr("POOL_AVG") = (int)FVGB_POOL_AVG;
}
