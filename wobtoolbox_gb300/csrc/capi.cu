// C ABI of the GB300 WoB engine (declarations and reference citations in include/wob_capi.h).
//
// A scene owns its device buffers (element records, intersection records, BVH nodes, CDFs and
// guide tables, the optional volume cache, a device error word) on the device that was current
// when it was created. Solves are asynchronous on the caller's stream; the *_host variants stage
// through a per-scene workspace and synchronise.
#include "../../include/wob_capi.h"

#include "launch.hpp"
#include "multi_rhs.hpp"
#include "scene_build_gpu.hpp"
#include "vpl.hpp"
#include "wos.hpp"
#include "scene_host.hpp"
#include "walk_generic.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
int fail_cuda(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WOB_ERR_OUT_OF_MEMORY : WOB_ERR_CUDA;
}
// Runs an entry point's body; a C++ exception (host allocation failure in the scene, table or
// staging builds) becomes a status instead of crossing the C ABI.
template <class F> int guarded(F &&body) {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        return fail(WOB_ERR_OUT_OF_MEMORY, "out of host memory");
    } catch (const std::exception &ex) {
        return fail(WOB_ERR_INVALID_ARGUMENT, ex.what());
    } catch (...) {
        return fail(WOB_ERR_INVALID_ARGUMENT, "unexpected error");
    }
}

// A device allocation freed with the scene.
// A device allocation. Owned alone (release frees it) until share() hands it to a second scene;
// from then on a reference count frees it with its last holder.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    std::shared_ptr<void> shared;  // set once the allocation is shared
    void release() {
        if (shared) shared.reset();
        else if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

// dst holds src's allocation too (for buffers that no entry point writes after the scene is built).
// The first share converts src to counted ownership; a process-wide lock makes concurrent clones of
// one scene convert it once.
std::mutex g_share_mutex;
void share(DevBuf &dst, DevBuf &src) {
    dst.release();
    if (!src.ptr) return;
    std::lock_guard<std::mutex> lock(g_share_mutex);
    if (!src.shared) src.shared = std::shared_ptr<void>(src.ptr, [](void *p) { cudaFree(p); });
    dst.ptr = src.ptr;
    dst.bytes = src.bytes;
    dst.shared = src.shared;
}

cudaError_t upload(DevBuf &b, const void *src, size_t bytes) {
    b.release();
    if (bytes == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) return e;
    b.bytes = bytes;
    return cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice);
}

}  // namespace

namespace wobgb {
void set_last_error(const char *msg) { g_last_error = msg; }
}  // namespace wobgb

struct wob_scene_s {
    int device = 0;
    wobgb::HostScene host;
    DevBuf elems, elem_aux, isect, nodes, area_cdf, area_guide, bv_cdf, bv_guide, err;
    DevBuf vol_values, vol_cdf, vol_guide;
    DevBuf lg_bins, lg_off, lg_ent;  // 2D line grid
    DevBuf cv_table;  // control-variate density per stored element
    DevBuf rhs;       // multi-RHS data [n][dim][n_rhs], storage order
    DevBuf rhs_cv;    // multi-RHS control variate [n][n_rhs], storage order
    uint32_t n_rhs = 0;
    uint32_t traversal_limit = 0;  // 0: 5 x nodes + 16; else the override of wob_scene_set_step_limits
    uint32_t wos_limit = 0;        // 0: kWosMaxSteps; else the override of wob_scene_set_step_limits
    bool has_volume = false;
    uint32_t area_G = 0, bv_G = 0;  // guide-table records
    uint32_t vol_res = 0, vol_n = 0, vol_G = 0;
    float vol_size = 0.0f;
    bool all_dirichlet = true;
    // workspace of the host-pointer entry points
    std::mutex ws_mutex;
    DevBuf ws;
    cudaStream_t ws_stream = nullptr;

    template <int D> wobgb::SceneView<D> view() const {
        wobgb::SceneView<D> v{};
        v.elems = (const float4 *)elems.ptr;
        v.elem_aux = (const float4 *)elem_aux.ptr;
        v.alpha_const = host.alpha_const ? 1u : 0u;
        v.alpha_value = host.alpha_value;
        v.isect = (const float4 *)isect.ptr;
        v.nodes = (const float4 *)nodes.ptr;
        v.area_cdf = (const float *)area_cdf.ptr;
        v.area_guide = (const uint4 *)area_guide.ptr;
        v.bv_cdf = (const float *)bv_cdf.ptr;
        v.bv_guide = (const uint4 *)bv_guide.ptr;
        v.vol_values = (const float *)vol_values.ptr;
        v.vol_cdf = (const float *)vol_cdf.ptr;
        v.vol_guide = (const uint4 *)vol_guide.ptr;
        v.err = (uint32_t *)err.ptr;
        v.cv_table = (const float *)cv_table.ptr;
        v.lg_bins = (const float4 *)lg_bins.ptr;
        v.lg_off = (const uint32_t *)lg_off.ptr;
        v.lg_ent = (const uint16_t *)lg_ent.ptr;
        v.lg_K = lg_bins.ptr ? host.line_grid.K : 0u;
        v.lg_M = host.line_grid.M;
        v.lg_cx = host.line_grid.cx;
        v.lg_cy = host.line_grid.cy;
        v.lg_far = host.line_grid.far;
        v.n_elems = host.n;
        v.n_nodes = host.n_nodes;
        v.area_G = area_G;
        v.bv_G = bv_G;
        v.vol_n = vol_n;
        v.vol_G = vol_G;
        v.vol_res = vol_res;
        v.traversal_limit = traversal_limit ? traversal_limit : 5u * host.n_nodes + 16u;
        v.wos_step_limit = wos_limit ? wos_limit : wobgb::kWosMaxSteps;
        v.total_area = host.total_area;
        v.total_bv = host.total_bv;
        v.vol_size = vol_size;
        return v;
    }
    ~wob_scene_s() { release_all(); }
    void release_all() {
        for (DevBuf *b : {&elems, &elem_aux, &isect, &nodes, &area_cdf, &area_guide, &bv_cdf, &bv_guide, &err, &vol_values,
                          &vol_cdf, &vol_guide, &cv_table, &rhs, &rhs_cv, &ws, &lg_bins, &lg_off, &lg_ent})
            b->release();
        if (ws_stream) cudaStreamDestroy(ws_stream);
        ws_stream = nullptr;
    }
};

// A batch of scenes solved in one persistent launch (k_batch.cu). The scenes must outlive it.
// The table is grouped by walk class (batch_walk_class): one persistent launch per class present,
// each over its contiguous part of the table with unit numbers restarting at 0.
struct wob_batch_s {
    int device = 0;
    int dim = 0;
    uint32_t n_scenes = 0;
    uint64_t total_units = 0;
    uint32_t total_points = 0;
    uint32_t cls_first[3] = {0, 0, 0}, cls_count[3] = {0, 0, 0};
    uint64_t cls_units[3] = {0, 0, 0};
    DevBuf table;
    ~wob_batch_s() { table.release(); }
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// Checks the parameters against the scene; fills the kernel parameter block.
int check_params(const wob_scene_s *s, const wob_params *p, wobgb::WalkParams &w) {
    if (!p) return fail(WOB_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->bie_model < 0 || p->bie_model > 2) return fail(WOB_ERR_INVALID_ARGUMENT, "bie_model must be 0 (IndirectSingleLayer), 1 (IndirectDoubleLayer) or 2 (Direct)");
    if (p->domain < 0 || p->domain > 1) return fail(WOB_ERR_INVALID_ARGUMENT, "domain must be 0 (InteriorDomain) or 1 (ExteriorDomain)");
    if (p->estimator < 0 || p->estimator > 1) return fail(WOB_ERR_INVALID_ARGUMENT, "estimator must be 0 (BackwardEstimator) or 1 (ForwardEstimator)");
    if (p->problem < 0 || p->problem > 3) return fail(WOB_ERR_INVALID_ARGUMENT, "problem must be 0..3 (Dirichlet, Neumann, Robin, Mixed)");
    if (p->path_length < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "path_length must be >= 1");
    if (p->num_sample_paths < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "num_sample_paths must be >= 1");
    if (p->num_resampling_candidates < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "num_resampling_candidates must be >= 1");
    if (!(p->eps > 0.0f) || !(p->eps < 3.0e38f)) return fail(WOB_ERR_INVALID_ARGUMENT, "eps must be positive and finite");
    const float fk = p->first_kind_equation_scaling_constant;
    if (!(fk > 0.0f) || !(fk < 3.0e38f)) return fail(WOB_ERR_INVALID_ARGUMENT, "first_kind_equation_scaling_constant must be positive and finite");
    if (p->flags != 0) return fail(WOB_ERR_INVALID_ARGUMENT, "flags must be 0");
    if (p->bie_model == WOB_INDIRECT_DOUBLE_LAYER && !s->all_dirichlet)
        return fail(WOB_ERR_UNSUPPORTED, "the double-layer model supports Dirichlet boundaries only (bie_models.cuh:383)");
    const bool needs_bv = (p->estimator == WOB_BACKWARD_ESTIMATOR && p->bie_model == WOB_DIRECT && p->problem == WOB_NEUMANN_PROBLEM) ||
                          (p->estimator == WOB_FORWARD_ESTIMATOR && p->bie_model == WOB_INDIRECT_SINGLE_LAYER && p->problem == WOB_NEUMANN_PROBLEM);
    if (needs_bv && !s->host.bv_valid)
        return fail(WOB_ERR_INVALID_ARGUMENT, "boundary-value sampling needs a nonzero, finite total |g|");
    if (p->num_volume_samples > 0 && !s->has_volume)
        return fail(WOB_ERR_INVALID_ARGUMENT, "num_volume_samples > 0 needs a volume cache (wob_scene_set_volume_cache)");
    w.bie = p->bie_model;
    w.domain = p->domain;
    w.estimator = p->estimator;
    w.problem = p->problem;
    w.path_length = p->path_length;
    w.n_paths = p->num_sample_paths;
    w.n_resampling = p->num_resampling_candidates;
    w.n_volume = p->num_volume_samples;
    w.eps = p->eps;
    w.fk = fk;
    w.seed = p->seed;
    w.path_offset = p->path_offset;
    w.point_offset = p->point_offset;
    w.ppt = 1;
    w.ppt_cap = 0;
    w.no_alloc = 0;
    w.ppt_points = 0;
    w.mode = 0;
    w.n_pot = 0;
    w.m_ker = 0;
    return WOB_OK;
}

// ------------------------------------------------------------------------------------------
// Allocation-free staging for wob_solve_domain_host_noalloc.
//
// Callers that may not allocate device memory (a host application that owns the GPU memory
// budget and forbids allocations by plugins, a real-time loop that must not allocate) still need
// the host-buffer solve. That entry point stages its points, running sums and bounce counter
// through this fixed array instead of a cudaMalloc'd workspace. It is a file-scope static device
// array, so every GPU that loads the library holds it until the process exits.
// ------------------------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;                        // serialises the entry point within a process
void *g_noalloc_addr[kNoAllocMaxDevices] = {};     // device address of the array, per device

inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Layout for n points of dimension D: points | sums | sums of squares | bounce counter.
size_t noalloc_bytes(int D, uint64_t n, size_t off[4]) {
    off[0] = 0;
    off[1] = align256(n * (uint64_t)D * 4);
    off[2] = off[1] + align256(n * (uint64_t)(D + 1) * 8);
    off[3] = off[2] + align256(n * (uint64_t)(D + 1) * 8);
    return off[3] + 256;
}

uint32_t noalloc_max_points(int D) {
    uint64_t lo = 0, hi = kNoAllocScratchBytes;
    size_t off[4];
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) / 2;
        if (noalloc_bytes(D, mid, off) <= kNoAllocScratchBytes) lo = mid;
        else hi = mid - 1;
    }
    return (uint32_t)lo;
}

// Device address of the scratch array on `device` (which must be current). The host-side name
// g_noalloc_scratch is only a stand-in: its address has to be looked up once per device. The
// lookup also makes the runtime load this module on the device if it has not yet (lazy module
// loading), which is when the array's memory is reserved. The cached address belongs to the
// device's current context; a cudaDeviceReset destroys that context, and the address must not be
// used after it.
int noalloc_scratch(int device, void **out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return fail(WOB_ERR_UNSUPPORTED, "device index out of range for the no-allocation scratch");
    if (!g_noalloc_addr[device]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_noalloc_addr[device] = ptr;
    }
    *out = g_noalloc_addr[device];
    return WOB_OK;
}

}  // namespace

extern "C" {

const char *wob_last_error(void) { return g_last_error.c_str(); }

int wob_version(void) { return WOB_CAPI_VERSION; }

int wob_device_info(int *device, int *sm_count) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
    if (device) *device = dev;
    if (sm_count) {
        e = cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail_cuda(e, "cudaDeviceGetAttribute");
    }
    return WOB_OK;
}

static int scene_create_impl(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                             const float *boundary_values, const float *robin_alphas, const int32_t *boundary_types,
                             wob_scene *out) {
    if (!out) return fail(WOB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    std::unique_ptr<wob_scene_s> owner(new wob_scene_s());
    wob_scene_s *s = owner.get();
    std::string err = wobgb::build_host_scene(dim, n_elems, vertices, normals, boundary_values, robin_alphas,
                                              boundary_types, s->host);
    if (!err.empty()) {
        return fail(WOB_ERR_INVALID_ARGUMENT, err);
    }
    for (uint32_t i = 0; i < n_elems; i++)
        if (boundary_types[i] != WOB_DIRICHLET) s->all_dirichlet = false;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        return fail_cuda(e, "cudaGetDevice");
    }
    const wobgb::HostScene &h = s->host;
    s->area_G = (uint32_t)(h.area_guide.size() / 4);
    s->bv_G = (uint32_t)(h.bv_guide.size() / 4);
    const uint32_t zero = 0;
    if ((e = upload(s->elems, h.elems.data(), h.elems.size() * 4)) != cudaSuccess ||
        (e = upload(s->elem_aux, h.elem_aux.data(), h.elem_aux.size() * 4)) != cudaSuccess ||
        (e = upload(s->isect, h.isect.data(), h.isect.size() * 4)) != cudaSuccess ||
        (e = upload(s->nodes, h.nodes.data(), h.nodes.size() * 4)) != cudaSuccess ||
        (e = upload(s->area_cdf, h.area_cdf.data(), h.area_cdf.size() * 4)) != cudaSuccess ||
        (e = upload(s->area_guide, h.area_guide.data(), h.area_guide.size() * 4)) != cudaSuccess ||
        (e = upload(s->bv_cdf, h.bv_cdf.data(), h.bv_cdf.size() * 4)) != cudaSuccess ||
        (e = upload(s->bv_guide, h.bv_guide.data(), h.bv_guide.size() * 4)) != cudaSuccess ||
        (e = upload(s->err, &zero, 4)) != cudaSuccess ||
        (e = upload(s->lg_bins, h.line_grid.bins.data(), h.line_grid.bins.size() * 4)) != cudaSuccess ||
        (e = upload(s->lg_off, h.line_grid.offsets.data(), h.line_grid.offsets.size() * 4)) != cudaSuccess ||
        (e = upload(s->lg_ent, h.line_grid.entries.data(), h.line_grid.entries.size() * 2)) != cudaSuccess) {
        s->release_all();
        return fail_cuda(e, "uploading the scene");
    }
    *out = owner.release();
    return WOB_OK;
}

int wob_scene_create(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                     const float *boundary_values, const float *robin_alphas, const int32_t *boundary_types,
                     wob_scene *out) {
    return guarded([&] {
        return scene_create_impl(dim, n_elems, vertices, normals, boundary_values, robin_alphas, boundary_types, out);
    });
}

static int scene_create_device_impl(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                                    const float *boundary_values, const float *robin_alphas, const int32_t *boundary_types,
                                    void *stream, wob_scene *out) {
    if (!out) return fail(WOB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    std::unique_ptr<wob_scene_s> owner(new wob_scene_s());
    wob_scene_s *s = owner.get();
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        return fail_cuda(e, "cudaGetDevice");
    }
    wobgb::DeviceSceneBuild b;
    std::string err = wobgb::build_device_scene(dim, n_elems, vertices, normals, boundary_values, robin_alphas,
                                                boundary_types, (cudaStream_t)stream, b, e);
    if (!err.empty()) {
        return e != cudaSuccess ? fail_cuda(e, "building the scene on the device") : fail(WOB_ERR_INVALID_ARGUMENT, err);
    }
    auto take = [](DevBuf &d, void *p, size_t bytes) {
        d.ptr = p;
        d.bytes = bytes;
    };
    take(s->elems, b.elems, b.elems_bytes);
    take(s->elem_aux, b.elem_aux, b.elem_aux_bytes);
    take(s->isect, b.isect, b.isect_bytes);
    take(s->nodes, b.nodes, b.nodes_bytes);
    take(s->area_cdf, b.area_cdf, b.area_cdf_bytes);
    take(s->area_guide, b.area_guide, b.area_guide_bytes);
    take(s->bv_cdf, b.bv_cdf, b.bv_cdf_bytes);
    take(s->bv_guide, b.bv_guide, b.bv_guide_bytes);
    wobgb::HostScene &h = s->host;
    h.dim = dim;
    h.n = n_elems;
    h.order = std::move(b.order);
    h.n_nodes = b.n_nodes;
    h.depth = b.depth;
    h.total_area = b.total_area;
    h.total_bv = b.total_bv;
    h.bv_valid = b.bv_valid;
    s->all_dirichlet = b.all_dirichlet;
    s->area_G = b.area_G;
    s->bv_G = b.bv_G;
    const uint32_t zero = 0;
    if ((e = upload(s->err, &zero, 4)) != cudaSuccess) {
        s->release_all();
        return fail_cuda(e, "allocating the error word");
    }
    *out = owner.release();
    return WOB_OK;
}

int wob_scene_create_device(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                            const float *boundary_values, const float *robin_alphas, const int32_t *boundary_types,
                            void *stream, wob_scene *out) {
    return guarded([&] {
        return scene_create_device_impl(dim, n_elems, vertices, normals, boundary_values, robin_alphas, boundary_types,
                                        stream, out);
    });
}

int wob_scene_destroy(wob_scene s) {
    if (!s) return WOB_OK;
    {
        DeviceGuard g(s->device);
        s->release_all();
    }
    delete s;
    return WOB_OK;
}

int wob_scene_get_info(wob_scene s, wob_scene_info *info) {
    if (!s || !info) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and info are required");
    info->dim = s->host.dim;
    info->n_elems = s->host.n;
    info->n_nodes = s->host.n_nodes;
    info->bvh_depth = s->host.depth;
    info->total_area = s->host.total_area;
    info->total_boundary_value = s->host.total_bv;
    info->has_volume_cache = s->has_volume ? 1 : 0;
    size_t bytes = 0;
    for (const DevBuf *b : {&s->elems, &s->elem_aux, &s->isect, &s->nodes, &s->area_cdf, &s->area_guide, &s->bv_cdf, &s->bv_guide,
                            &s->vol_values, &s->vol_cdf, &s->vol_guide, &s->lg_bins, &s->lg_off, &s->lg_ent})
        bytes += b->bytes;
    info->bytes_on_device = (uint32_t)(bytes > 0xFFFFFFFFu ? 0xFFFFFFFFu : bytes);
    info->line_grid_bins = s->lg_bins.ptr ? s->host.line_grid.K : 0u;
    info->line_grid_cells = s->lg_bins.ptr ? s->host.line_grid.M : 0u;
    return WOB_OK;
}

int wob_scene_get_element_order(wob_scene s, uint32_t *order) {
    if (!s || !order) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and order are required");
    std::memcpy(order, s->host.order.data(), s->host.order.size() * 4);
    return WOB_OK;
}

static int scene_set_volume_cache_impl(wob_scene s, uint32_t grid_res, float domain_size, const float *values) {
    if (!s || !values) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and values are required");
    if (grid_res < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "grid_res must be >= 1");
    if (!(domain_size > 0.0f) || !(domain_size < 3.0e38f)) return fail(WOB_ERR_INVALID_ARGUMENT, "domain_size must be positive and finite");
    const int dim = s->host.dim;
    uint64_t n = 1;
    for (int i = 0; i < dim; i++) n *= grid_res;
    if (n > (1ull << 30)) return fail(WOB_ERR_INVALID_ARGUMENT, "volume cache too large");
    std::vector<float> cdf;
    std::string err = wobgb::build_volume_cdf(dim, grid_res, values, cdf);
    if (!err.empty()) return fail(WOB_ERR_INVALID_ARGUMENT, err);
    std::vector<uint32_t> guide = wobgb::build_guide(cdf);
    DeviceGuard g(s->device);
    cudaError_t e;
    if ((e = upload(s->vol_values, values, n * 4)) != cudaSuccess || (e = upload(s->vol_cdf, cdf.data(), n * 4)) != cudaSuccess ||
        (e = upload(s->vol_guide, guide.data(), guide.size() * 4)) != cudaSuccess) {
        s->vol_values.release();
        s->vol_cdf.release();
        s->vol_guide.release();
        s->has_volume = false;
        return fail_cuda(e, "uploading the volume cache");
    }
    s->has_volume = true;
    s->vol_res = grid_res;
    s->vol_n = (uint32_t)n;
    s->vol_G = (uint32_t)(guide.size() / 4);
    s->vol_size = domain_size;
    return WOB_OK;
}

int wob_scene_set_volume_cache(wob_scene s, uint32_t grid_res, float domain_size, const float *values) {
    return guarded([&] { return scene_set_volume_cache_impl(s, grid_res, domain_size, values); });
}

int wob_scene_clear_volume_cache(wob_scene s) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    DeviceGuard g(s->device);
    s->vol_values.release();
    s->vol_cdf.release();
    s->vol_guide.release();
    s->has_volume = false;
    s->vol_res = s->vol_n = s->vol_G = 0;
    return WOB_OK;
}

static int solve_domain_impl(wob_scene s, const wob_params *params, const float *points, uint32_t n_points,
                             double *sum, double *sumsq, uint64_t *bounces, float *per_path, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (n_points == 0) return WOB_OK;
    if (!points) return fail(WOB_ERR_INVALID_ARGUMENT, "points is NULL");
    if (!per_path && !sum) return fail(WOB_ERR_INVALID_ARGUMENT, "sum is NULL");
    DeviceGuard g(s->device);
    cudaError_t e;
    if (s->host.dim == 2)
        e = wobgb::launch_domain_2d(s->view<2>(), w, points, n_points, sum, sumsq, (unsigned long long *)bounces,
                                    per_path, (cudaStream_t)stream);
    else
        e = wobgb::launch_domain_3d(s->view<3>(), w, points, n_points, sum, sumsq, (unsigned long long *)bounces,
                                    per_path, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail_cuda(e, "launching the domain walk");
    return WOB_OK;
}

int wob_solve_domain(wob_scene s, const wob_params *params, const float *points, uint32_t n_points, double *sum,
                     double *sumsq, uint64_t *bounces, void *stream) {
    return solve_domain_impl(s, params, points, n_points, sum, sumsq, bounces, nullptr, stream);
}

int wob_debug_domain_paths(wob_scene s, const wob_params *params, const float *points, uint32_t n_points,
                           float *values, void *stream) {
    if (!values) return fail(WOB_ERR_INVALID_ARGUMENT, "values is NULL");
    return solve_domain_impl(s, params, points, n_points, nullptr, nullptr, nullptr, values, stream);
}

static int solve_domain_host_impl(wob_scene s, const wob_params *params, const float *points, uint32_t n_points, double *sum,
                                  double *sumsq, uint64_t *bounces) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (n_points == 0) return WOB_OK;
    if (!points || !sum) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum are required");
    const int D = s->host.dim;
    const size_t pts_bytes = (size_t)n_points * D * 4, out_bytes = (size_t)n_points * (D + 1) * 8;
    const size_t off_sum = (pts_bytes + 255) / 256 * 256;
    const size_t off_sq = off_sum + (out_bytes + 255) / 256 * 256;
    const size_t off_b = off_sq + (out_bytes + 255) / 256 * 256;
    const size_t total = off_b + 256;
    std::lock_guard<std::mutex> lock(s->ws_mutex);
    DeviceGuard g(s->device);
    cudaError_t e;
    if (!s->ws_stream && (e = cudaStreamCreateWithFlags(&s->ws_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail_cuda(e, "cudaStreamCreate");
    if (s->ws.bytes < total) {
        s->ws.release();
        if ((e = cudaMalloc(&s->ws.ptr, total)) != cudaSuccess) return fail_cuda(e, "cudaMalloc workspace");
        s->ws.bytes = total;
    }
    char *base = (char *)s->ws.ptr;
    float *d_pts = (float *)base;
    double *d_sum = (double *)(base + off_sum);
    double *d_sq = (double *)(base + off_sq);
    uint64_t *d_b = (uint64_t *)(base + off_b);
    cudaStream_t st_ = s->ws_stream;
    if ((e = cudaMemcpyAsync(d_pts, points, pts_bytes, cudaMemcpyHostToDevice, st_)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_sum, 0, out_bytes, st_)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_sq, 0, out_bytes, st_)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_b, 0, 8, st_)) != cudaSuccess)
        return fail_cuda(e, "staging inputs");
    e = D == 2 ? wobgb::launch_domain_2d(s->view<2>(), w, d_pts, n_points, d_sum, sumsq ? d_sq : nullptr,
                                         (unsigned long long *)d_b, nullptr, st_)
               : wobgb::launch_domain_3d(s->view<3>(), w, d_pts, n_points, d_sum, sumsq ? d_sq : nullptr,
                                         (unsigned long long *)d_b, nullptr, st_);
    if (e != cudaSuccess) return fail_cuda(e, "launching the domain walk");
    std::vector<double> tmp((size_t)n_points * (D + 1));
    uint64_t b = 0;
    uint32_t errw = 0;
    if ((e = cudaMemcpyAsync(tmp.data(), d_sum, out_bytes, cudaMemcpyDeviceToHost, st_)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&b, d_b, 8, cudaMemcpyDeviceToHost, st_)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&errw, s->err.ptr, 4, cudaMemcpyDeviceToHost, st_)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st_)) != cudaSuccess)
        return fail_cuda(e, "reading results");
    for (size_t i = 0; i < tmp.size(); i++) sum[i] += tmp[i];
    if (sumsq) {
        if ((e = cudaMemcpyAsync(tmp.data(), d_sq, out_bytes, cudaMemcpyDeviceToHost, st_)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st_)) != cudaSuccess)
            return fail_cuda(e, "reading results");
        for (size_t i = 0; i < tmp.size(); i++) sumsq[i] += tmp[i];
    }
    if (bounces) *bounces += b;
    if (errw) return fail(WOB_ERR_DEVICE_LIMIT, "a BVH traversal hit its stack or step bound");
    return WOB_OK;
}

int wob_solve_domain_host(wob_scene s, const wob_params *params, const float *points, uint32_t n_points, double *sum,
                          double *sumsq, uint64_t *bounces) {
    return guarded([&] { return solve_domain_host_impl(s, params, points, n_points, sum, sumsq, bounces); });
}

static int solve_boundary_impl(wob_scene s, const wob_params *params, const float *p, const float *n,
                               const float *interior_angle, const float *boundary_value,
                               const int32_t *boundary_type, const float *robin_alpha, uint32_t n_points,
                               double *sum, double *sumsq, uint64_t *bounces, float *per_path, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (n_points == 0) return WOB_OK;
    if (!p || !n || !interior_angle || !boundary_value || !boundary_type)
        return fail(WOB_ERR_INVALID_ARGUMENT, "p, n, interior_angle, boundary_value and boundary_type are required");
    if (!per_path && !sum) return fail(WOB_ERR_INVALID_ARGUMENT, "sum is NULL");
    wobgb::BoundaryInput bin{p, n, interior_angle, boundary_value, boundary_type, robin_alpha};
    DeviceGuard g(s->device);
    cudaError_t e;
    if (s->host.dim == 2)
        e = wobgb::launch_boundary_2d(s->view<2>(), w, bin, n_points, sum, sumsq, (unsigned long long *)bounces,
                                      per_path, (cudaStream_t)stream);
    else
        e = wobgb::launch_boundary_3d(s->view<3>(), w, bin, n_points, sum, sumsq, (unsigned long long *)bounces,
                                      per_path, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail_cuda(e, "launching the boundary walk");
    return WOB_OK;
}

int wob_solve_boundary(wob_scene s, const wob_params *params, const float *p, const float *n,
                       const float *interior_angle, const float *boundary_value, const int32_t *boundary_type,
                       const float *robin_alpha, uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                       void *stream) {
    return solve_boundary_impl(s, params, p, n, interior_angle, boundary_value, boundary_type, robin_alpha, n_points,
                               sum, sumsq, bounces, nullptr, stream);
}

int wob_debug_boundary_paths(wob_scene s, const wob_params *params, const float *p, const float *n,
                             const float *interior_angle, const float *boundary_value, const int32_t *boundary_type,
                             const float *robin_alpha, uint32_t n_points, float *values, void *stream) {
    if (!values) return fail(WOB_ERR_INVALID_ARGUMENT, "values is NULL");
    return solve_boundary_impl(s, params, p, n, interior_angle, boundary_value, boundary_type, robin_alpha, n_points,
                               nullptr, nullptr, nullptr, values, stream);
}

int wob_line_query(wob_scene s, const float *origins, const float *dirs, uint32_t n_rays, uint32_t *counts,
                   uint32_t *hits, float *hit_points, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n_rays == 0) return WOB_OK;
    if (!origins || !dirs || !counts || !hits) return fail(WOB_ERR_INVALID_ARGUMENT, "origins, dirs, counts and hits are required");
    DeviceGuard g(s->device);
    cudaError_t e = s->host.dim == 2
                        ? wobgb::launch_line_query_2d(s->view<2>(), origins, dirs, n_rays, counts, hits, hit_points, (cudaStream_t)stream)
                        : wobgb::launch_line_query_3d(s->view<3>(), origins, dirs, n_rays, counts, hits, hit_points, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail_cuda(e, "launching the line query");
    return WOB_OK;
}

int wob_scene_poll_error(wob_scene s, uint32_t *bits) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    DeviceGuard g(s->device);
    uint32_t v = 0;
    cudaError_t e = cudaMemcpy(&v, s->err.ptr, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail_cuda(e, "reading the error word");
    const uint32_t zero = 0;
    if (v && (e = cudaMemcpy(s->err.ptr, &zero, 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail_cuda(e, "clearing the error word");
    if (bits) *bits = v;
    return WOB_OK;
}

int wob_noalloc_max_points(int dim, uint32_t *max_points) {
    if ((dim != 2 && dim != 3) || !max_points) return fail(WOB_ERR_INVALID_ARGUMENT, "dim must be 2 or 3 and max_points non-NULL");
    *max_points = noalloc_max_points(dim);
    return WOB_OK;
}

static int solve_domain_host_noalloc_impl(wob_scene s, const wob_params *params, const float *points,
                                         uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                                         void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    w.no_alloc = 1;  // kernels whose launchers allocate (the forward wavefront) are not chosen
    if (n_points == 0) return WOB_OK;
    if (!points || !sum) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum are required");
    const int D = s->host.dim;
    const uint32_t max_points = noalloc_max_points(D);
    if (n_points > max_points)
        return fail(WOB_ERR_INVALID_ARGUMENT, "n_points = " + std::to_string(n_points) + " exceeds the no-allocation limit of " +
                                                  std::to_string(max_points) + " points for dim " + std::to_string(D) +
                                                  " (16 MiB static device scratch); split the points or use wob_solve_domain_host");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    DeviceGuard g(s->device);
    void *base_v = nullptr;
    if ((st = noalloc_scratch(s->device, &base_v)) != WOB_OK) return st;
    char *base = (char *)base_v;
    size_t off[4];
    noalloc_bytes(D, n_points, off);
    float *d_pts = (float *)(base + off[0]);
    double *d_sum = (double *)(base + off[1]);
    double *d_sq = (double *)(base + off[2]);
    uint64_t *d_b = (uint64_t *)(base + off[3]);
    const size_t pts_bytes = (size_t)n_points * D * 4, out_bytes = (size_t)n_points * (D + 1) * 8;
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e;
    // The array keeps the previous call's contents: the sums are loaded from the caller's arrays
    // (the solve accumulates into them) and the bounce counter is cleared.
    if ((e = cudaMemcpyAsync(d_pts, points, pts_bytes, cudaMemcpyHostToDevice, cs)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_sum, sum, out_bytes, cudaMemcpyHostToDevice, cs)) != cudaSuccess ||
        (sumsq && (e = cudaMemcpyAsync(d_sq, sumsq, out_bytes, cudaMemcpyHostToDevice, cs)) != cudaSuccess) ||
        (e = cudaMemsetAsync(d_b, 0, 8, cs)) != cudaSuccess)
        return fail_cuda(e, "staging inputs in the no-allocation scratch");
    e = D == 2 ? wobgb::launch_domain_2d(s->view<2>(), w, d_pts, n_points, d_sum, sumsq ? d_sq : nullptr,
                                         (unsigned long long *)d_b, nullptr, cs)
               : wobgb::launch_domain_3d(s->view<3>(), w, d_pts, n_points, d_sum, sumsq ? d_sq : nullptr,
                                         (unsigned long long *)d_b, nullptr, cs);
    if (e != cudaSuccess) return fail_cuda(e, "launching the domain walk");
    uint64_t b = 0;
    uint32_t errw = 0;
    if ((e = cudaMemcpyAsync(sum, d_sum, out_bytes, cudaMemcpyDeviceToHost, cs)) != cudaSuccess ||
        (sumsq && (e = cudaMemcpyAsync(sumsq, d_sq, out_bytes, cudaMemcpyDeviceToHost, cs)) != cudaSuccess) ||
        (e = cudaMemcpyAsync(&b, d_b, 8, cudaMemcpyDeviceToHost, cs)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&errw, s->err.ptr, 4, cudaMemcpyDeviceToHost, cs)) != cudaSuccess ||
        (e = cudaStreamSynchronize(cs)) != cudaSuccess)
        return fail_cuda(e, "reading results from the no-allocation scratch");
    if (bounces) *bounces += b;
    if (errw) return fail(WOB_ERR_DEVICE_LIMIT, "a BVH traversal hit its stack or step bound");
    return WOB_OK;
}

int wob_solve_domain_host_noalloc(wob_scene s, const wob_params *params, const float *points, uint32_t n_points,
                                  double *sum, double *sumsq, uint64_t *bounces, void *stream) {
    return guarded([&] {
        return solve_domain_host_noalloc_impl(s, params, points, n_points, sum, sumsq, bounces, stream);
    });
}

int wob_autotune_domain(wob_scene s, const wob_params *params, const float *points, uint32_t n_points,
                        int32_t *chosen, float *ms_per_config, int32_t *n_configs, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    const int D = s->host.dim;
    const int v = wobgb::tunable_domain_variant(D, w);
    if (chosen) *chosen = -1;
    if (n_configs) *n_configs = 0;
    if (v < 0 || n_points == 0) return WOB_OK;
    if (!points) return fail(WOB_ERR_INVALID_ARGUMENT, "points is NULL");
    // Time each configuration on enough points for about 2^23 paths (or all points), with the paths
    // per lane that a launch over all n_points would choose (a subset would choose fewer).
    const uint64_t want = ((1ull << 23) + w.n_paths - 1) / w.n_paths;
    const uint32_t n_sub = (uint32_t)(want < n_points ? want : n_points);
    w.ppt_points = n_points;
    DeviceGuard g(s->device);
    cudaStream_t cs = (cudaStream_t)stream;
    double *tmp = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&tmp, (size_t)n_sub * (D + 1) * 8)) != cudaSuccess) return fail_cuda(e, "cudaMalloc (autotune)");
    if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaFree(tmp);
        return fail_cuda(e, "cudaEventCreate");
    }
    const wobgb::SceneView<2> v2 = s->view<2>();
    const wobgb::SceneView<3> v3 = s->view<3>();
    const void *view = D == 2 ? (const void *)&v2 : (const void *)&v3;
    int best = 0;
    float best_ms = 3.0e38f;
    for (int c = 0; c < wobgb::kTuneConfigs && e == cudaSuccess; c++) {
        e = wobgb::launch_domain_config(D, v, c, view, w, points, n_sub, tmp, nullptr, nullptr, nullptr, cs);
        if (e != cudaSuccess) break;
        cudaEventRecord(e0, cs);
        for (int r = 0; r < 2 && e == cudaSuccess; r++)
            e = wobgb::launch_domain_config(D, v, c, view, w, points, n_sub, tmp, nullptr, nullptr, nullptr, cs);
        cudaEventRecord(e1, cs);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        ms *= 0.5f;
        if (ms_per_config) ms_per_config[c] = ms;
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail_cuda(e, "autotuning");
    wobgb::set_domain_config(v, best);
    if (chosen) *chosen = best;
    if (n_configs) *n_configs = wobgb::kTuneConfigs;
    return WOB_OK;
}

int wob_set_domain_config(int32_t variant, int32_t config) {
    if (variant < 0 || variant >= wobgb::kNumTunable || config < 0 || config >= wobgb::kTuneConfigs)
        return fail(WOB_ERR_INVALID_ARGUMENT, "variant or config out of range");
    wobgb::set_domain_config(variant, config);
    return WOB_OK;
}

int wob_get_domain_config(int32_t variant, int32_t *config) {
    if (variant < 0 || variant >= wobgb::kNumTunable || !config) return fail(WOB_ERR_INVALID_ARGUMENT, "variant out of range or config NULL");
    *config = wobgb::domain_config(variant);
    return WOB_OK;
}

int wob_tunable_variant(wob_scene s, const wob_params *params, int32_t *variant) {
    if (!s || !variant) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and variant are required");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    *variant = wobgb::tunable_domain_variant(s->host.dim, w);
    return WOB_OK;
}

static int batch_create_impl(const wob_scene *scenes, const wob_params *params, const uint32_t *n_points, uint32_t n_scenes,
                             wob_batch *out) {
    if (!out || !scenes || !params || !n_points || n_scenes == 0)
        return fail(WOB_ERR_INVALID_ARGUMENT, "scenes, params, n_points and out are required, n_scenes >= 1");
    *out = nullptr;
    const int dim = scenes[0] ? scenes[0]->host.dim : 0;
    const int device = scenes[0] ? scenes[0]->device : 0;
    std::vector<wobgb::BatchEntry<2>> t2;
    std::vector<wobgb::BatchEntry<3>> t3;
    uint64_t units = 0, points = 0;
    for (uint32_t i = 0; i < n_scenes; i++) {
        const wob_scene_s *s = scenes[i];
        if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene " + std::to_string(i) + " is NULL");
        if (s->host.dim != dim || s->device != device)
            return fail(WOB_ERR_INVALID_ARGUMENT, "all scenes of a batch need the same dimension and device");
        wobgb::WalkParams w;
        int st = check_params(s, params + i, w);
        if (st != WOB_OK) return fail(st, "scene " + std::to_string(i) + ": " + g_last_error);
        w.ppt = wobgb::choose_ppt(n_points[i], w.n_paths);
        const uint32_t slabs = (w.n_paths + 32u * w.ppt - 1u) / (32u * w.ppt);
        if (dim == 2) {
            wobgb::BatchEntry<2> e{};
            e.view = s->view<2>(); e.params = w; e.unit_begin = units; e.point_begin = (uint32_t)points;
            e.n_points = n_points[i]; e.slabs = slabs; e.cls = wobgb::batch_walk_class(w);
            t2.push_back(e);
        } else {
            wobgb::BatchEntry<3> e{};
            e.view = s->view<3>(); e.params = w; e.unit_begin = units; e.point_begin = (uint32_t)points;
            e.n_points = n_points[i]; e.slabs = slabs; e.cls = wobgb::batch_walk_class(w);
            t3.push_back(e);
        }
        units += (uint64_t)n_points[i] * slabs;
        points += n_points[i];
        if (points > 0xFFFFFFFFull) return fail(WOB_ERR_INVALID_ARGUMENT, "a batch holds at most 2^32 - 1 points");
    }
    std::unique_ptr<wob_batch_s> owner(new wob_batch_s());
    wob_batch_s *b = owner.get();
    b->device = device;
    b->dim = dim;
    b->n_scenes = n_scenes;
    b->total_units = units;
    b->total_points = (uint32_t)points;
    // group by walk class, keeping the caller's order within a class; unit numbers per class
    auto group = [b](auto &t) {
        std::stable_sort(t.begin(), t.end(), [](const auto &x, const auto &y) { return x.cls < y.cls; });
        uint32_t first = 0;
        for (uint32_t c = 0; c < 3; c++) {
            uint64_t u = 0;
            uint32_t k = first;
            while (k < t.size() && t[k].cls == c) {
                t[k].unit_begin = u;
                u += (uint64_t)t[k].n_points * t[k].slabs;
                k++;
            }
            b->cls_first[c] = first;
            b->cls_count[c] = k - first;
            b->cls_units[c] = u;
            first = k;
        }
    };
    if (dim == 2) group(t2);
    else group(t3);
    DeviceGuard g(device);
    cudaError_t e = dim == 2 ? upload(b->table, t2.data(), t2.size() * sizeof(t2[0]))
                             : upload(b->table, t3.data(), t3.size() * sizeof(t3[0]));
    if (e != cudaSuccess) {
        return fail_cuda(e, "uploading the batch table");
    }
    *out = owner.release();
    return WOB_OK;
}

int wob_batch_create(const wob_scene *scenes, const wob_params *params, const uint32_t *n_points, uint32_t n_scenes,
                     wob_batch *out) {
    return guarded([&] { return batch_create_impl(scenes, params, n_points, n_scenes, out); });
}

int wob_batch_solve(wob_batch b, const float *points, double *sum, double *sumsq, uint64_t *bounces,
                    uint64_t path_offset_add, void *stream) {
    if (!b) return fail(WOB_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->total_points == 0) return WOB_OK;
    if (!points || !sum) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum are required");
    DeviceGuard g(b->device);
    cudaError_t e = cudaSuccess;
    for (uint32_t c = 0; c < 3 && e == cudaSuccess; c++) {
        if (b->cls_count[c] == 0 || b->cls_units[c] == 0) continue;
        e = b->dim == 2
            ? wobgb::launch_batch_2d((const wobgb::BatchEntry<2> *)b->table.ptr + b->cls_first[c], b->cls_count[c], c,
                                     b->cls_units[c], points, sum, sumsq, (unsigned long long *)bounces,
                                     path_offset_add, (cudaStream_t)stream)
            : wobgb::launch_batch_3d((const wobgb::BatchEntry<3> *)b->table.ptr + b->cls_first[c], b->cls_count[c], c,
                                     b->cls_units[c], points, sum, sumsq, (unsigned long long *)bounces,
                                     path_offset_add, (cudaStream_t)stream);
    }
    if (e != cudaSuccess) return fail_cuda(e, "launching the batched walk");
    return WOB_OK;
}

int wob_batch_destroy(wob_batch b) {
    if (!b) return WOB_OK;
    {
        DeviceGuard g(b->device);
        b->table.release();
    }
    delete b;
    return WOB_OK;
}

// ---- residual control variate (k_cv_tables.cu)

namespace {
// Copies a device buffer of the scene into a new allocation (empty buffers stay empty).
cudaError_t clone_buf(DevBuf &dst, const DevBuf &src) {
    dst.release();
    if (!src.ptr || src.bytes == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&dst.ptr, src.bytes);
    if (e != cudaSuccess) return e;
    dst.bytes = src.bytes;
    return cudaMemcpy(dst.ptr, src.ptr, src.bytes, cudaMemcpyDeviceToDevice);
}

int scene_clone_impl(wob_scene src, wob_scene *out) {
    if (!src || !out) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and out are required");
    *out = nullptr;
    DeviceGuard g(src->device);
    std::unique_ptr<wob_scene_s> owner(new wob_scene_s());
    wob_scene_s *s = owner.get();
    s->device = src->device;
    // host copy: what wob_scene_add_boundary_offsets and a further clone read (the element records,
    // areas, storage order, |g| tables and scalars); the BVH, intersection records, area tables and
    // line grid stay on the device only, shared with the source
    const wobgb::HostScene &h0 = src->host;
    wobgb::HostScene &h = s->host;
    h.dim = h0.dim;
    h.n = h0.n;
    h.order = h0.order;
    h.elems = h0.elems;
    h.elem_aux = h0.elem_aux;
    h.alpha_const = h0.alpha_const;
    h.alpha_value = h0.alpha_value;
    h.bv_cdf = h0.bv_cdf;
    h.bv_guide = h0.bv_guide;
    h.total_area = h0.total_area;
    h.total_bv = h0.total_bv;
    h.bv_valid = h0.bv_valid;
    h.n_nodes = h0.n_nodes;
    h.depth = h0.depth;
    h.line_grid.K = h0.line_grid.K;
    h.line_grid.M = h0.line_grid.M;
    h.line_grid.cx = h0.line_grid.cx;
    h.line_grid.cy = h0.line_grid.cy;
    h.line_grid.far = h0.line_grid.far;
    s->has_volume = src->has_volume;
    s->area_G = src->area_G;
    s->bv_G = src->bv_G;
    s->vol_res = src->vol_res;
    s->vol_n = src->vol_n;
    s->vol_G = src->vol_G;
    s->vol_size = src->vol_size;
    s->all_dirichlet = src->all_dirichlet;
    // shared: buffers that no entry point writes in place (a later upload to either scene, such as
    // the |g| tables wob_scene_add_boundary_offsets rebuilds, replaces that scene's reference
    // only); copied: the element records, which wob_scene_add_boundary_offsets updates in place
    for (auto b : {&wob_scene_s::elem_aux, &wob_scene_s::isect, &wob_scene_s::nodes, &wob_scene_s::area_cdf,
                   &wob_scene_s::area_guide, &wob_scene_s::bv_cdf, &wob_scene_s::bv_guide, &wob_scene_s::vol_values,
                   &wob_scene_s::vol_cdf, &wob_scene_s::vol_guide, &wob_scene_s::lg_bins, &wob_scene_s::lg_off,
                   &wob_scene_s::lg_ent})
        share(s->*b, src->*b);
    cudaError_t e = clone_buf(s->elems, src->elems);
    if (e != cudaSuccess) {
        s->release_all();
        return fail_cuda(e, "copying the scene");
    }
    const uint32_t zero = 0;
    if ((e = upload(s->err, &zero, 4)) != cudaSuccess) {
        s->release_all();
        return fail_cuda(e, "allocating the error word");
    }
    *out = owner.release();
    return WOB_OK;
}

int scene_add_boundary_offsets_impl(wob_scene s, const float *delta, uint32_t n, int on_device, void *stream) {
    if (!s || !delta) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and delta are required");
    if (n != s->host.n) return fail(WOB_ERR_INVALID_ARGUMENT, "need one offset per element");
    if (s->host.elems.empty()) return fail(WOB_ERR_UNSUPPORTED, "the scene keeps no host records (built on the device)");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> d(n);
    cudaError_t e;
    if (on_device) {
        if ((e = cudaMemcpyAsync(d.data(), delta, (size_t)n * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail_cuda(e, "reading the offsets");
    } else {
        std::memcpy(d.data(), delta, (size_t)n * 4);
    }
    for (uint32_t i = 0; i < n; i++)
        if (!(d[i] == d[i]) || d[i] > 3.0e38f || d[i] < -3.0e38f)
            return fail(WOB_ERR_INVALID_ARGUMENT, "offsets must be finite");
    wobgb::HostScene &h = s->host;
    const int EF = wobgb::elem_record_floats(h.dim);
    const int first = h.dim == 2 ? 6 : 12;
    for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < h.dim; k++) h.elems[(size_t)i * EF + first + k] = h.elems[(size_t)i * EF + first + k] + d[i];
    // the device records get the same adds (offsets read from the caller's device buffer, or from
    // a scratch copy of the host array)
    DevBuf scratch;
    const float *dd = delta;
    if (!on_device) {
        if ((e = upload(scratch, d.data(), (size_t)n * 4)) != cudaSuccess) return fail_cuda(e, "uploading the offsets");
        dd = (const float *)scratch.ptr;
    }
    e = wobgb::launch_add_boundary_offsets((float *)s->elems.ptr, dd, n, (uint32_t)EF, (uint32_t)first,
                                           (uint32_t)h.dim, st);
    wobgb::rebuild_bv_tables(h);
    s->bv_G = (uint32_t)(h.bv_guide.size() / 4);
    if (e != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess ||
        (e = upload(s->bv_cdf, h.bv_cdf.data(), h.bv_cdf.size() * 4)) != cudaSuccess ||
        (e = upload(s->bv_guide, h.bv_guide.data(), h.bv_guide.size() * 4)) != cudaSuccess) {
        scratch.release();
        return fail_cuda(e, "updating the boundary values");
    }
    scratch.release();
    return WOB_OK;
}

// Triangle sources and clusters of sigma~ in a scratch allocation freed on return.
struct CvSources {
    DevBuf src, near2, clusters;
};
int cv_sources(wob_scene s, const float *sigma, float near_factor, float theta, CvSources &cs, cudaStream_t st) {
    if (s->host.dim != 3) return fail(WOB_ERR_UNSUPPORTED, "the control-variate tables are implemented for 3D scenes");
    if (!sigma) return fail(WOB_ERR_INVALID_ARGUMENT, "sigma is required");
    if (!(near_factor >= 0.0f) || !(near_factor < 1e6f)) return fail(WOB_ERR_INVALID_ARGUMENT, "near_factor must be in [0, 1e6)");
    if (!(theta >= 0.0f) || !(theta < 1.0f)) return fail(WOB_ERR_INVALID_ARGUMENT, "theta must be in [0, 1)");
    const size_t n = s->host.n;
    const size_t n_rec = wobgb::cv_cluster_records((uint32_t)n);  // clusters and their two group levels
    cudaError_t e;
    if ((e = cudaMalloc(&cs.src.ptr, n * 16)) != cudaSuccess || (e = cudaMalloc(&cs.near2.ptr, n * 4)) != cudaSuccess ||
        (e = cudaMalloc(&cs.clusters.ptr, n_rec * 64)) != cudaSuccess)
        return fail_cuda(e, "allocating the control-variate sources");
    cs.src.bytes = n * 16;
    cs.near2.bytes = n * 4;
    cs.clusters.bytes = n_rec * 64;
    e = wobgb::launch_cv_sources(s->view<3>(), sigma, near_factor, theta, (float4 *)cs.src.ptr, (float *)cs.near2.ptr,
                                 (float4 *)cs.clusters.ptr, st);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the control-variate sources");
}
}  // namespace

int wob_scene_set_step_limits(wob_scene s, uint32_t max_traversal_steps, uint32_t max_wos_jumps) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (max_wos_jumps > wobgb::kWosMaxSteps) return fail(WOB_ERR_INVALID_ARGUMENT, "max_wos_jumps above the 4096 bound");
    s->traversal_limit = max_traversal_steps;
    s->wos_limit = max_wos_jumps;
    return WOB_OK;
}

int wob_measure_gather_peak(uint32_t n_records, uint32_t n_guide, uint32_t iters, double *samples_per_s, float *ms) {
    if (!samples_per_s || !ms || n_records == 0 || n_guide == 0 || iters == 0)
        return fail(WOB_ERR_INVALID_ARGUMENT, "n_records, n_guide, iters > 0 and the outputs are required");
    if (n_records > (1u << 26) || n_guide > (1u << 26)) return fail(WOB_ERR_INVALID_ARGUMENT, "tables too large");
    int dev = 0, sms = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess || (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return fail_cuda(e, "querying the device");
    e = wobgb::measure_gather_peak(n_records, n_guide, iters, sms, samples_per_s, ms);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "measuring the gather ceiling");
}

int wob_scene_sample_boundary(wob_scene s, uint32_t n, uint64_t seed, float *p, float *normals, float *interior_angle,
                              float *boundary_value, int32_t *boundary_type, float *robin_alpha, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n == 0) return WOB_OK;
    if (!p || !normals || !interior_angle || !boundary_value || !boundary_type)
        return fail(WOB_ERR_INVALID_ARGUMENT, "p, normals, interior_angle, boundary_value and boundary_type are required");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = s->host.dim == 2 ? wobgb::launch_sample_boundary<2>(s->view<2>(), n, seed, p, normals, interior_angle,
                                                                        boundary_value, boundary_type, robin_alpha, st)
                                     : wobgb::launch_sample_boundary<3>(s->view<3>(), n, seed, p, normals, interior_angle,
                                                                        boundary_value, boundary_type, robin_alpha, st);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the boundary sampler");
}

int wob_clip_magnitude_quantile(float *values, uint32_t n, float quantile, float *threshold, void *stream) {
    if (n == 0) return WOB_OK;
    if (!values) return fail(WOB_ERR_INVALID_ARGUMENT, "values is NULL");
    if (!(quantile > 0.0f && quantile <= 1.0f)) return fail(WOB_ERR_INVALID_ARGUMENT, "quantile must be in (0, 1]");
    cudaError_t e = wobgb::launch_clip_quantile(values, n, quantile, threshold, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "clipping the values");
}

int wob_scene_element_frames(wob_scene s, float *out, void *stream) {
    if (!s || !out) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and out are required");
    DeviceGuard g(s->device);
    cudaError_t e = s->host.dim == 2 ? wobgb::launch_element_frames<2>(s->view<2>(), out, (cudaStream_t)stream)
                                     : wobgb::launch_element_frames<3>(s->view<3>(), out, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the element frames");
}

int wob_scene_clone(wob_scene scene, wob_scene *out) {
    return guarded([&] { return scene_clone_impl(scene, out); });
}

int wob_scene_add_boundary_offsets(wob_scene scene, const float *delta, uint32_t n_elems, int delta_on_device,
                                   void *stream) {
    return guarded([&] { return scene_add_boundary_offsets_impl(scene, delta, n_elems, delta_on_device, stream); });
}

int wob_cv_residual_data(wob_scene s, const float *sigma, int domain, float near_factor, float theta, float *delta,
                         void *stream) {
    return guarded([&] {
        if (!s || !delta) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and delta are required");
        if (domain != WOB_INTERIOR_DOMAIN && domain != WOB_EXTERIOR_DOMAIN)
            return fail(WOB_ERR_INVALID_ARGUMENT, "domain must be 0 (interior) or 1 (exterior)");
        DeviceGuard g(s->device);
        cudaStream_t st = (cudaStream_t)stream;
        CvSources cs;
        int r = cv_sources(s, sigma, near_factor, theta, cs, st);
        if (r == WOB_OK) {
            // c = domain_type_coefficient / integral_free_term(1/2) (bie_models.cuh:66-78)
            const float c = domain == WOB_INTERIOR_DOMAIN ? 2.0f : -2.0f;
            cudaError_t e = wobgb::launch_cv_residual(s->view<3>(), (const float4 *)cs.src.ptr, (const float *)cs.near2.ptr,
                                                      (const float4 *)cs.clusters.ptr, sigma, c, delta, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) r = fail_cuda(e, "computing the residual data");
        }
        cs.src.release();
        cs.near2.release();
        cs.clusters.release();
        return r;
    });
}

int wob_cv_potential(wob_scene s, const float *sigma, float near_factor, float theta, const float *points,
                     uint32_t n_points, float *out, void *stream) {
    return guarded([&] {
        if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
        if (n_points == 0) return (int)WOB_OK;
        if (!points || !out) return fail(WOB_ERR_INVALID_ARGUMENT, "points and out are required");
        DeviceGuard g(s->device);
        cudaStream_t st = (cudaStream_t)stream;
        CvSources cs;
        DevBuf order;
        int r = cv_sources(s, sigma, near_factor, theta, cs, st);
        if (r == WOB_OK) {
            const size_t words = wobgb::cv_point_order_words(n_points);
            cudaError_t e = cudaMalloc(&order.ptr, words * 4);
            if (e == cudaSuccess) {
                order.bytes = words * 4;
                e = wobgb::launch_cv_potential(s->view<3>(), (const float4 *)cs.src.ptr, (const float *)cs.near2.ptr,
                                               (const float4 *)cs.clusters.ptr, sigma, points, n_points,
                                               (uint32_t *)order.ptr, out, st);
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) r = fail_cuda(e, "computing the control-variate potential");
        }
        cs.src.release();
        cs.near2.release();
        cs.clusters.release();
        order.release();
        return r;
    });
}

int wob_scene_set_control_variate(wob_scene s, const float *values, uint32_t n) {
    if (!s || !values) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and values are required");
    if (n != s->host.n) return fail(WOB_ERR_INVALID_ARGUMENT, "need one value per element");
    for (uint32_t i = 0; i < n; i++)
        if (!(values[i] == values[i]) || values[i] > 3.0e38f || values[i] < -3.0e38f)
            return fail(WOB_ERR_INVALID_ARGUMENT, "control-variate values must be finite");
    DeviceGuard g(s->device);
    cudaError_t e = upload(s->cv_table, values, (size_t)n * 4);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "uploading the control variate");
}

int wob_solve_domain_cv(wob_scene s, const wob_params *params, uint32_t n_potential_samples, uint32_t n_kernel_samples,
                        const float *points, uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                        float *per_path, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (w.bie != WOB_INDIRECT_SINGLE_LAYER || w.estimator != WOB_FORWARD_ESTIMATOR || w.problem != WOB_NEUMANN_PROBLEM)
        return fail(WOB_ERR_UNSUPPORTED, "the control-variate estimator is the forward single-layer Neumann estimator");
    if (w.n_volume != 0) return fail(WOB_ERR_UNSUPPORTED, "the control-variate estimator takes no source term");
    if (!s->cv_table.ptr) return fail(WOB_ERR_INVALID_ARGUMENT, "no control variate set (wob_scene_set_control_variate)");
    if (n_points == 0) return WOB_OK;
    if (!points || (!sum && !per_path)) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum (or per_path) are required");
    w.n_pot = n_potential_samples;
    w.m_ker = n_kernel_samples;
    DeviceGuard g(s->device);
    cudaError_t e = s->host.dim == 2
        ? wobgb::launch_domain_cv_2d(s->view<2>(), w, points, n_points, sum, sumsq, (unsigned long long *)bounces, per_path, (cudaStream_t)stream)
        : wobgb::launch_domain_cv_3d(s->view<3>(), w, points, n_points, sum, sumsq, (unsigned long long *)bounces, per_path, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the control-variate walk");
}

static int scene_set_rhs_impl(wob_scene s, const float *values, uint32_t n_rhs) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n_rhs > wobgb::kMaxRhs) return fail(WOB_ERR_INVALID_ARGUMENT, "n_rhs must be at most WOB_MAX_RHS (64)");
    DeviceGuard g(s->device);
    s->rhs_cv.release();
    if (n_rhs == 0) {
        s->rhs.release();
        s->n_rhs = 0;
        return WOB_OK;
    }
    if (!values) return fail(WOB_ERR_INVALID_ARGUMENT, "values are required");
    const uint32_t n = s->host.n, D = (uint32_t)s->host.dim;
    const size_t row = (size_t)D * n_rhs;
    std::vector<float> stored((size_t)n * row);
    for (uint32_t i = 0; i < n; i++) {
        const float *src = values + (size_t)s->host.order[i] * row;
        for (size_t k = 0; k < row; k++) {
            const float v = src[k];
            if (!(v == v) || v > 3.0e38f || v < -3.0e38f) return fail(WOB_ERR_INVALID_ARGUMENT, "RHS values must be finite");
            stored[(size_t)i * row + k] = v;
        }
    }
    cudaError_t e = upload(s->rhs, stored.data(), stored.size() * 4);
    if (e != cudaSuccess) {
        s->n_rhs = 0;
        return fail_cuda(e, "uploading the RHS table");
    }
    s->n_rhs = n_rhs;
    return WOB_OK;
}

int wob_scene_set_rhs(wob_scene s, const float *values, uint32_t n_rhs) {
    return guarded([&] { return scene_set_rhs_impl(s, values, n_rhs); });
}

namespace {
int check_multi(const wob_scene_s *s, const wob_params *params, wobgb::WalkParams &w) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (!wobgb::multi_rhs_supported(w))
        return fail(WOB_ERR_UNSUPPORTED, "multi-RHS walks need sampling that ignores the boundary data: backward "
                                         "IndirectSingleLayer, or backward Direct without NeumannProblem, and no source term");
    if (s->n_rhs == 0) return fail(WOB_ERR_INVALID_ARGUMENT, "no RHS table set (wob_scene_set_rhs)");
    return WOB_OK;
}
}  // namespace

int wob_solve_domain_multi(wob_scene s, const wob_params *params, const float *points, uint32_t n_points, double *sum,
                           double *sumsq, uint64_t *bounces, float *per_path, void *stream) {
    wobgb::WalkParams w;
    int st = check_multi(s, params, w);
    if (st != WOB_OK) return st;
    if (n_points == 0) return WOB_OK;
    if (!points || (!sum && !per_path)) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum (or per_path) are required");
    DeviceGuard g(s->device);
    wobgb::MultiRhsArgs a{};
    a.unknown = false;
    a.points = points;
    a.rhs_table = (const float *)s->rhs.ptr;
    a.n_rhs = s->n_rhs;
    a.n_points = n_points;
    a.sum = sum;
    a.sumsq = sumsq;
    a.bounces = (unsigned long long *)bounces;
    a.per_path = per_path;
    a.stream = (cudaStream_t)stream;
    cudaError_t e = s->host.dim == 2 ? wobgb::launch_multi_rhs_2d(s->view<2>(), w, a) : wobgb::launch_multi_rhs_3d(s->view<3>(), w, a);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the multi-RHS walk");
}

int wob_scene_set_rhs_control_variate(wob_scene s, const float *values, uint32_t n_elems, uint32_t n_rhs) {
    if (!s || !values) return fail(WOB_ERR_INVALID_ARGUMENT, "scene and values are required");
    if (s->n_rhs == 0) return fail(WOB_ERR_INVALID_ARGUMENT, "no RHS table set (wob_scene_set_rhs)");
    if (n_elems != s->host.n || n_rhs != s->n_rhs)
        return fail(WOB_ERR_INVALID_ARGUMENT, "need [n_elems][n_rhs] values matching the scene and its RHS table");
    const size_t cnt = (size_t)n_elems * n_rhs;
    for (size_t i = 0; i < cnt; i++)
        if (!(values[i] == values[i]) || values[i] > 3.0e38f || values[i] < -3.0e38f)
            return fail(WOB_ERR_INVALID_ARGUMENT, "control-variate values must be finite");
    DeviceGuard g(s->device);
    cudaError_t e = upload(s->rhs_cv, values, cnt * 4);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "uploading the multi-RHS control variate");
}

int wob_solve_domain_multi_cv(wob_scene s, const wob_params *params, uint32_t n_potential_samples, const float *points,
                              uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces, float *per_path,
                              void *stream) {
    wobgb::WalkParams w;
    int st = check_multi(s, params, w);
    if (st != WOB_OK) return st;
    if (!s->rhs_cv.ptr) return fail(WOB_ERR_INVALID_ARGUMENT, "no control variate set (wob_scene_set_rhs_control_variate)");
    if (n_potential_samples < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "n_potential_samples must be >= 1");
    if (n_points == 0) return WOB_OK;
    if (!points || (!sum && !per_path)) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum (or per_path) are required");
    DeviceGuard g(s->device);
    wobgb::MultiRhsArgs a{};
    a.unknown = false;
    a.points = points;
    a.rhs_table = (const float *)s->rhs.ptr;
    a.cv_table = (const float *)s->rhs_cv.ptr;
    a.n_rhs = s->n_rhs;
    a.n_potential = n_potential_samples;
    a.n_points = n_points;
    a.sum = sum;
    a.sumsq = sumsq;
    a.bounces = (unsigned long long *)bounces;
    a.per_path = per_path;
    a.stream = (cudaStream_t)stream;
    cudaError_t e = s->host.dim == 2 ? wobgb::launch_multi_rhs_2d(s->view<2>(), w, a) : wobgb::launch_multi_rhs_3d(s->view<3>(), w, a);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the multi-RHS control-variate walk");
}

int wob_solve_unknown_boundary_multi(wob_scene s, const wob_params *params, const float *p, const float *n,
                                     const float *interior_angle, const float *boundary_values,
                                     const int32_t *boundary_type, const float *robin_alpha, uint32_t n_points,
                                     double *sum, double *sumsq, uint64_t *bounces, float *per_path, void *stream) {
    wobgb::WalkParams w;
    int st = check_multi(s, params, w);
    if (st != WOB_OK) return st;
    if (n_points == 0) return WOB_OK;
    if (!p || !n || !interior_angle || !boundary_values || !boundary_type || (!sum && !per_path))
        return fail(WOB_ERR_INVALID_ARGUMENT,
                    "p, n, interior_angle, boundary_values, boundary_type and sum (or per_path) are required");
    DeviceGuard g(s->device);
    wobgb::MultiRhsArgs a{};
    a.unknown = true;
    a.bin = wobgb::BoundaryInput{p, n, interior_angle, nullptr, boundary_type, robin_alpha};
    a.rhs_table = (const float *)s->rhs.ptr;
    a.rhs_input = boundary_values;
    a.n_rhs = s->n_rhs;
    a.n_points = n_points;
    a.sum = sum;
    a.sumsq = sumsq;
    a.bounces = (unsigned long long *)bounces;
    a.per_path = per_path;
    a.stream = (cudaStream_t)stream;
    cudaError_t e = s->host.dim == 2 ? wobgb::launch_multi_rhs_2d(s->view<2>(), w, a) : wobgb::launch_multi_rhs_3d(s->view<3>(), w, a);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the multi-RHS unknown-boundary walk");
}

int wob_solve_wos(wob_scene s, const wob_params *params, const float *points, uint32_t n_points, double *sum,
                  double *sumsq, uint64_t *queries, float *per_path, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (s->host.dim != 2) return fail(WOB_ERR_UNSUPPORTED, "walk on spheres is implemented for 2D scenes");
    if (!s->all_dirichlet) return fail(WOB_ERR_UNSUPPORTED, "walk on spheres needs Dirichlet data on every element");
    if (!params) return fail(WOB_ERR_INVALID_ARGUMENT, "params is NULL");
    if (params->num_sample_paths < 1) return fail(WOB_ERR_INVALID_ARGUMENT, "num_sample_paths must be >= 1");
    if (!(params->eps > 0.0f)) return fail(WOB_ERR_INVALID_ARGUMENT, "eps must be positive");
    if (n_points == 0) return WOB_OK;
    if (!points || (!sum && !per_path)) return fail(WOB_ERR_INVALID_ARGUMENT, "points and sum (or per_path) are required");
    wobgb::WalkParams w{};
    w.n_paths = params->num_sample_paths;
    w.eps = params->eps;
    w.seed = params->seed;
    w.path_offset = params->path_offset;
    w.point_offset = params->point_offset;
    DeviceGuard g(s->device);
    cudaError_t e = wobgb::launch_wos_2d(s->view<2>(), w, points, n_points, sum, sumsq, (unsigned long long *)queries,
                                         per_path, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the walk on spheres");
}

int wob_closest_point(wob_scene s, const float *points, uint32_t n_points, uint32_t *elems, float *dist2,
                      float *values, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (s->host.dim != 2) return fail(WOB_ERR_UNSUPPORTED, "the closest-point query is implemented for 2D scenes");
    if (n_points == 0) return WOB_OK;
    if (!points || !elems || !dist2 || !values) return fail(WOB_ERR_INVALID_ARGUMENT, "all arrays are required");
    DeviceGuard g(s->device);
    cudaError_t e = wobgb::launch_closest_point_2d(s->view<2>(), points, n_points, elems, dist2, values,
                                                   (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the closest-point query");
}

int wob_vpl_paths(wob_scene s, const wob_params *params, uint32_t n_paths, float *vpl_points, float *vpl_values,
                  uint64_t *bounces, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (w.bie != WOB_INDIRECT_SINGLE_LAYER || w.estimator != WOB_BACKWARD_ESTIMATOR || w.n_volume != 0)
        return fail(WOB_ERR_UNSUPPORTED, "VPL walks use the backward single-layer estimator without a source term");
    if (n_paths == 0) return WOB_OK;
    if (!vpl_points || !vpl_values) return fail(WOB_ERR_INVALID_ARGUMENT, "vpl_points and vpl_values are required");
    DeviceGuard g(s->device);
    cudaError_t e = s->host.dim == 2
        ? wobgb::launch_vpl_paths_2d(s->view<2>(), w, n_paths, vpl_points, vpl_values, (unsigned long long *)bounces, (cudaStream_t)stream)
        : wobgb::launch_vpl_paths_3d(s->view<3>(), w, n_paths, vpl_points, vpl_values, (unsigned long long *)bounces, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the VPL walks");
}

int wob_vpl_aggregate(wob_scene s, float eps, const float *vpl_points, const float *vpl_values, uint32_t n_vpl,
                      const float *points, uint32_t n_points, double *sum, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!(eps > 0.0f)) return fail(WOB_ERR_INVALID_ARGUMENT, "eps must be positive");
    if (n_points == 0) return WOB_OK;
    if (!points || !sum || (n_vpl && (!vpl_points || !vpl_values)))
        return fail(WOB_ERR_INVALID_ARGUMENT, "points, sum, vpl_points and vpl_values are required");
    DeviceGuard g(s->device);
    cudaError_t e = wobgb::launch_vpl_aggregate(s->host.dim, vpl_points, vpl_values, n_vpl, s->host.total_area, eps,
                                                points, n_points, sum, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the VPL aggregation");
}

int wob_solve_unknown_boundary(wob_scene s, const wob_params *params, const float *p, const float *n,
                               const float *interior_angle, const float *boundary_value, const int32_t *boundary_type,
                               const float *robin_alpha, uint32_t n_points, double *sum, double *sumsq,
                               uint64_t *bounces, void *stream) {
    if (!s) return fail(WOB_ERR_INVALID_ARGUMENT, "scene is NULL");
    wobgb::WalkParams w;
    int st = check_params(s, params, w);
    if (st != WOB_OK) return st;
    if (w.estimator != WOB_BACKWARD_ESTIMATOR) return fail(WOB_ERR_UNSUPPORTED, "the unknown boundary density comes from the backward estimator");
    if (n_points == 0) return WOB_OK;
    if (!p || !n || !interior_angle || !boundary_value || !boundary_type || !sum)
        return fail(WOB_ERR_INVALID_ARGUMENT, "p, n, interior_angle, boundary_value, boundary_type and sum are required");
    w.mode = 1;
    wobgb::BoundaryInput bin{p, n, interior_angle, boundary_value, boundary_type, robin_alpha};
    DeviceGuard g(s->device);
    cudaError_t e = s->host.dim == 2
        ? wobgb::launch_boundary_2d(s->view<2>(), w, bin, n_points, sum, sumsq, (unsigned long long *)bounces, nullptr, (cudaStream_t)stream)
        : wobgb::launch_boundary_3d(s->view<3>(), w, bin, n_points, sum, sumsq, (unsigned long long *)bounces, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? WOB_OK : fail_cuda(e, "launching the unknown-boundary walk");
}

}  // extern "C"
