// Scene construction on the GPU (scene_build_gpu.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace wobgb {

// Device buffers of a scene built on the GPU (owned by the caller after a successful build) and
// the figures the host keeps.
struct DeviceSceneBuild {
    void *elems = nullptr, *elem_aux = nullptr, *isect = nullptr, *nodes = nullptr, *area_cdf = nullptr,
         *area_guide = nullptr, *bv_cdf = nullptr, *bv_guide = nullptr;
    size_t elems_bytes = 0, elem_aux_bytes = 0, isect_bytes = 0, nodes_bytes = 0, area_cdf_bytes = 0,
           area_guide_bytes = 0, bv_cdf_bytes = 0, bv_guide_bytes = 0;
    uint32_t n_nodes = 0, depth = 0, area_G = 0, bv_G = 0;
    float total_area = 0.0f, total_bv = 0.0f;
    bool bv_valid = false, all_dirichlet = true;
    std::vector<uint32_t> order;  // order[i] = caller index of stored element i
    void release();
};

// Device arrays in caller order, laid out as for wob_scene_create. Returns "" on success, else a
// message (cuda_error holds the CUDA error when one occurred). Synchronises the stream.
std::string build_device_scene(int dim, uint32_t n, const float *verts, const float *normals, const float *bvals,
                               const float *alphas, const int32_t *types, cudaStream_t stream, DeviceSceneBuild &out,
                               cudaError_t &cuda_error);

}  // namespace wobgb
