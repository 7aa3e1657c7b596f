// Handle types behind the opaque C ABI pointers and the shared error helpers.
#pragma once

#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sel_internal.h"

struct SelDeviceTy {
    int cuda_device = 0;
    cudaStream_t stream = nullptr;  // internal stream for the host-memory entry points
    uint32_t* d_err = nullptr;      // kernel error word (iteration cap / stack overflow bits)
    std::mutex mu;
};

struct SelSceneTy {
    SelDeviceTy* dev = nullptr;
    int kind = SEL_BVH_WIDE8_Q8;
    std::vector<sel::MeshInput> meshes;
    bool committed = false;
    void* d_nodes = nullptr;
    void* d_tris = nullptr;
    SelSceneInfo info{};
    void* scratch = nullptr;  // staging buffer of the host-memory query forms
    size_t scratch_bytes = 0;
    std::mutex mu;
};

namespace sel {
struct DeviceBvh;
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
int set_device(SelDeviceTy* dev);
int read_error_word(SelDeviceTy* dev, cudaStream_t s);
DeviceBvh device_bvh(const SelSceneTy* sc);
}  // namespace sel
