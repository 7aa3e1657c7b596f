// Closest-hit queries for callers that must not allocate GPU memory.
//
// sel_intersect1M stages the caller's records in a device buffer that it allocates (and grows) with
// cudaMalloc.  Some callers cannot allow that: a host application that owns the GPU's memory and hands out
// all of it through its own pool (a renderer plugin, a game engine), a real-time loop that must not risk
// the implicit device synchronisation cudaMalloc/cudaFree may cause, or code that has budgeted every
// byte of HBM up front.  sel_intersect1M_noalloc is the same query with the staging area in a fixed
// file-scope __device__ array instead, so the call itself allocates nothing.
#include "capi_internal.h"
#include "query.h"

using namespace sel;

namespace {

constexpr unsigned int kStaticRecords = 65536;  // 6 MiB of SelRayHit records

// Every GPU that loads the library holds this array until the process exits.  Host code only ever sees
// a host-side stand-in under this name; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) SelRayHit g_static_rayhits[kStaticRecords];

}  // namespace

namespace sel {

// Called by sel_device_new with the device current.  With lazy module loading this is where the module
// holding the array is loaded and the array created, so the query itself neither loads nor allocates.
// The address belongs to the SelDevice (and to its context): a device handle made after a context reset
// resolves it again.
int resolve_noalloc_staging(SelDeviceTy* dev) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_rayhits);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static staging array)");
    dev->noalloc_staging = p;
    return SEL_OK;
}

}  // namespace sel

extern "C" int sel_intersect1M_noalloc(SelScene scene, SelRayHit* rayhits, unsigned int M, size_t byte_stride) {
    if (!scene) return fail(SEL_ERR_INVALID_ARGUMENT, "scene is null");
    if (!scene->committed) return fail(SEL_ERR_INVALID_OPERATION, "scene not committed");
    // A scene whose instanced scenes were re-committed points at their freed trees: refuse it, as every
    // other query does, before anything is launched.
    if (!instances_fresh(scene))
        return fail(SEL_ERR_INVALID_OPERATION, "an instanced scene changed since this scene was committed");
    if (M == 0) return SEL_OK;
    if (!rayhits) return fail(SEL_ERR_INVALID_ARGUMENT, "ray buffer is null");
    if (byte_stride < sizeof(SelRayHit)) return fail(SEL_ERR_INVALID_ARGUMENT, "byte_stride smaller than the record");
    if (M > kStaticRecords)
        return fail(SEL_ERR_INVALID_ARGUMENT,
                    "sel_intersect1M_noalloc takes at most 65536 records per call; split the batch or use sel_intersect1M");
    std::lock_guard<std::mutex> lock(scene->mu);
    if (int rc = set_device(scene->dev)) return rc;
    SelDeviceTy* dev = scene->dev;
    std::lock_guard<std::mutex> dlock(dev->mu);
    SelRayHit* staging = static_cast<SelRayHit*>(dev->noalloc_staging);
    if (!staging) return fail(SEL_ERR_INVALID_OPERATION, "device has no staging array address");
    const cudaStream_t s = dev->stream;
    // Records are copied in whole, so nothing in the array has to start at zero; strided records are
    // gathered by a pitched copy rather than through a host-side buffer.
    cudaError_t e = cudaMemcpy2DAsync(staging, sizeof(SelRayHit), rayhits, byte_stride, sizeof(SelRayHit), M,
                                      cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync(rays to device)");
    e = launch_intersect(device_bvh(scene), staging, M, dev->d_err, s);
    if (e != cudaSuccess) return cuda_fail(e, "query launch");
    e = cudaMemcpy2DAsync(rayhits, byte_stride, staging, sizeof(SelRayHit), sizeof(SelRayHit), M,
                          cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync(rays to host)");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "query");
    return read_error_word(dev, s);
}
