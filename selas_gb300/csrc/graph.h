// CUDA-graph replay of a launch sequence that is identical from one progressive pass (or path batch) to the
// next: the sequence is captured once per argument set, instantiated, and launched once per pass.
#pragma once

#include <cstring>
#include <vector>

#include <cuda_runtime.h>

namespace sel {

struct GraphCache {
    std::vector<unsigned char> key;  // the bytes the captured launches were built from
    cudaGraphExec_t exec = nullptr;
    uint64_t captures = 0;           // how many times a sequence was captured (for tests)

    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
    GraphCache() = default;
    GraphCache(const GraphCache&) = delete;
    GraphCache& operator=(const GraphCache&) = delete;
    ~GraphCache() { reset(); }
};

// Launches `enqueue(stream)` `count` times.  With a cache, the sequence is captured into a graph on first
// use (or when `key` changes) and the graph is launched instead.  Streams that cannot be captured (the
// legacy default stream, or a stream the caller is already capturing) get the launches directly.
template <typename Enqueue>
cudaError_t replay(GraphCache* cache, const void* key, size_t key_bytes, cudaStream_t stream, uint64_t count,
                   Enqueue enqueue) {
    if (count == 0) return cudaSuccess;
    cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
    if (cache && stream) {
        if (cudaStreamIsCapturing(stream, &status) != cudaSuccess) status = cudaStreamCaptureStatusActive;
    }
    if (!cache || !stream || status != cudaStreamCaptureStatusNone) {
        for (uint64_t i = 0; i < count; ++i) enqueue(stream);
        return cudaGetLastError();
    }
    const unsigned char* k = static_cast<const unsigned char*>(key);
    if (!cache->exec || cache->key.size() != key_bytes || std::memcmp(cache->key.data(), k, key_bytes) != 0) {
        cache->reset();
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        enqueue(stream);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&cache->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            cache->exec = nullptr;
            return e;
        }
        cache->key.assign(k, k + key_bytes);
        ++cache->captures;
    }
    for (uint64_t i = 0; i < count; ++i) {
        cudaError_t e = cudaGraphLaunch(cache->exec, stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sel
