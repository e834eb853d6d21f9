// Runtime utilities of include/halcuda.h: pinned host memory, asynchronous copies, events with
// bounded waits, and device-memory queries.
#include <chrono>
#include <thread>

#include "common.cuh"

struct hc_event_s {
    cudaEvent_t ev;
};

struct hc_graph_s {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    uint64_t launches;  // kernels recorded during capture, credited on every replay
};

namespace hc {
uint64_t launch_counter(hc_context ctx);
}

using namespace hc;

extern "C" {

hc_status hc_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(HC_ERR_ARG, "null output");
    count_alloc();
    return cuda_check(cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault), "pinned host allocation");
}

hc_status hc_host_free(void* ptr) {
    if (!ptr) return HC_OK;
    return cuda_check(cudaFreeHost(ptr), "pinned host free");
}

hc_status hc_memcpy_async(hc_context ctx, void* dst, const void* src, size_t bytes, hc_copy_kind kind) {
    if (!ctx || (bytes && (!dst || !src))) return fail(HC_ERR_ARG, "null argument");
    cudaMemcpyKind k = kind == HC_H2D ? cudaMemcpyHostToDevice
                       : kind == HC_D2H ? cudaMemcpyDeviceToHost
                                        : cudaMemcpyDeviceToDevice;
    return cuda_check(cudaMemcpyAsync(dst, src, bytes, k, stream_of(ctx)), "async copy");
}

hc_status hc_memset_async(hc_context ctx, void* dst, int value, size_t bytes) {
    if (!ctx || (bytes && !dst)) return fail(HC_ERR_ARG, "null argument");
    return cuda_check(cudaMemsetAsync(dst, value, bytes, stream_of(ctx)), "async memset");
}

hc_status hc_event_create(hc_event* out) {
    if (!out) return fail(HC_ERR_ARG, "null output");
    auto* e = new hc_event_s();
    hc_status st = cuda_check(cudaEventCreate(&e->ev), "event creation");
    if (st) {
        delete e;
        return st;
    }
    *out = e;
    return HC_OK;
}

hc_status hc_event_destroy(hc_event ev) {
    if (!ev) return HC_OK;
    cudaEventDestroy(ev->ev);
    delete ev;
    return HC_OK;
}

hc_status hc_event_record(hc_context ctx, hc_event ev) {
    if (!ctx || !ev) return fail(HC_ERR_ARG, "null argument");
    return cuda_check(cudaEventRecord(ev->ev, stream_of(ctx)), "event record");
}

hc_status hc_stream_wait_event(hc_context ctx, hc_event ev) {
    if (!ctx || !ev) return fail(HC_ERR_ARG, "null argument");
    return cuda_check(cudaStreamWaitEvent(stream_of(ctx), ev->ev, 0), "stream wait");
}

hc_status hc_stream_create(void** out) {
    if (!out) return fail(HC_ERR_ARG, "null argument");
    cudaStream_t s = nullptr;
    hc_status st = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream creation");
    *out = st ? nullptr : (void*)s;
    return st;
}

hc_status hc_stream_destroy(void* stream) {
    if (!stream) return HC_OK;
    cudaStreamSynchronize((cudaStream_t)stream);
    return cuda_check(cudaStreamDestroy((cudaStream_t)stream), "stream destroy");
}

hc_status hc_event_query(hc_event ev, int* done) {
    if (!ev || !done) return fail(HC_ERR_ARG, "null argument");
    cudaError_t e = cudaEventQuery(ev->ev);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return HC_OK;
    }
    *done = 1;
    return cuda_check(e, "event query");
}

hc_status hc_event_elapsed_ms(hc_event start, hc_event end, double timeout_ms, float* ms) {
    if (!start || !end || !ms) return fail(HC_ERR_ARG, "null argument");
    auto t0 = std::chrono::steady_clock::now();
    // poll with a deadline instead of blocking forever
    while (true) {
        cudaError_t q = cudaEventQuery(end->ev);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) return cuda_check(q, "event query");
        double waited = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms > 0 && waited > timeout_ms) return fail(HC_ERR_TIMEOUT, "event wait timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return cuda_check(cudaEventElapsedTime(ms, start->ev, end->ev), "event elapsed time");
}

namespace {
thread_local uint64_t g_capture_start = 0;
}

hc_status hc_graph_begin_capture(hc_context ctx) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    g_capture_start = launch_counter(ctx);
    return cuda_check(cudaStreamBeginCapture(stream_of(ctx), cudaStreamCaptureModeRelaxed), "begin capture");
}

hc_status hc_graph_end_capture(hc_context ctx, hc_graph* out) {
    if (!ctx || !out) return fail(HC_ERR_ARG, "null argument");
    cudaGraph_t g = nullptr;
    hc_status st = cuda_check(cudaStreamEndCapture(stream_of(ctx), &g), "end capture");
    if (st) return st;
    auto* h = new hc_graph_s();
    h->graph = g;
    h->launches = launch_counter(ctx) - g_capture_start;
    count_launch(ctx, 0);
    st = cuda_check(cudaGraphInstantiate(&h->exec, g, 0), "graph instantiation");
    if (st) {
        cudaGraphDestroy(g);
        delete h;
        return st;
    }
    *out = h;
    return HC_OK;
}

hc_status hc_graph_launch(hc_context ctx, hc_graph graph) {
    if (!ctx || !graph) return fail(HC_ERR_ARG, "null argument");
    count_launch(ctx, graph->launches);
    return cuda_check(cudaGraphLaunch(graph->exec, stream_of(ctx)), "graph launch");
}

hc_status hc_graph_destroy(hc_graph graph) {
    if (!graph) return HC_OK;
    cudaGraphExecDestroy(graph->exec);
    cudaGraphDestroy(graph->graph);
    delete graph;
    return HC_OK;
}

hc_status hc_device_memory(hc_context ctx, size_t* free_bytes, size_t* total_bytes) {
    if (!ctx || !free_bytes || !total_bytes) return fail(HC_ERR_ARG, "null argument");
    return cuda_check(cudaMemGetInfo(free_bytes, total_bytes), "memory query");
}

hc_status hc_memory_stats(hc_context ctx, int reset_high, uint64_t out[3]) {
    if (!ctx || !out) return fail(HC_ERR_ARG, "null argument");
    cudaMemPool_t pool;
    hc_status st = cuda_check(cudaDeviceGetDefaultMemPool(&pool, device_of(ctx)), "default memory pool");
    if (st) return st;
    unsigned long long used = 0, high = 0;  // the pool attributes are 64-bit unsigned
    if (reset_high) {
        unsigned long long zero = 0;  // resets the high-water mark to the bytes in use now
        if ((st = cuda_check(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero), "pool high-water reset")))
            return st;
    }
    if ((st = cuda_check(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used), "pool use")))
        return st;
    if ((st = cuda_check(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high), "pool high-water")))
        return st;
    out[0] = alloc_calls();
    out[1] = used;
    out[2] = high;
    return HC_OK;
}

}  // extern "C"
