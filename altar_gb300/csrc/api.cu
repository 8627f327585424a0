// C ABI plumbing: per-thread error strings, version, CUDA graph capture.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "internal.h"

namespace ag {

static thread_local char g_err[512] = {0};

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_status(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return AG_OK;
    return set_error(AG_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
}

}  // namespace ag

using namespace ag;

extern "C" int ag_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return AG_ERR_ARG;
    strncpy(buf, g_err, len - 1);
    buf[len - 1] = '\0';
    return AG_OK;
}

extern "C" const char* ag_version(void) { return "altar_gb300 0.1 sm_103a"; }

extern "C" int ag_graph_begin(void* stream) {
    AG_REQUIRE(stream != nullptr, "graph capture needs a non-default stream");
    return cuda_status(cudaStreamBeginCapture(as_stream(stream), cudaStreamCaptureModeThreadLocal),
                       "cudaStreamBeginCapture");
}

extern "C" int ag_graph_end(void* stream, void** graph_exec) {
    AG_REQUIRE(stream != nullptr && graph_exec != nullptr, "invalid arguments");
    cudaGraph_t g = nullptr;
    int rc = cuda_status(cudaStreamEndCapture(as_stream(stream), &g), "cudaStreamEndCapture");
    if (rc) return rc;
    cudaGraphExec_t ex = nullptr;
    rc = cuda_status(cudaGraphInstantiate(&ex, g, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(g);
    if (rc) return rc;
    *graph_exec = reinterpret_cast<void*>(ex);
    return AG_OK;
}

extern "C" int ag_graph_launch(void* graph_exec, void* stream) {
    AG_REQUIRE(graph_exec != nullptr, "graph_exec is NULL");
    return cuda_status(cudaGraphLaunch(reinterpret_cast<cudaGraphExec_t>(graph_exec), as_stream(stream)),
                       "cudaGraphLaunch");
}

extern "C" int ag_graph_destroy(void* graph_exec) {
    if (!graph_exec) return AG_OK;
    return cuda_status(cudaGraphExecDestroy(reinterpret_cast<cudaGraphExec_t>(graph_exec)),
                       "cudaGraphExecDestroy");
}
