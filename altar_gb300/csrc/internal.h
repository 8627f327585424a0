// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "../../include/altar_gb300.h"

namespace ag {

// records the calling thread's last error message and returns `code`
int set_error(int code, const char* fmt, ...);

// translate a CUDA runtime status: AG_OK or AG_ERR_CUDA with the message recorded
int cuda_status(cudaError_t e, const char* where);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<size_t>(p) % a) == 0; }

// checks a kernel launch and returns the ABI status
inline int launch_status(const char* name) { return cuda_status(cudaGetLastError(), name); }

}  // namespace ag

#define AG_REQUIRE(cond, ...)                                   \
    do {                                                        \
        if (!(cond)) return ::ag::set_error(AG_ERR_ARG, __VA_ARGS__); \
    } while (0)
