// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <string>

#include "stride_common.cuh"

namespace stride {

extern thread_local std::string g_last_error;

// Record a message for stride_last_error_message() and return `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// Device bytes reserved for a stream of `len` bytes (256-aligned, zero pad).
size_t blob_alloc_bytes(size_t len);

// Device Status word -> STRIDE_OK / STRIDE_ERR_*.
int status_to_code(const Status& st, uint32_t* bad_meshlet);
const char* status_message(int code);

}  // namespace stride
