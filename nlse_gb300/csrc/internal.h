// Library-internal helpers defined in capi.cu and used by the other
// translation units (error reporting through nlse_last_error, shared twiddle
// tables).
#pragma once
#include <cuda_runtime.h>

namespace nlse {
int shared_twiddles(int dev, int dtype, const void** out);
int shared_fail(int code, const char* msg);
int shared_cuda_fail(cudaError_t e, const char* what);
void shared_clear_error();
}  // namespace nlse
