// Host-side helpers shared by the translation units of libgbgpu_gb300.
#pragma once

#include <cuda_runtime.h>

int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);
int num_sms();
int ensure_init(cudaStream_t st);
int gbx_twiddle_init(cudaStream_t st);
