// Host-side helpers shared by the C-ABI entry points.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/smartinterp.h"

namespace si {

// Records a message for si_last_error() and returns code.
int set_error(int code, const char* fmt, ...);

// Clears the error message of this thread.
void clear_error();

// Turns a pending launch error into SI_ERR_CUDA with the given context.
int check_launch(const char* what);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int dtype_size(int dtype) {
  switch (dtype) {
    case SI_U8:
    case SI_I8:
      return 1;
    case SI_U16:
    case SI_I16:
      return 2;
    case SI_I32:
    case SI_F32:
      return 4;
    default:
      return 0;
  }
}

// Number of SMs of the current device (cached per device).
int sm_count();

// 16 -> 16 channel 3x3x3 convolution on the tensor cores (si_umma.cu).
int conv16_umma(const void* x, const void* w, const float* bias, const void* residual, void* y, int N, int D, int H,
                int W, int dil, int relu, int out_f32, cudaStream_t st);

}  // namespace si
