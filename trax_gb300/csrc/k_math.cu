// k_math.cu -- the shared single-precision math (trax_math.h) evaluated on
// the device, for the tests that hold it to the CPU build bit for bit and
// to CUDA's own functions within a few ulp.
#include <cuda_runtime.h>

#include "trax/trax.h"
#include "trax_math.h"

namespace {

__global__ void math_eval_kernel(int fn, const float* __restrict__ a, const float* __restrict__ b, float* out,
                                 uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float x = a[i], y = b[i];
    float r = 0.0f;
    switch (fn) {
      case 0: r = trax::atan2_(x, y); break;
      case 1: r = trax::acos_(x); break;
      case 2: r = trax::atan_(x); break;
      case 3: r = trax::asinh_(x); break;
      case 4: r = trax::log_(x); break;
      case 5: r = trax::div_(x, y); break;
      case 6: r = trax::sqrt_(x); break;
      case 7: r = trax::floor_(x); break;
      case 8: r = __uint_as_float(trax::f2u_sat(x)); break;
      case 9: r = __int_as_float(trax::f2i_sat(x)); break;
      // CUDA's own functions, the accuracy reference
      case 10: r = atan2f(x, y); break;
      case 11: r = acosf(x); break;
      case 12: r = atanf(x); break;
      case 13: r = asinhf(x); break;
      case 14: r = logf(x); break;
      default: break;
    }
    out[i] = r;
  }
}

}  // namespace

extern "C" int trax_math_eval(int device, int fn, const float* a, const float* b, float* out, uint64_t n) {
  if (fn < 0 || fn > 14 || !a || !out || (n && !b && (fn == 0 || fn == 5 || fn == 10))) return TRAX_ERR_ARG;
  if (n == 0) return TRAX_OK;
  if (cudaSetDevice(device) != cudaSuccess) return TRAX_ERR_CUDA;
  float *da = nullptr, *db = nullptr, *dout = nullptr;
  const size_t bytes = n * sizeof(float);
  int rc = TRAX_OK;
  if (cudaMalloc(&da, bytes) != cudaSuccess || cudaMalloc(&db, bytes) != cudaSuccess ||
      cudaMalloc(&dout, bytes) != cudaSuccess) {
    rc = TRAX_ERR_CUDA;
  } else if (cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(db, b ? b : a, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = TRAX_ERR_CUDA;
  } else {
    const uint64_t blocks = (n + 255) / 256;
    math_eval_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256>>>(fn, da, db, dout, n);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = TRAX_ERR_CUDA;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dout);
  return rc;
}
