// Measured CUDA-core peaks for the roofline of the FP64 and FP32 kernels
// (the measured peaks cover HBM and the bf16 tensor pipe only):
// every thread runs 8 independent FMA chains for iters rounds (a multiple
// of 8; the loop is unrolled 8 deep), on a grid of 16 CTAs x 256 threads
// per SM. The caller times the launch with CUDA
// events on the same stream; work = 2 * 8 * iters * threads FLOP. The
// chains' results are stored so that nothing is optimised away.
#include "spi_common.cuh"

namespace spi {

template <typename T>
__global__ __launch_bounds__(256) void k_peak_fma(int64_t iters, T* __restrict__ sink) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  T a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = (T)(1.0 + 1e-7 * (double)((t + c) & 1023));
  const T b = (T)0.9999999, d = (T)1e-7;
  const int rounds = (int)(iters / 8);  // 8 x 8 FMAs per loop iteration
  for (int i = 0; i < rounds; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < 8; ++c) a[c] = fma(a[c], b, d);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += a[c];
  sink[t] = s;
}

}  // namespace spi

extern "C" int spi_peak_fma(int32_t f64, int64_t iters, void* sink, int64_t* threads,
                            spi_stream_t stream) {
  if (iters < 8 || iters % 8 || !sink || !threads) return SPI_ERR_ARG;
  const int blocks = 152 * 16;
  *threads = (int64_t)blocks * 256;
  cudaStream_t st = (cudaStream_t)stream;
  if (f64)
    spi::k_peak_fma<double><<<blocks, 256, 0, st>>>(iters, (double*)sink);
  else
    spi::k_peak_fma<float><<<blocks, 256, 0, st>>>(iters, (float*)sink);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
