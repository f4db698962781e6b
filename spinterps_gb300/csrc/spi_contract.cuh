// Shared-memory-tiled contraction used by the cell kernels.
//
// acc[c][r] = sum_{j < jmax} cvT[j][cg*CPT + c] * B_{rg*4 + r}[j]
// where cvT [npad][TC] holds TC cells' right-hand sides (or weights),
// cell-contiguous, and B_v[j] is produced by a loader functor. 256 threads:
// thread t owns cell group cg = t % 16 (CPT = TC / 16 cells) and vector
// group rg = t / 16 (4 vectors), so a CTA computes a TC x 64 block per
// pass. B is staged through shared memory in KC-long chunks; each inner
// step reads CPT + 4 values (two vector loads) for 4*CPT FMAs.
#pragma once
#include "spi_common.cuh"

namespace spi {

constexpr int CT = 256;         // threads per cell CTA
constexpr int KC = 32;          // contraction chunk
constexpr int VB = 64;          // vectors (columns) per contraction block
constexpr int BSTR = VB + 4;    // Bs row stride (16-byte aligned rows)

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  __device__ static void load(const float* p, float* o) {
    float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <>
struct Vec4<double> {
  __device__ static void load(const double* p, double* o) {
    double2 a = *reinterpret_cast<const double2*>(p);
    double2 b = *reinterpret_cast<const double2*>(p + 2);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
};

// Loads B_v[j] (FP64) from a table of vector base pointers (nullptr: zeros).
struct PtrLoader {
  const double* const* vptr;
  __device__ __forceinline__ double operator()(int v, int j) const { return vptr[v][j]; }
};

// FP64 cvT: plain FP64 contraction.
// FP32 cvT (split precision): each FP64 B value is staged as an FP32 pair
// b = b_hi + b_lo (48 significant bits), both multiplied with a, and the
// FP32 partial sums are flushed into FP64 accumulators every 2 * KC terms,
// so the only FP32-level error left is the rounding of cvT itself.
// Bs must hold 2 * KC * BSTR floats (= KC * BSTR doubles).
template <typename T, int TC, typename Loader>
__device__ __forceinline__ void tile_contract(const T* __restrict__ cvT, T* __restrict__ Bs,
                                              const Loader& ld, int nv, int jmax, int n,
                                              double (&out)[TC / 16][4]) {
  constexpr int CPT = TC / 16;
  const int tid = threadIdx.x, cg = tid % 16, rg = tid / 16;
#pragma unroll
  for (int c = 0; c < CPT; ++c)
#pragma unroll
    for (int r = 0; r < 4; ++r) out[c][r] = 0.0;
  if constexpr (sizeof(T) == 8) {
    for (int k0 = 0; k0 < jmax; k0 += KC) {
      __syncthreads();
      for (int e = tid; e < VB * KC; e += CT) {
        int v = e / KC, jj = e % KC;
        int j = k0 + jj;
        Bs[jj * BSTR + v] = (v < nv && j < n) ? ld(v, j) : 0.0;
      }
      __syncthreads();
#pragma unroll 8
      for (int jj = 0; jj < KC; ++jj) {
        double a[CPT], b[4];
        const double* ap = cvT + (int64_t)(k0 + jj) * TC + cg * CPT;
#pragma unroll
        for (int c = 0; c < CPT; ++c) a[c] = ap[c];
        Vec4<double>::load(Bs + jj * BSTR + rg * 4, b);
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < 4; ++r) out[c][r] += a[c] * b[r];
      }
    }
  } else {
    float* Bh = Bs;
    float* Bl = Bs + KC * BSTR;
    float acc[CPT][4];
#pragma unroll
    for (int c = 0; c < CPT; ++c)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[c][r] = 0.f;
    int chunk = 0;
    for (int k0 = 0; k0 < jmax; k0 += KC, ++chunk) {
      __syncthreads();
      for (int e = tid; e < VB * KC; e += CT) {
        int v = e / KC, jj = e % KC;
        int j = k0 + jj;
        double x = (v < nv && j < n) ? ld(v, j) : 0.0;
        float h = (float)x;
        Bh[jj * BSTR + v] = h;
        Bl[jj * BSTR + v] = (float)(x - (double)h);
      }
      __syncthreads();
#pragma unroll 8
      for (int jj = 0; jj < KC; ++jj) {
        float a[CPT], bh[4], bl[4];
        const float* ap = cvT + (int64_t)(k0 + jj) * TC + cg * CPT;
        if constexpr (CPT == 4) {
          Vec4<float>::load(ap, a);
        } else {
#pragma unroll
          for (int c = 0; c < CPT; ++c) a[c] = ap[c];
        }
        Vec4<float>::load(Bh + jj * BSTR + rg * 4, bh);
        Vec4<float>::load(Bl + jj * BSTR + rg * 4, bl);
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            acc[c][r] = fmaf(a[c], bh[r], acc[c][r]);
            acc[c][r] = fmaf(a[c], bl[r], acc[c][r]);
          }
      }
      if (chunk & 1) {
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            out[c][r] += (double)acc[c][r];
            acc[c][r] = 0.f;
          }
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
#pragma unroll
      for (int r = 0; r < 4; ++r) out[c][r] += (double)acc[c][r];
  }
}

}  // namespace spi
