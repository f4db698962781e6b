// Shared-memory-tiled contraction used by the cell kernels.
//
// out[c][r] = sum_{jmin <= j < jmax} cvT[j][cell(c)] * B_{vec(r)}[j]
// (jmin a multiple of KC, 0 by default)
// cvT [npad][TC] holds TC cells' right-hand sides (or weights),
// cell-contiguous; B_v[j] comes from a loader functor. 256 threads, in two
// layouts:
//   wide   (W = true):  16 cell groups x 16 vector groups, CPT = TC/16
//                       cells x 4 vectors per thread, 64 vectors per pass;
//   narrow (W = false): TC cell groups x 256/TC vector groups, 1 cell x 1
//                       vector per thread, 256/TC vectors per pass (for the
//                       few dual / step vectors, so no FMAs go to padding).
// B is staged through shared memory in KC-long chunks.
//
// FP64 cvT (the plain FP64 path): FP64 B, FP64 accumulation.
// FP32 cvT (split precision): B arrives as FP32 (hi, lo) pairs made once
// per system from the FP64 factor / duals (b = hi + lo to 48 bits); both
// are multiplied with a and the FP32 partial sums are flushed into FP64
// accumulators every 4 * KC terms (GB300's FP64 pipe is ~1/64 of FP32, so
// the flush rate is kept low), leaving the rounding of cvT and the FP32
// summation of 128-term partials as the FP32-level errors.
#pragma once
#include "spi_common.cuh"

namespace spi {

constexpr int CT = 256;         // threads per cell CTA
constexpr int KC = 32;          // contraction chunk
constexpr int VB = 64;          // vectors per wide pass
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

// Vector base pointers in shared memory (nullptr rows are never read).
struct PtrLoader64 {
  const double* const* vptr;
  __device__ __forceinline__ double operator()(int v, int j) const { return vptr[v][j]; }
};
struct PtrLoader32 {
  const float* const* hptr;
  const float* const* lptr;
  __device__ __forceinline__ float2 operator()(int v, int j) const {
    return make_float2(hptr[v][j], lptr[v][j]);
  }
};

template <int TC, bool W>
struct Layout {
  static constexpr int NCG = W ? 16 : TC;          // cell groups
  static constexpr int CPT = TC / NCG;             // cells per thread
  static constexpr int NVG = CT / NCG;             // vector groups
  static constexpr int VPT = W ? 4 : 1;            // vectors per thread
  static constexpr int NV = NVG * VPT;             // vectors per pass
};

template <typename T, int TC, bool W, typename Loader>
__device__ __forceinline__ void tile_contract(const T* __restrict__ cvT, T* __restrict__ Bs,
                                              const Loader& ld, int nv, int jmax, int n,
                                              double (&out)[Layout<TC, W>::CPT][Layout<TC, W>::VPT],
                                              int jmin = 0) {
  using LY = Layout<TC, W>;
  constexpr int CPT = LY::CPT, VPT = LY::VPT, NV = LY::NV;
  const int tid = threadIdx.x, cg = tid % LY::NCG, rg = tid / LY::NCG;
#pragma unroll
  for (int c = 0; c < CPT; ++c)
#pragma unroll
    for (int r = 0; r < VPT; ++r) out[c][r] = 0.0;
  if constexpr (sizeof(T) == 8) {
    for (int k0 = jmin; k0 < jmax; k0 += KC) {
      __syncthreads();
      for (int e = tid; e < NV * KC; e += CT) {
        int v = e / KC, jj = e % KC;
        int j = k0 + jj;
        Bs[jj * BSTR + v] = (v < nv && j < n) ? ld(v, j) : 0.0;
      }
      __syncthreads();
#pragma unroll 8
      for (int jj = 0; jj < KC; ++jj) {
        double a[CPT], b[VPT];
        const double* ap = cvT + (int64_t)(k0 + jj) * TC + cg * CPT;
#pragma unroll
        for (int c = 0; c < CPT; ++c) a[c] = ap[c];
        if constexpr (VPT == 4) {
          Vec4<double>::load(Bs + jj * BSTR + rg * 4, b);
        } else {
          b[0] = Bs[jj * BSTR + rg];
        }
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < VPT; ++r) out[c][r] += a[c] * b[r];
      }
    }
  } else {
    float* Bh = Bs;
    float* Bl = Bs + KC * BSTR;
    float acc[CPT][VPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c)
#pragma unroll
      for (int r = 0; r < VPT; ++r) acc[c][r] = 0.f;
    int chunk = 0;
    for (int k0 = jmin; k0 < jmax; k0 += KC, ++chunk) {
      __syncthreads();
      for (int e = tid; e < NV * KC; e += CT) {
        int v = e / KC, jj = e % KC;
        int j = k0 + jj;
        float2 x = (v < nv && j < n) ? ld(v, j) : make_float2(0.f, 0.f);
        Bh[jj * BSTR + v] = x.x;
        Bl[jj * BSTR + v] = x.y;
      }
      __syncthreads();
#pragma unroll 8
      for (int jj = 0; jj < KC; ++jj) {
        float a[CPT], bh[VPT], bl[VPT];
        const float* ap = cvT + (int64_t)(k0 + jj) * TC + cg * CPT;
        if constexpr (CPT == 4) {
          Vec4<float>::load(ap, a);
        } else {
#pragma unroll
          for (int c = 0; c < CPT; ++c) a[c] = ap[c];
        }
        if constexpr (VPT == 4) {
          Vec4<float>::load(Bh + jj * BSTR + rg * 4, bh);
          Vec4<float>::load(Bl + jj * BSTR + rg * 4, bl);
        } else {
          bh[0] = Bh[jj * BSTR + rg];
          bl[0] = Bl[jj * BSTR + rg];
        }
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < VPT; ++r) {
            acc[c][r] = fmaf(a[c], bh[r], acc[c][r]);
            acc[c][r] = fmaf(a[c], bl[r], acc[c][r]);
          }
      }
      if ((chunk & 3) == 3) {
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < VPT; ++r) {
            out[c][r] += (double)acc[c][r];
            acc[c][r] = 0.f;
          }
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
#pragma unroll
      for (int r = 0; r < VPT; ++r) out[c][r] += (double)acc[c][r];
  }
}

}  // namespace spi
