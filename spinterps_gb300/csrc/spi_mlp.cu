// The learned variogram warm start: a small MLP trained and run on the GPU.
//
// No counterpart in the reference (its fitter starts every differential
// evolution from the whole parameter box, variograms/vgs.py:758-764). The
// network maps 20 features of a step's values -- an empirical variogram in
// 20 equal-width lag bins up to half the box diagonal, divided by the
// variance -- to the logits of the model permutation the fitter would pick
// and 3 normalised parameters (log range, structured sill / variance,
// nugget / variance); the fitter then starts its DE from a narrow box around
// that proposal.
//
// Layout: in -> h1 (tanh) -> h2 (tanh) -> out, FP32, parameters packed as
// W1[in][h1], b1[h1], W2[h1][h2], b2[h2], W3[h2][out], b3[out]. Loss of a
// batch of B samples: mean over samples of softmax cross-entropy on the
// first n_class outputs plus wp * 0.5 * sum_k m_k (o_{n_class+k} - y_k)^2
// over the remaining outputs (m: which parameters the sample's class has).
// Small sizes: one thread per output element, no tensor cores needed.
#include "spi_common.cuh"

namespace spi {

struct MlpDims {
  int in, h1, h2, out, n_class;
  int64_t oW1, ob1, oW2, ob2, oW3, ob3, n_par;
};

__host__ __device__ inline MlpDims mlp_dims(int in, int h1, int h2, int out, int n_class) {
  MlpDims d{in, h1, h2, out, n_class, 0, 0, 0, 0, 0, 0, 0};
  d.oW1 = 0;
  d.ob1 = d.oW1 + (int64_t)in * h1;
  d.oW2 = d.ob1 + h1;
  d.ob2 = d.oW2 + (int64_t)h1 * h2;
  d.oW3 = d.ob2 + h2;
  d.ob3 = d.oW3 + (int64_t)h2 * out;
  d.n_par = d.ob3 + out;
  return d;
}

// Y[b][o] = act(b_o + sum_i X[b][i] W[i][o])
__global__ void k_lin_fwd(const float* __restrict__ X, const float* __restrict__ W,
                          const float* __restrict__ bias, float* __restrict__ Y, int B, int nin,
                          int nout, int act_tanh) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)B * nout;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / nout), o = (int)(e % nout);
    float acc = bias[o];
    for (int i = 0; i < nin; ++i) acc = fmaf(X[(int64_t)b * nin + i], W[(int64_t)i * nout + o], acc);
    Y[e] = act_tanh ? tanhf(acc) : acc;
  }
}

// dX[b][i] = (sum_o dY[b][o] W[i][o]) * (tanh' of X when act)
__global__ void k_lin_bwd_x(const float* __restrict__ dY, const float* __restrict__ W,
                            const float* __restrict__ Xact, float* __restrict__ dX, int B,
                            int nin, int nout, int act_tanh) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)B * nin;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / nin), i = (int)(e % nin);
    float acc = 0.f;
    for (int o = 0; o < nout; ++o) acc = fmaf(dY[(int64_t)b * nout + o], W[(int64_t)i * nout + o], acc);
    if (act_tanh) {
      const float h = Xact[e];
      acc *= (1.f - h * h);
    }
    dX[e] = acc;
  }
}

// dW[i][o] = sum_b X[b][i] dY[b][o]; db[o] = sum_b dY[b][o]
__global__ void k_lin_bwd_w(const float* __restrict__ X, const float* __restrict__ dY,
                            float* __restrict__ dW, float* __restrict__ db, int B, int nin,
                            int nout) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)(nin + 1) * nout;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / nout), o = (int)(e % nout);
    float acc = 0.f;
    if (i < nin) {
      for (int b = 0; b < B; ++b) acc = fmaf(X[(int64_t)b * nin + i], dY[(int64_t)b * nout + o], acc);
      dW[(int64_t)i * nout + o] = acc;
    } else {
      for (int b = 0; b < B; ++b) acc += dY[(int64_t)b * nout + o];
      db[o] = acc;
    }
  }
}

// per-sample loss and dL/dO (the 1/B of the batch mean included)
__global__ void k_mlp_loss(const float* __restrict__ O, const int32_t* __restrict__ cls,
                           const float* __restrict__ yp, const float* __restrict__ mk,
                           float* __restrict__ dO, float* __restrict__ loss, int B, int out,
                           int n_class, float wp) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* o = O + (int64_t)b * out;
  float* d = dO + (int64_t)b * out;
  float mx = o[0];
  for (int c = 1; c < n_class; ++c) mx = fmaxf(mx, o[c]);
  float se = 0.f;
  for (int c = 0; c < n_class; ++c) se += expf(o[c] - mx);
  const int y = cls[b];
  float l = logf(se) + mx - o[y];
  for (int c = 0; c < n_class; ++c) d[c] = (expf(o[c] - mx) / se - (c == y ? 1.f : 0.f)) / B;
  const int np_ = out - n_class;
  for (int k = 0; k < np_; ++k) {
    const float r = o[n_class + k] - yp[(int64_t)b * np_ + k];
    const float m = mk[(int64_t)b * np_ + k];
    l += wp * 0.5f * m * r * r;
    d[n_class + k] = wp * m * r / B;
  }
  loss[b] = l / B;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

static unsigned grid_of(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (unsigned)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

}  // namespace spi

using namespace spi;

static int mlp_check(int in, int h1, int h2, int out, int n_class) {
  if (in < 1 || h1 < 1 || h2 < 1 || out < 1 || n_class < 1 || n_class > out) return SPI_ERR_ARG;
  return SPI_OK;
}

// forward pass into ws (H1 [B][h1], H2 [B][h2], O [B][out]) -- returns O
static void mlp_forward(const MlpDims& d, const float* par, const float* X, int B, float* ws,
                        cudaStream_t st) {
  float* H1 = ws;
  float* H2 = H1 + (int64_t)B * d.h1;
  float* O = H2 + (int64_t)B * d.h2;
  k_lin_fwd<<<grid_of((int64_t)B * d.h1), 256, 0, st>>>(X, par + d.oW1, par + d.ob1, H1, B, d.in,
                                                        d.h1, 1);
  k_lin_fwd<<<grid_of((int64_t)B * d.h2), 256, 0, st>>>(H1, par + d.oW2, par + d.ob2, H2, B, d.h1,
                                                        d.h2, 1);
  k_lin_fwd<<<grid_of((int64_t)B * d.out), 256, 0, st>>>(H2, par + d.oW3, par + d.ob3, O, B,
                                                         d.h2, d.out, 0);
}

extern "C" int spi_mlp_forward(int32_t in, int32_t h1, int32_t h2, int32_t out, int32_t n_class,
                               const float* params, const float* X, int32_t B, float* ws,
                               float* O, spi_stream_t stream) {
  int rc = mlp_check(in, h1, h2, out, n_class);
  if (rc) return rc;
  if (B < 0) return SPI_ERR_ARG;
  if (B == 0) return SPI_OK;
  if (!params || !X || !ws || !O) return SPI_ERR_ARG;
  MlpDims d = mlp_dims(in, h1, h2, out, n_class);
  cudaStream_t st = (cudaStream_t)stream;
  mlp_forward(d, params, X, B, ws, st);
  SPI_LAUNCH_CHECK();
  cudaMemcpyAsync(O, ws + (int64_t)B * (d.h1 + d.h2), sizeof(float) * (size_t)B * d.out,
                  cudaMemcpyDeviceToDevice, st);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

// loss (per sample, summing to the batch mean) and gradients of one batch
extern "C" int spi_mlp_grad(int32_t in, int32_t h1, int32_t h2, int32_t out, int32_t n_class,
                            const float* params, const float* X, const int32_t* cls,
                            const float* yp, const float* mask, float wp, int32_t B, float* ws,
                            float* grad, float* loss, spi_stream_t stream) {
  int rc = mlp_check(in, h1, h2, out, n_class);
  if (rc) return rc;
  if (B < 1) return SPI_ERR_ARG;
  if (!params || !X || !cls || !yp || !mask || !ws || !grad || !loss) return SPI_ERR_ARG;
  MlpDims d = mlp_dims(in, h1, h2, out, n_class);
  cudaStream_t st = (cudaStream_t)stream;
  mlp_forward(d, params, X, B, ws, st);
  float* H1 = ws;
  float* H2 = H1 + (int64_t)B * d.h1;
  float* O = H2 + (int64_t)B * d.h2;
  float* dO = O + (int64_t)B * d.out;
  float* dH2 = dO + (int64_t)B * d.out;
  float* dH1 = dH2 + (int64_t)B * d.h2;
  k_mlp_loss<<<(B + 127) / 128, 128, 0, st>>>(O, cls, yp, mask, dO, loss, B, d.out, d.n_class, wp);
  k_lin_bwd_w<<<grid_of((int64_t)(d.h2 + 1) * d.out), 256, 0, st>>>(H2, dO, grad + d.oW3,
                                                                     grad + d.ob3, B, d.h2, d.out);
  k_lin_bwd_x<<<grid_of((int64_t)B * d.h2), 256, 0, st>>>(dO, params + d.oW3, H2, dH2, B, d.h2,
                                                          d.out, 1);
  k_lin_bwd_w<<<grid_of((int64_t)(d.h1 + 1) * d.h2), 256, 0, st>>>(H1, dH2, grad + d.oW2,
                                                                    grad + d.ob2, B, d.h1, d.h2);
  k_lin_bwd_x<<<grid_of((int64_t)B * d.h1), 256, 0, st>>>(dH2, params + d.oW2, H1, dH1, B, d.h1,
                                                          d.h2, 1);
  k_lin_bwd_w<<<grid_of((int64_t)(d.in + 1) * d.h1), 256, 0, st>>>(X, dH1, grad + d.oW1,
                                                                    grad + d.ob1, B, d.in, d.h1);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_mlp_adam(float* params, const float* grad, float* m, float* v,
                            int64_t n_par, float lr, float beta1, float beta2, float eps,
                            int32_t t, spi_stream_t stream) {
  if (n_par < 0 || t < 1) return SPI_ERR_ARG;
  if (n_par == 0) return SPI_OK;
  if (!params || !grad || !m || !v) return SPI_ERR_ARG;
  const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
  k_adam<<<grid_of(n_par), 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n_par, lr, beta1,
                                                           beta2, eps, c1, c2);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int64_t spi_mlp_n_params(int32_t in, int32_t h1, int32_t h2, int32_t out) {
  return mlp_dims(in, h1, h2, out, 1).n_par;
}

namespace spi {
// Features of a step's values for the warm start: the classical semivariance
// sum (z_i - z_j)^2 / (2 N_b) in nb equal-width lag bins up to half the
// diagonal of the step's bounding box, divided by the values' variance
// (0 for empty bins). One CTA per step; bins accumulated in shared memory.
__global__ void k_vg_features(const int64_t* __restrict__ pt_off, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              int nb, float* __restrict__ feat) {
  const int s = blockIdx.x;
  const int64_t p0 = pt_off[s];
  const int n = (int)(pt_off[s + 1] - p0);
  __shared__ double sum[64];
  __shared__ double cnt[64];
  __shared__ double red[4][256];
  const int tid = threadIdx.x;
  for (int b = tid; b < nb; b += blockDim.x) {
    sum[b] = 0.0;
    cnt[b] = 0.0;
  }
  double mx = 0.0, mnx = 1e300, mxx = -1e300, mny = 1e300, mxy = -1e300, sq = 0.0;
  for (int i = tid; i < n; i += blockDim.x) {
    mx += z[p0 + i];
    mnx = fmin(mnx, x[p0 + i]);
    mxx = fmax(mxx, x[p0 + i]);
    mny = fmin(mny, y[p0 + i]);
    mxy = fmax(mxy, y[p0 + i]);
  }
  red[0][tid] = mx;
  red[1][tid] = mnx;
  red[2][tid] = mxx;
  red[3][tid] = mny;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (tid < o) {
      red[0][tid] += red[0][tid + o];
      red[1][tid] = fmin(red[1][tid], red[1][tid + o]);
      red[2][tid] = fmax(red[2][tid], red[2][tid + o]);
      red[3][tid] = fmin(red[3][tid], red[3][tid + o]);
    }
    __syncthreads();
  }
  const double mean = red[0][0] / n;
  const double x0 = red[1][0], x1 = red[2][0], y0 = red[3][0];
  __syncthreads();
  red[0][tid] = mxy;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (tid < o) red[0][tid] = fmax(red[0][tid], red[0][tid + o]);
    __syncthreads();
  }
  const double y1 = red[0][0];
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    double d = z[p0 + i] - mean;
    sq += d * d;
  }
  red[0][tid] = sq;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (tid < o) red[0][tid] += red[0][tid + o];
    __syncthreads();
  }
  const double var = red[0][0] / n;
  const double hmax = 0.5 * sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
  const int64_t P = (int64_t)n * (n - 1) / 2;
  for (int64_t p = tid; p < P; p += blockDim.x) {
    int64_t ii = (int64_t)((1.0 + sqrt(1.0 + 8.0 * (double)p)) * 0.5);
    while (ii * (ii - 1) / 2 > p) --ii;
    while ((ii + 1) * ii / 2 <= p) ++ii;
    const int i = (int)ii, j = (int)(p - ii * (ii - 1) / 2);
    const double dx = x[p0 + i] - x[p0 + j], dy = y[p0 + i] - y[p0 + j];
    const double h = sqrt(dx * dx + dy * dy);
    if (!(h < hmax)) continue;
    int b = (int)(h / hmax * nb);
    if (b >= nb) b = nb - 1;
    const double dz = z[p0 + i] - z[p0 + j];
    atomicAdd(&sum[b], dz * dz);
    atomicAdd(&cnt[b], 1.0);
  }
  __syncthreads();
  for (int b = tid; b < nb; b += blockDim.x)
    feat[(int64_t)s * nb + b] =
        (cnt[b] > 0 && var > 0) ? (float)(sum[b] / (2.0 * cnt[b]) / var) : 0.f;
}
}  // namespace spi

extern "C" int spi_vg_features(int32_t n_steps, const int64_t* pt_off, const double* x,
                               const double* y, const double* z, int32_t n_bins, float* feat,
                               spi_stream_t stream) {
  if (n_steps < 0 || n_bins < 1 || n_bins > 64) return SPI_ERR_ARG;
  if (n_steps == 0) return SPI_OK;
  if (!pt_off || !x || !y || !z || !feat) return SPI_ERR_ARG;
  spi::k_vg_features<<<n_steps, 256, 0, (cudaStream_t)stream>>>(pt_off, x, y, z, n_bins, feat);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
