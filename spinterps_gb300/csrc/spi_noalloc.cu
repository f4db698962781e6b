// spi_krige_ok_noalloc: ordinary kriging of one station set without any
// device allocation.
//
// Some callers cannot allocate device memory: host applications that own
// every byte of the GPU through their own pool allocator and forbid raw
// cudaMalloc, and latency-bound services for which a cudaMalloc per call
// (which can synchronise the device and stall their other streams) costs
// more than the interpolation itself. The regular kriging entry points
// take a caller-provided workspace; this one instead keeps its workspace
// (factor arenas, dual weights, system descriptors) in one file-scope
// static device array, so the caller passes only inputs and outputs.
// The system's route (route_out, optional) tells the caller whether the
// step is one the reference would report as a problem step: route 2 means
// the system was exactly singular and every cell took its nearest station.
//
// The array holds one system of at most SPI_NOALLOC_MAX_STNS stations and
// SPI_NOALLOC_MAX_STEPS steps, and one slot of the pinv check that
// spi_krige_factor runs on exact-inverse systems of up to SPI_PINV_MAX_M
// rows (see spinterps_gb300.h); it is reserved on
// every GPU that loads this library, until the process exits. Every call
// shares it: calls whose work overlaps on the GPU (other streams, other
// host threads) race on it and must be serialised by the caller.
#include <mutex>

#include "spi_common.cuh"

namespace {

constexpr int GA = SPI_MAX_DRIFT + 1;
constexpr int MAXN = SPI_NOALLOC_MAX_STNS;
constexpr int MAXT = SPI_NOALLOC_MAX_STEPS;
constexpr int64_t ARENA = (int64_t)(MAXN + GA) * (MAXN + GA);

constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }

// byte offsets of the pieces of the scratch array
constexpr size_t OFF_L = 0;
constexpr size_t OFF_X = OFF_L + al(ARENA * 8);
constexpr size_t OFF_WHAT = OFF_X + al(ARENA * 8);
constexpr size_t OFF_BETA = OFF_WHAT + al((size_t)MAXT * MAXN * 8);
constexpr size_t OFF_GCOLS = OFF_BETA + al((size_t)MAXT * GA * 8);
constexpr size_t OFF_SINV = OFF_GCOLS + al((size_t)MAXN * GA * 8);
constexpr size_t OFF_GSUM = OFF_SINV + al((size_t)GA * GA * 8);
constexpr size_t OFF_COND = OFF_GSUM + al((size_t)GA * 8);
constexpr size_t OFF_SHIFT = OFF_COND + al(8);
constexpr size_t OFF_STATUS = OFF_SHIFT + al(8);
constexpr size_t OFF_ROUTE = OFF_STATUS + al(4);
constexpr size_t OFF_STNOFF = OFF_ROUTE + al(4);
constexpr size_t OFF_MATOFF = OFF_STNOFF + al(2 * 8);
constexpr size_t OFF_STEPOFF = OFF_MATOFF + al(8);
constexpr size_t OFF_VALOFF = OFF_STEPOFF + al(2 * 8);
constexpr size_t OFF_STEPS = OFF_VALOFF + al((size_t)MAXT * 8);
constexpr size_t OFF_OUTROW = OFF_STEPS + al((size_t)MAXT * 4);
constexpr size_t OFF_VG = OFF_OUTROW + al((size_t)MAXT * 4);
// one slot of the pinv check (spi_krige_factor): a one-system batch uses
// slot 0 only
constexpr size_t OFF_PINV = OFF_VG + al(sizeof(spi_vg_t));
constexpr size_t OFF_PUSED = OFF_PINV + al((size_t)2 * SPI_PINV_MAX_M * SPI_PINV_MAX_M * 8);
constexpr size_t SCRATCH_BYTES = OFF_PUSED + al(4);

static_assert(SCRATCH_BYTES == SPI_NOALLOC_SCRATCH_BYTES,
              "SPI_NOALLOC_SCRATCH_BYTES in spinterps_gb300.h is out of date");

// The scratch. Host code must never use this name as a device address:
// on the host it names a stand-in object, so its address comes from
// cudaGetSymbolAddress below, per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_ptr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached.
int scratch_ptr(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPI_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SPI_ERR_CUDA;
    g_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_ptr[dev];
  return SPI_OK;
}

// Descriptors of the one system, and zeroed dual columns / Lagrange
// coefficients (the scratch keeps the previous call's contents).
__global__ void k_noalloc_setup(unsigned char* base, int n, int n_steps, spi_vg_t vg) {
  int64_t* stn_off = reinterpret_cast<int64_t*>(base + OFF_STNOFF);
  int64_t* mat_off = reinterpret_cast<int64_t*>(base + OFF_MATOFF);
  int64_t* step_off = reinterpret_cast<int64_t*>(base + OFF_STEPOFF);
  int64_t* val_off = reinterpret_cast<int64_t*>(base + OFF_VALOFF);
  int32_t* steps = reinterpret_cast<int32_t*>(base + OFF_STEPS);
  int32_t* out_row = reinterpret_cast<int32_t*>(base + OFF_OUTROW);
  double* g_cols = reinterpret_cast<double*>(base + OFF_GCOLS);
  double* beta = reinterpret_cast<double*>(base + OFF_BETA);
  const int t = threadIdx.x;
  if (t == 0) {
    stn_off[0] = 0;
    stn_off[1] = n;
    mat_off[0] = 0;
    step_off[0] = 0;
    step_off[1] = n_steps;
    *reinterpret_cast<spi_vg_t*>(base + OFF_VG) = vg;
  }
  for (int j = t; j < n_steps; j += blockDim.x) {
    steps[j] = j;
    val_off[j] = (int64_t)j * n;
    out_row[j] = j;
  }
  for (int i = t; i < MAXN * GA; i += blockDim.x) g_cols[i] = 0.0;
  for (int i = t; i < MAXT * GA; i += blockDim.x) beta[i] = 0.0;
}

// The system's route, copied out of the scratch in stream order.
__global__ void k_noalloc_route(const unsigned char* base, int32_t* route_out) {
  *route_out = *reinterpret_cast<const int32_t*>(base + OFF_ROUTE);
}

}  // namespace

extern "C" int spi_krige_ok_noalloc(const spi_domain_t* dom, const int32_t* stn_idx,
                                    int32_t n, const spi_vg_t* vg, const double* vals,
                                    int32_t n_steps, int32_t want_var, const spi_out_t* out,
                                    spi_stream_t stream, int32_t* route_out) {
  if (!dom || !stn_idx || !vg || !vals || !out || !out->est) return SPI_ERR_ARG;
  if (n < 2 || n_steps < 1) return SPI_ERR_ARG;
  if (n > MAXN || n_steps > MAXT) return SPI_ERR_TOO_LARGE;
  if (vg->n_comp < 1 || vg->n_comp > SPI_MAX_VG_COMP) return SPI_ERR_VG;
  unsigned char* base = nullptr;
  int rc = scratch_ptr(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_setup<<<1, 256, 0, st>>>(base, n, n_steps, *vg);
  SPI_LAUNCH_CHECK();
  spi_systems_t sy;
  sy.n_sys = 1;
  sy.kind = SPI_KIND_OK;
  sy.stn_off = reinterpret_cast<const int64_t*>(base + OFF_STNOFF);
  sy.stn_idx = stn_idx;
  sy.vg = reinterpret_cast<const spi_vg_t*>(base + OFF_VG);
  sy.mat_off = reinterpret_cast<const int64_t*>(base + OFF_MATOFF);
  sy.step_off = reinterpret_cast<const int64_t*>(base + OFF_STEPOFF);
  sy.steps = reinterpret_cast<const int32_t*>(base + OFF_STEPS);
  sy.val_off = reinterpret_cast<const int64_t*>(base + OFF_VALOFF);
  sy.out_row = reinterpret_cast<const int32_t*>(base + OFF_OUTROW);
  sy.max_n = n;
  spi_krige_ws_t ws = {};
  ws.l_arena = reinterpret_cast<double*>(base + OFF_L);
  ws.linv_arena = reinterpret_cast<double*>(base + OFF_X);
  ws.status = reinterpret_cast<int32_t*>(base + OFF_STATUS);
  ws.route = reinterpret_cast<int32_t*>(base + OFF_ROUTE);
  ws.cond = reinterpret_cast<double*>(base + OFF_COND);
  ws.shift = reinterpret_cast<double*>(base + OFF_SHIFT);
  ws.w_hat = reinterpret_cast<double*>(base + OFF_WHAT);
  ws.beta = reinterpret_cast<double*>(base + OFF_BETA);
  ws.g_cols = reinterpret_cast<double*>(base + OFF_GCOLS);
  ws.s_inv = reinterpret_cast<double*>(base + OFF_SINV);
  ws.g_colsum = reinterpret_cast<double*>(base + OFF_GSUM);
  ws.pinv_scratch = reinterpret_cast<double*>(base + OFF_PINV);
  ws.pinv_used = reinterpret_cast<int32_t*>(base + OFF_PUSED);
  spi_domain_t d = *dom;
  d.n_drift = 0;  // ordinary kriging: the unbiasedness row only
  if ((rc = spi_krige_factor(&d, &sy, &ws, 1e13, stream))) return rc;
  if ((rc = spi_krige_duals(&d, &sy, vals, &ws, stream))) return rc;
  if ((rc = spi_krige_cells(&d, &sy, vals, &ws, want_var, 0, 0, 1e7, out, stream))) return rc;
  if (route_out) {
    k_noalloc_route<<<1, 1, 0, st>>>(base, route_out);
    SPI_LAUNCH_CHECK();
  }
  return SPI_OK;
}
