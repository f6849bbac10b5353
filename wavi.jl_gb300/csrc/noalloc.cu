// noalloc.cu — wavi_residual_noalloc: the float64 momentum-operator residual r = b - A x with its
// squared norm, for callers that cannot allocate device memory.
//
// Who cannot allocate: code that runs inside another runtime's memory discipline — a host framework
// that owns the whole device heap through its own pool allocator, code running inside a CUDA graph
// capture or a callback where cudaMalloc is forbidden, or long-running services whose allocation
// budget is fixed at start-up.  Such a caller already holds the operator coefficients and vectors in
// its own buffers; this entry point needs nothing else from it.
//
// The reduction scratch (block partial sums and the last-block counter) is a file-scope static
// __device__ array of a fixed size, resident on every device that loads the library until the process
// exits.  Host code cannot use the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current) and caches it for the life
// of the process.  cudaDeviceReset() unloads the module that holds the array, which leaves the cached
// address stale: the header tells callers not to use this entry point on a device after a reset.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/wavi_gpu.h"
#include "kernels.cuh"
#include "fused.cuh"

namespace wavi {
void set_global_error(const std::string& msg);  // wavi_gpu.cu
}

namespace {

using namespace wavi;

// At most this many 32 x 8 operator tiles, i.e. (nx+1)*(ny+1) up to about 4.19 million points.
constexpr int kMaxBlocks = WAVI_NOALLOC_MAX_TILES;
constexpr int kScratchDoubles = 2 * kMaxBlocks + 32;  // two partial sums per block, then the counter

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

int noalloc_fail(int code, const std::string& msg) {
  wavi::set_global_error(msg);  // reported by wavi_last_error(NULL)
  return code;
}

// r = b - A x on one tile; |r|^2 reduced by the last block into *rr_out.  The same stencil as the
// solve's float64 residual kernel, with its scratch taken from g_noalloc_scratch (passed as `scratch`).
template <int TX, int TY>
__global__ void __launch_bounds__(TX* TY)
    k_residual_noalloc(Dims d, OpCoef<double> cf, const double* __restrict__ x, const double* __restrict__ b,
                       double* __restrict__ r, double* __restrict__ rr_out, double* __restrict__ scratch) {
  __shared__ OpTile<double, TX, TY> s;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  stage_x(d, i0, j0, s, [&](int q) { return x[q]; });
  __syncthreads();
  stage_stress(d, cf, i0, j0, s);
  __syncthreads();
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1, i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  double rr = 0.0;
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    const double v = cf.inner[q] ? b[q] - stage_out_u(d, cf, s, li, lj, q) : 0.0;
    r[q] = v;
    rr += v * v;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    const double v = cf.inner[q] ? b[q] - stage_out_v(d, cf, s, li, lj, q) : 0.0;
    r[q] = v;
    rr += v * v;
  }
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + 2 * kMaxBlocks);
  double tot[2];
  if (last_block_sum2(rr, 0.0, scratch, counter, tot)) {
    if (flat_tid() == 0) *rr_out = tot[0];
  }
}

// Once per device, with that device current: the device address of the scratch array.
int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(WAVI_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(WAVI_ERR_ARGUMENT, "device ordinal beyond the supported range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return noalloc_fail(WAVI_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return 0;
}

}  // namespace

extern "C" {

int wavi_residual_noalloc(const wavi_operator_desc* op, const double* x_uv, const double* b_uv, double* r_uv,
                          double* rr_out, void* stream) {
  if (!op || !x_uv || !b_uv || !r_uv || !rr_out) return noalloc_fail(WAVI_ERR_ARGUMENT, "null argument");
  if (!op->heta_h || !op->heta_c || !op->dimp || !op->beta_m || !op->h_m || !op->inner)
    return noalloc_fail(WAVI_ERR_ARGUMENT, "null coefficient array");
  if (op->nx < 2 || op->ny < 2 || !(op->dx > 0) || !(op->dy > 0))
    return noalloc_fail(WAVI_ERR_ARGUMENT, "nx, ny must be > 1 and dx, dy positive");
  const long gx = (op->nx + 1 + OP_TX - 1) / OP_TX, gy = (op->ny + 1 + OP_TY - 1) / OP_TY;
  if (gx * gy > kMaxBlocks)
    return noalloc_fail(WAVI_ERR_ARGUMENT,
                        "grid too large for wavi_residual_noalloc: (nx+1)*(ny+1) needs " + std::to_string(gx * gy) +
                            " tiles of 32x8 points, the static scratch holds " + std::to_string(kMaxBlocks));
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  Dims d{};
  d.nx = op->nx;
  d.ny = op->ny;
  d.ns = 0;
  d.Nh = d.nx * d.ny;
  d.Nu = (d.nx + 1) * d.ny;
  d.Nv = d.nx * (d.ny + 1);
  d.Nc = (d.nx - 1) * (d.ny - 1);
  d.N = d.Nu + d.Nv;
  d.dx = op->dx;
  d.dy = op->dy;
  d.rdx = 1.0 / op->dx;
  d.rdy = 1.0 / op->dy;
  d.rdx_f = (float)d.rdx;
  d.rdy_f = (float)d.rdy;
  OpCoef<double> cf{op->heta_h, op->heta_c, op->dimp, op->beta_m, op->h_m, op->inner};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the last-block counter must start at zero; the partial sums are fully rewritten by every call
  cudaError_t e = cudaMemsetAsync(scratch + 2 * kMaxBlocks, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return noalloc_fail(WAVI_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  k_residual_noalloc<OP_TX, OP_TY><<<dim3((unsigned)gx, (unsigned)gy), dim3(OP_TX, OP_TY), 0, st>>>(d, cf, x_uv, b_uv, r_uv,
                                                                                                    rr_out, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(WAVI_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return WAVI_OK;
}

}  // extern "C"
