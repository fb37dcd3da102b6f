// G x without any device allocation, for callers that cannot allocate.
//
// Who needs it: code that runs the product while a device allocation is not
// allowed or not affordable -- between the kernels of another library's CUDA
// stream capture (cudaMalloc is illegal while a capture is open), under a
// device-memory budget owned by the caller's own allocator, or on a latency
// path where cudaMalloc/cudaFree would synchronise the whole device.  The
// regular entry point (grada_G_vec_mul_dev) takes its scratch from the
// library context, which allocates it on first use; this one takes it from a
// fixed array compiled into the library instead.
//
// The scratch is the file-scope array below: 8 MiB (1,048,576 doubles) on
// every GPU that loads the library, held until the process exits.  It holds
// the per-column-range partial row sums of the product, so a call needs
// splits * ld doubles with ld the padded row count; ld up to 1,048,576 is
// accepted (the column ranges shrink to fit) and larger G is rejected with
// GRADA_ERR_SCRATCH_LIMIT.  Every call overwrites the partial sums it reads,
// so nothing has to start at zero; but all calls on a device share the one
// array, so calls whose kernels can overlap on the GPU (different streams
// without ordering between them) race on it.
//
// The host cannot use the array's name as a device address: host code sees a
// stand-in, and a kernel given that stand-in would fault or touch the wrong
// memory.  The first call on each device (with that device current) looks up
// the real address with cudaGetSymbolAddress and caches it; make that first
// call before any stream capture that should contain later calls.  The cached
// address belongs to the device's current context: after cudaDeviceReset (or
// any teardown of the primary context) the library's module is loaded again
// at a new address, so a process that resets a device must not call this
// entry point on that device again.
//
// Errors: the kernels are launched with cudaLaunchKernel and only those
// launches' own status is checked, so an error left pending by the caller's
// earlier work is neither reported as this call's nor cleared.
#include <mutex>

#include "../../include/grada_gpu.h"
#include "common.cuh"

namespace {

constexpr int64_t kScratchDoubles = 1 << 20;  // 8 MiB
constexpr int NA_THREADS = 256;
constexpr int NA_VEC = 2;       // doubles per 16-byte load
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {};

// Partial row sums of G x over one column range per blockIdx.y.
__global__ void __launch_bounds__(NA_THREADS)
    noalloc_gx_partial_kernel(const double *__restrict__ G, int64_t ld, int64_t nm,
                              int64_t cols_per_split, const double *__restrict__ x,
                              double *__restrict__ partial) {
  constexpr int XCH = 256;
  __shared__ double xs[XCH];
  const int64_t row = ((int64_t)blockIdx.x * NA_THREADS + threadIdx.x) * NA_VEC;
  const int64_t c_begin = (int64_t)blockIdx.y * cols_per_split;
  const int64_t c_end = min(nm, c_begin + cols_per_split);
  double a0 = 0.0, a1 = 0.0;
  for (int64_t c0 = c_begin; c0 < c_end; c0 += XCH) {
    const int nc = (int)min((int64_t)XCH, c_end - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc; t += NA_THREADS) xs[t] = x[c0 + t];
    __syncthreads();
    if (row < ld) {
      const double *g = G + row + c0 * ld;
      for (int c = 0; c < nc; c++) {
        const double2 v = __ldcs(reinterpret_cast<const double2 *>(g + (int64_t)c * ld));
        a0 = fma(v.x, xs[c], a0);
        a1 = fma(v.y, xs[c], a1);
      }
    }
  }
  if (row < ld) {
    double *out = partial + (int64_t)blockIdx.y * ld + row;
    out[0] = a0;
    out[1] = a1;
  }
}

__global__ void noalloc_gx_finish_kernel(const double *__restrict__ partial, int n_split,
                                         int64_t ld, int64_t nd, double *__restrict__ y) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  double s = 0.0;
  for (int k = 0; k < n_split; k++) s += partial[(int64_t)k * ld + r];
  y[r] = s;
}

// Device address of the scratch array on the current device (looked up once).
int scratch_address(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GRADA_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GRADA_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GRADA_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[dev];
  return GRADA_OK;
}

}  // namespace

extern "C" int grada_G_vec_mul_noalloc(const double *d_G, int64_t nd, int64_t nm, int64_t ld,
                                       const double *d_x, double *d_y, void *stream) {
  if (!d_G || !d_x || !d_y || nd <= 0 || nm <= 0 || ld < nd || (ld % NA_VEC) != 0)
    return GRADA_ERR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(d_G) & 15u) != 0) return GRADA_ERR_INVALID_ARGUMENT;
  if (ld > kScratchDoubles) return GRADA_ERR_SCRATCH_LIMIT;
  double *scratch = nullptr;
  const int st = scratch_address(&scratch);
  if (st != GRADA_OK) return st;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return GRADA_ERR_CUDA;
  const int64_t tiles = grada::ceil_div(ld, (int64_t)NA_THREADS * NA_VEC);
  int64_t splits = grada::ceil_div((int64_t)sms * 8, tiles);
  splits = std::min<int64_t>(splits, grada::ceil_div(nm, 64));
  splits = std::min<int64_t>(splits, kScratchDoubles / ld);  // fits the fixed scratch
  splits = std::max<int64_t>(std::min<int64_t>(splits, 65535), 1);
  const int64_t per = grada::ceil_div(nm, splits);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid((unsigned)tiles, (unsigned)splits);
  void *partial_args[] = {(void *)&d_G, (void *)&ld, (void *)&nm, (void *)&per, (void *)&d_x,
                          (void *)&scratch};
  if (cudaLaunchKernel(reinterpret_cast<const void *>(&noalloc_gx_partial_kernel), grid,
                       dim3(NA_THREADS), partial_args, 0, s) != cudaSuccess)
    return GRADA_ERR_CUDA;
  int n_split = (int)splits;
  void *finish_args[] = {(void *)&scratch, (void *)&n_split, (void *)&ld, (void *)&nd,
                         (void *)&d_y};
  if (cudaLaunchKernel(reinterpret_cast<const void *>(&noalloc_gx_finish_kernel),
                       dim3((unsigned)grada::ceil_div(nd, 256)), dim3(256), finish_args, 0,
                       s) != cudaSuccess)
    return GRADA_ERR_CUDA;
  return GRADA_OK;
}
