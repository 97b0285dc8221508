// Allocation-free per-vector inner products.
//
// qg_dot (qgpu_krylov.cu) takes its block partial sums from the context's scratch buffer and
// its result buffer from cudaMalloc.  Some callers cannot allocate: a serving loop that has
// handed all device memory to admitted jobs, or code that must not call cudaMalloc/cudaFree
// because those calls can synchronise the whole device.  qg_dot_noalloc serves them: the
// partial sums live in a file-scope device array of fixed size, the caller passes the inputs
// and a device output, and nothing is allocated.
//
// The call works on the calling thread's current device (cudaGetDevice): the pointers and the
// stream must belong to it.  The array's name is only a host-side stand-in for host code; the
// device address is obtained once per device with cudaGetSymbolAddress (the first call on a device does this set-up, so
// that first call should come before any stream capture).  Every call on a device shares the
// array and leaves its partial sums behind; calls that overlap on the GPU (other streams, or
// without ordering between them) race on it.  Each call writes every partial it later reads,
// so no clearing is needed.
#include <mutex>

#include "qgpu_internal.cuh"

// Limits of the static scratch: at most QG_NOALLOC_MAX_BLOCKS partial blocks per vector and
// QG_NOALLOC_MAX_VECTORS vectors (1 MiB of complex partial sums per device).
#define QG_NOALLOC_MAX_VECTORS 64
#define QG_NOALLOC_MAX_BLOCKS 1024

static __device__ __align__(256) double2 g_noalloc_partials[QG_NOALLOC_MAX_VECTORS * QG_NOALLOC_MAX_BLOCKS];

// the reduction kernels of qgpu_krylov.cu: per vector (one vector), or over the flat row-major
// block with a fixed vector per thread (several vectors: coalesced, every row read once)
__global__ void k_dot_partial(int64_t n, int nvec, const double2 *__restrict__ x, const double2 *__restrict__ y,
                              double2 *part);
__global__ void k_dot_partial_flat(int64_t len, int nvec, const double2 *__restrict__ x,
                                   const double2 *__restrict__ y, double2 *part);
__global__ void k_reduce_partials(const double2 *part, int nblk, int nvec, double2 *out);

namespace {

const int kMaxDevices = 64;
std::mutex g_mu;
double2 *g_ptr[kMaxDevices] = {nullptr};
int g_sms[kMaxDevices] = {0};

// Device address of the static partials on the current device (set up on first use).
cudaError_t setup(int dev, double2 **ptr, int *sms) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = (double2 *)p;
    g_sms[dev] = n;
  }
  *ptr = g_ptr[dev];
  *sms = g_sms[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" qg_status qg_dot_noalloc(int64_t n, int32_t nvec, const double *x_dev, const double *y_dev,
                                    double *out_dev, void *stream) {
  if (n < 0 || nvec <= 0 || nvec > QG_NOALLOC_MAX_VECTORS || !out_dev || (n > 0 && (!x_dev || !y_dev)))
    return QG_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return QG_ERR_CUDA;
  }
  double2 *part = nullptr;
  int sms = 0;
  if (setup(dev, &part, &sms) != cudaSuccess) {
    cudaGetLastError();
    return QG_ERR_CUDA;
  }
  int64_t blocks = (n + 255) / 256;
  int64_t cap = 4LL * sms;
  if (blocks > cap) blocks = cap;
  if (blocks > QG_NOALLOC_MAX_BLOCKS) blocks = QG_NOALLOC_MAX_BLOCKS;
  if (blocks < 1) blocks = 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (nvec > 1) {  // threads per block a multiple of nvec, so each thread keeps one vector
    const int T = nvec * (256 / nvec);
    k_dot_partial_flat<<<(unsigned)blocks, T, T * sizeof(double2), s>>>(n * nvec, nvec, (const double2 *)x_dev,
                                                                       (const double2 *)y_dev, part);
  } else {
    k_dot_partial<<<(unsigned)blocks, 256, (256 / 32) * sizeof(double2), s>>>(n, nvec, (const double2 *)x_dev,
                                                                            (const double2 *)y_dev, part);
  }
  k_reduce_partials<<<1, 256, 0, s>>>(part, (int)blocks, nvec, (double2 *)out_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}
