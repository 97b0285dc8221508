// Measurement probes of bench.py (not part of libqgpu): the FP64 issue ceiling and the
// random-sector gather bandwidth of the device, the denominators of the H*psi roofline's FP64
// and gather figures.  Built by __graft_entry__.build() into bench_probe.so; plain C ABI, the
// caller's CUDA stream, no state.
#include <cuda_runtime.h>
#include <stdint.h>

// every thread runs 8 independent FMA chains in registers, all lanes active, no memory traffic
__global__ void k_fp64_probe(int iters, double m, double c, double *out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  if (s == -1.0) out[0] = s;  // never taken (the chains stay positive), keeps the work
}

static __host__ __device__ inline uint64_t mix64(uint64_t h) {
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

// each thread reads four 32-byte sectors at independent pseudo-random positions
__global__ void k_gather_probe(const double2 *__restrict__ a, uint64_t mask, int64_t n, double *out, uint64_t salt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint64_t j = mix64((uint64_t)i * 4 + k + salt) & mask;
    double2 v0 = __ldg(a + 2 * j), v1 = __ldg(a + 2 * j + 1);
    s += v0.x + v1.y;
  }
  if (s != 0.0) out[0] = s;  // the buffer is zero: never taken, keeps the loads
}

// FP64 lane operations per second (G) on num_sms * 8 blocks of 256 threads; 0 ok, 1 CUDA error
extern "C" int bench_fp64_peak(void *stream, double *gops) {
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&out, 8);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int iters = 4096, bs = 256;
  const unsigned grid = (unsigned)sms * 8;
  float ms = 0;
  if (e == cudaSuccess) {
    k_fp64_probe<<<grid, bs, 0, s>>>(iters, 0.9999999, 1e-9, out);  // warm
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; r++) k_fp64_probe<<<grid, bs, 0, s>>>(iters, 0.9999999, 1e-9, out);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return 1;
  *gops = (double)grid * bs * iters * 8 * 3 / (ms * 1e-3) / 1e9;
  return 0;
}

// GB/s of 32-byte sectors read at unrelated addresses spread over `bytes` (>= 1 MiB)
extern "C" int bench_gather_bandwidth(void *stream, int64_t bytes, double *gbs) {
  if (bytes < (1 << 20)) return 1;
  cudaStream_t s = (cudaStream_t)stream;
  uint64_t nsec = 1;
  while (nsec * 2 * 32 <= (uint64_t)bytes) nsec *= 2;
  double2 *a = nullptr;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&a, nsec * 32);
  if (e == cudaSuccess) e = cudaMalloc(&out, 8);
  if (e == cudaSuccess) e = cudaMemsetAsync(a, 0, nsec * 32, s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0;
  int64_t nthr = (int64_t)(nsec / 4);  // 4 sectors per thread: one pass reads nsec sectors
  unsigned grid = (unsigned)((nthr + 255) / 256);
  if (e == cudaSuccess) {
    k_gather_probe<<<grid, 256, 0, s>>>(a, nsec - 1, nthr, out, 1);  // warm
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; r++) k_gather_probe<<<grid, 256, 0, s>>>(a, nsec - 1, nthr, out, 2 + r);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(out);
  if (e != cudaSuccess) return 1;
  *gbs = (double)nthr * 4 * 32 * 3 / (ms * 1e-3) / 1e9;
  return 0;
}
