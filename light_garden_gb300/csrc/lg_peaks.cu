// lg_peaks.cu — throughput ceilings of the GPU the benchmark runs on (liblg_peaks.so).
//
// The tile raster accumulates in shared memory (32-bit atomic adds on the split planes), the
// trace issues FP32 and, in the exact precision mode, FP64 arithmetic.  Their rooflines are
// measured here, on the same GPU and in the same process as the benchmark, with kernels that
// do nothing but that one operation:
//   smem_atomics_per_s  32-bit shared-memory atomicAdd, 256 threads x 4 CTAs per SM (the
//                       raster's launch shape), each warp on 32 distinct banks of a 32 KB plane
//   fp32_fma_per_s      independent FFMA chains, 8 per thread
//   fp64_op_per_s       independent DADD / DMUL chains (never fused), 4 per thread
// Each figure is lane operations per second over the whole GPU, from CUDA events after a
// warm-up launch.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__global__ void __launch_bounds__(256, 4) k_smem_atomics(unsigned* out, int iters) {
  __shared__ unsigned plane[8192];
  for (int i = threadIdx.x; i < 8192; i += blockDim.x) plane[i] = 0u;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  unsigned cell = warp * 1024u + lane;
  for (int it = 0; it < iters; ++it) {
    atomicAdd(&plane[cell], 1u);
    atomicAdd(&plane[(cell + 32u) & 8191u], 3u);
    cell = (cell + 64u) & 8191u;
  }
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = plane[lane];
}

__global__ void k_fp32(float* out, float a, float b, int iters) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_fp64(double* out, double a, double b, int iters) {
  double x[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = __dadd_rn(__dmul_rn(x[k], a), b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class L>
float time_ms(L&& launch) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch();  // warm-up
  cudaEventRecord(a);
  launch();
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

}  // namespace

extern "C" {

typedef struct lgp_peaks {
  double smem_atomics_per_s;
  double fp32_fma_per_s;
  double fp64_op_per_s;
  int32_t n_sm;
  int32_t status;  // 0 ok, else a cudaError_t
} lgp_peaks;

int lgp_measure(int device, lgp_peaks* out) {
  if (!out) return 1;
  out->status = 0;
  cudaError_t e = cudaSetDevice(device);
  int n_sm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return out->status = (int)e;
  out->n_sm = n_sm;
  const int blocks = n_sm * 4, threads = 256;
  void* buf = nullptr;
  if ((e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double))) != cudaSuccess) return out->status = (int)e;
  const int it_a = 1 << 14, it_f = 1 << 15, it_d = 1 << 11;
  float ms = time_ms([&] { k_smem_atomics<<<blocks, threads>>>((unsigned*)buf, it_a); });
  out->smem_atomics_per_s = 2.0 * it_a * (double)blocks * threads / (ms * 1e-3);
  ms = time_ms([&] { k_fp32<<<blocks, threads>>>((float*)buf, 0.999f, 1e-3f, it_f); });
  out->fp32_fma_per_s = 8.0 * it_f * (double)blocks * threads / (ms * 1e-3);
  ms = time_ms([&] { k_fp64<<<blocks, threads>>>((double*)buf, 0.999, 1e-3, it_d); });
  out->fp64_op_per_s = 8.0 * it_d * (double)blocks * threads / (ms * 1e-3);
  e = cudaGetLastError();
  cudaFree(buf);
  return out->status = (int)e;
}

}  // extern "C"
