// lg_trace_common.cuh — small device helpers shared by the trace kernels of both precision
// modes (lg_trace.cu: FP32 scan and double-float solve; lg_exact.cu: exact FP64 solve).
#pragma once
#include "lg_kernels.cuh"

namespace lgd {

__device__ __forceinline__ bool below_cutoff(const float* c, const float* k) {
  return (c[0] < k[0] && c[1] < k[1] && c[2] < k[2]) || c[3] < k[3];
}
__device__ __forceinline__ bool near_cutoff(const float* c, const float* k) {
  bool n = false;
#pragma unroll
  for (int i = 0; i < 4; ++i) n |= fabsf(c[i] - k[i]) <= 1e-6f * k[i];
  return n;
}

// FP32 bounding-circle test shared by both scan passes: false if the object cannot hold a
// hit at a ray parameter <= thr; lb receives a lower bound of its hit distances.
__device__ __forceinline__ bool bound_test(const float4& h, float ox, float oy, float dx, float dy, float thr,
                                           float& lb) {
  const float ocx = h.x - ox, ocy = h.y - oy;
  const float b = ocx * dx + ocy * dy, perp = ocx * dy - ocy * dx;
  const float btol = 2e-6f * (fabsf(b) + fabsf(perp) + h.z) + 1e-6f;
  if (fabsf(perp) > h.z + btol || b + h.z + btol < -TAU32) return false;
  lb = b - h.z - btol;
  return lb <= thr;
}

// Queued rays a launch takes (the children of the previous generation or step) ...
__device__ __forceinline__ uint64_t n_real_of(const SceneDev& S, const TraceBufs& B, uint32_t gen) {
  if (gen == 0 && !S.serve) return 0;
  const unsigned long long n = B.ctr->queue_count[gen];
  return n < B.queue_cap ? n : B.queue_cap;
}
// ... and primaries it generates (virtual queue entries after the queued ones)
__device__ __forceinline__ uint64_t n_new_of(const SceneDev& S, uint32_t gen) {
  return S.serve ? S.n_new : (gen == 0 ? S.n_primary : 0);
}
__device__ __forceinline__ uint64_t n_in_of(const SceneDev& S, const TraceBufs& B, uint32_t gen) {
  const uint64_t n = n_real_of(S, B, gen) + n_new_of(S, gen);
  return n < B.queue_cap ? n : B.queue_cap;
}

}  // namespace lgd
