// lg_noalloc.cu — segment accumulation for callers that cannot allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: plug-ins whose host
// owns every device allocation and hands them only the buffers it made, real-time frame
// loops that must not take the allocator's locks or trigger the implicit device
// synchronisation cudaMalloc / cudaFree can cause, and code that runs against a fixed
// device-memory budget.  lg_accumulate_segments_noalloc serves them: it rasterises the
// caller's segments into the caller's accumulation image exactly like
// lg_accumulate_segments, without a context, and keeps all of its binning scratch (tile
// counts, offsets, cursors, work units and (segment, tile) references) in one file-scope
// device array of fixed size, g_noalloc_scratch, instead of allocating.
//
// The array exists once per device that loads the library and stays resident until the
// process exits.  Every call shares it: each call clears the parts that must start at
// zero, and calls that overlap on the GPU (different streams or host threads at the same
// time) race on it and must be serialised by the caller.  The first call on a device looks
// the array's device address up (cudaGetSymbolAddress) and configures the kernels; make
// that first call before any stream capture.
#include <cstring>
#include <mutex>

#include "lg_host.hpp"

using namespace lgd;

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 32ull << 20;  // 32 MiB per device
constexpr uint32_t NOALLOC_MAX_TILES = 4096;           // e.g. 2048 x 2048 pixels in 32 x 32 tiles
constexpr uint32_t NOALLOC_MAX_BINS = 2 * NOALLOC_MAX_TILES;
constexpr uint64_t NOALLOC_MAX_REFS = 8000000;         // (segment, tile) pairs per call
constexpr uint32_t NOALLOC_UNIT_REFS = 1024;           // units well within the shared-atomic raster's bound
constexpr uint64_t NOALLOC_MAX_UNITS = NOALLOC_MAX_BINS + NOALLOC_MAX_REFS / NOALLOC_UNIT_REFS + 1;
constexpr int MAX_DEVICES = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t OFF_CTR = 0;
constexpr size_t OFF_COUNT = align256(OFF_CTR + sizeof(Counters));
constexpr size_t OFF_TOFF = align256(OFF_COUNT + NOALLOC_MAX_BINS * 4);
constexpr size_t OFF_CURSOR = align256(OFF_TOFF + NOALLOC_MAX_BINS * 8);
constexpr size_t OFF_UOFF = align256(OFF_CURSOR + NOALLOC_MAX_BINS * 8);
constexpr size_t OFF_UNITS = align256(OFF_UOFF + NOALLOC_MAX_BINS * 8);
constexpr size_t OFF_REFS = align256(OFF_UNITS + NOALLOC_MAX_UNITS * sizeof(Unit));
constexpr size_t SCRATCH_END = OFF_REFS + NOALLOC_MAX_REFS * 4;
static_assert(SCRATCH_END <= NOALLOC_SCRATCH_BYTES, "no-alloc scratch layout exceeds the array");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

struct DeviceSetup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int n_sm = 0;
  int raster_grid = 0;
};

DeviceSetup g_setup[MAX_DEVICES];
std::mutex g_setup_mu;

__global__ void k_noalloc_init(Counters* ctr, unsigned long long n_segments) {
  unsigned int* w = reinterpret_cast<unsigned int*>(ctr);
  for (size_t i = threadIdx.x; i < sizeof(Counters) / 4; i += blockDim.x) w[i] = 0u;
  __syncthreads();
  if (threadIdx.x == 0) ctr->seg_count = n_segments;
}

// once per device, with that device current
lg_status setup_device(int dev, DeviceSetup*& out) {
  if (dev < 0 || dev >= MAX_DEVICES) return LG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& d = g_setup[dev];
  if (!d.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      return LG_ERR_CUDA;
    }
    int n_sm = 0;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LG_ERR_CUDA;
    const int rsm[3] = {raster_smem_bytes(RM_FIXED_SPLIT_), raster_smem_bytes(RM_FIXED_MINMAX_), raster_smem_bytes(RM_F32_)};
    cudaError_t e = cudaFuncSetAttribute(k_raster<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm[0]);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_raster<RM_FIXED_MINMAX_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm[1]);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_raster<RM_F32_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm[2]);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_bin_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(MAX_SMEM_TILES * 4));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_bin_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(MAX_SMEM_TILES * 4));
    int occ = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_SPLIT_>, 256, rsm[0]);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return LG_ERR_CUDA;
    }
    d.scratch = static_cast<unsigned char*>(p);
    d.n_sm = n_sm;
    d.raster_grid = n_sm * (occ > 0 ? occ : 1);
    d.ready = true;
  }
  out = &d;
  return LG_OK;
}

}  // namespace

extern "C" lg_status lg_accumulate_segments_noalloc(const lg_segment* segments, uint64_t n, const lg_params* params,
                                                    void* accum, void* stream, uint64_t* pixels_out) {
  if (!params || !accum || (n && !segments)) return LG_ERR_INVALID_ARGUMENT;
  const lg_params& p = *params;
  // the same canvas, accumulation and blend rules as a context's lg_params
  if (p.width == 0 || p.height == 0 || p.width > 32768 || p.height > 32768 ||
      (p.accum != LG_ACCUM_FIXED64 && p.accum != LG_ACCUM_F32))
    return LG_ERR_INVALID_ARGUMENT;
  if (!lgh::blend_supported(p.color_blend) || !lgh::blend_supported(p.alpha_blend)) return LG_ERR_UNSUPPORTED;
  const uint32_t ntx = (p.width + TILE - 1) / TILE, nty = (p.height + TILE - 1) / TILE;
  if ((uint64_t)ntx * nty > NOALLOC_MAX_TILES || n > 0xffffffffull) return LG_ERR_BUDGET;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LG_ERR_CUDA;
  DeviceSetup* d = nullptr;
  lg_status st = setup_device(dev, d);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = d->scratch;
  const uint32_t n_tiles = ntx * nty;

  RasterArgs A;
  std::memset(&A, 0, sizeof A);
  A.segs = segments;
  A.seg_cap = n;
  A.W = p.width;
  A.H = p.height;
  A.ntx = ntx;
  A.nty = nty;
  A.n_tiles = 2 * n_tiles;  // bins: x-major and y-major segments of each tile
  A.unit_refs = NOALLOC_UNIT_REFS;
  for (int ch = 0; ch < 4; ++ch) {
    const lg_blend_component& b = ch < 3 ? p.color_blend : p.alpha_blend;
    A.blend.src[ch] = b.src_factor;
    A.blend.op[ch] = b.op;
    A.blend.constant[ch] = p.blend_constant[ch];
    A.blend.clear[ch] = p.clear_color[ch];
  }
  A.ctr = reinterpret_cast<Counters*>(base + OFF_CTR);
  A.tile_count = reinterpret_cast<uint32_t*>(base + OFF_COUNT);
  A.tile_off = reinterpret_cast<uint64_t*>(base + OFF_TOFF);
  A.tile_cursor = reinterpret_cast<unsigned long long*>(base + OFF_CURSOR);
  A.unit_off = reinterpret_cast<uint64_t*>(base + OFF_UOFF);
  A.units = reinterpret_cast<Unit*>(base + OFF_UNITS);
  A.units_cap = NOALLOC_MAX_UNITS;
  A.refs = reinterpret_cast<uint32_t*>(base + OFF_REFS);
  A.refs_cap = NOALLOC_MAX_REFS;
  A.accum = accum;

  const int fixed = p.accum == LG_ACCUM_FIXED64;
  const uint32_t bins = A.n_tiles;
  const int smem_tiles = bins <= MAX_SMEM_TILES ? 1 : 0;
  const size_t bsm = smem_tiles ? (size_t)bins * 4 : 0;
  const int mode = lgh::raster_mode(p);
  const size_t rsm = (size_t)raster_smem_bytes(mode);
  // the previous call's contents stay in the array: counters and tile counts restart at 0
  k_noalloc_init<<<1, 256, 0, s>>>(A.ctr, (unsigned long long)n);
  if (cudaMemsetAsync(A.tile_count, 0, (size_t)bins * 4, s) != cudaSuccess) return LG_ERR_CUDA;
  k_clear_accum<<<d->n_sm * 8, 256, 0, s>>>(A, fixed);
  k_bin_count<<<d->n_sm * 8, 256, bsm, s>>>(A, smem_tiles);
  k_scan_tiles<<<1, 1024, 0, s>>>(A);
  k_build_units<<<(bins + 255) / 256, 256, 0, s>>>(A);
  k_bin_scatter<<<scatter_grid(d->n_sm, smem_tiles), SCATTER_THREADS, bsm, s>>>(A, smem_tiles);
  if (mode == RM_FIXED_SPLIT_)
    k_raster<RM_FIXED_SPLIT_><<<d->raster_grid, 256, rsm, s>>>(A);
  else if (mode == RM_FIXED_MINMAX_)
    k_raster<RM_FIXED_MINMAX_><<<d->raster_grid, 256, rsm, s>>>(A);
  else
    k_raster<RM_F32_><<<d->raster_grid, 256, rsm, s>>>(A);
  if (cudaGetLastError() != cudaSuccess) return LG_ERR_CUDA;
  unsigned long long counts[2] = {0, 0};
  if (cudaMemcpyAsync(&counts[0], &A.ctr->tile_refs, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&counts[1], &A.ctr->pixels, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    (void)cudaGetLastError();
    return LG_ERR_CUDA;
  }
  if (counts[0] > NOALLOC_MAX_REFS) return LG_ERR_BUDGET;  // the image is incomplete
  if (pixels_out) *pixels_out = counts[1];
  return LG_OK;
}
