// lg_raster.cu — line accumulation and resolve (sm_103a).
//
// The reference draws its segment list as a 1-px LineList with additive blending into an
// Rgba16Float texture (src/sub_render_pass.rs:43-101, src/light_garden/mod.rs:57-73,
// src/texture_renderer.rs:5) and resolves it with a textured quad
// (src/render_to_texture.wgsl:17-28).  Here:
//   1. k_bin_count / k_scan_tiles / k_build_units / k_bin_scatter sort (segment, tile)
//      pairs into per-tile lists (32 x 32 px tiles) and cut each list into work units;
//   2. k_raster: persistent CTAs take units from a device counter, accumulate the unit's
//      segments into a shared-memory tile with shared atomics (one warp per segment, one
//      lane per major-axis pixel), then flush the tile with one global atomic per pixel
//      channel.  Fixed-point (int64 Q31.32) sums make the image independent of the order
//      in which units and segments are processed, so it is bit-reproducible;
//   3. k_resolve_f16: Q31.32 -> f32 -> binary16 (RNE), 8 B per pixel.
#include <cuda_fp16.h>

#include <type_traits>

#include "lg_kernels.cuh"

namespace lgd {

// ------------------------------------------------------------------ blend helpers
__device__ __forceinline__ float blend_factor(int f, int ch, const float* src, const float* k) {
  switch (f) {
    case LG_BF_ZERO: return 0.0f;
    case LG_BF_ONE: return 1.0f;
    case LG_BF_SRC: return src[ch];
    case LG_BF_ONE_MINUS_SRC: return __fsub_rn(1.0f, src[ch]);
    case LG_BF_SRC_ALPHA: return src[3];
    case LG_BF_ONE_MINUS_SRC_ALPHA: return __fsub_rn(1.0f, src[3]);
    case LG_BF_CONSTANT: return k[ch];
    default: return __fsub_rn(1.0f, k[ch]);
  }
}

__device__ __forceinline__ float contribution(const BlendDev& B, int ch, const float* src) {
  if (B.op[ch] == LG_BO_MIN || B.op[ch] == LG_BO_MAX) return src[ch];
  return __fmul_rn(src[ch], blend_factor(B.src[ch], ch, src, B.constant));
}

__device__ __forceinline__ long long ident64(int op) {
  return op == LG_BO_MIN ? 0x7fffffffffffffffll : (op == LG_BO_MAX ? (long long)0x8000000000000000ull : 0ll);
}
__device__ __forceinline__ float ident32(int op) {
  return op == LG_BO_MIN ? INFINITY : (op == LG_BO_MAX ? -INFINITY : 0.0f);
}

// ------------------------------------------------------------------ clear
__global__ void k_clear_accum(RasterArgs A, int fixed) {
  const uint64_t n = (uint64_t)A.W * A.H;
  if (fixed) {
    longlong4_32a c;
    c.x = to_fixed(A.blend.clear[0]);
    c.y = to_fixed(A.blend.clear[1]);
    c.z = to_fixed(A.blend.clear[2]);
    c.w = to_fixed(A.blend.clear[3]);
    longlong4_32a* p = reinterpret_cast<longlong4_32a*>(A.accum);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
      p[i] = c;
  } else {
    const float4 c = make_float4(A.blend.clear[0], A.blend.clear[1], A.blend.clear[2], A.blend.clear[3]);
    float4* p = reinterpret_cast<float4*>(A.accum);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
      p[i] = c;
  }
}

// ------------------------------------------------------------------ canvases
// The canvas a segment or a bin belongs to: the context's one canvas, or in a
// multi-scene accumulation the scene's own.
struct CanvasLoc {
  uint32_t W, H, ntx;
  uint64_t bin_base, px_base;
};
__device__ __forceinline__ CanvasLoc canvas_one(const RasterArgs& A) {
  CanvasLoc C;
  C.W = A.W; C.H = A.H; C.ntx = A.ntx; C.bin_base = 0; C.px_base = 0;
  return C;
}
__device__ __forceinline__ CanvasLoc canvas_at(const RasterArgs& A, uint32_t s) {
  const SceneCanvas& K = A.canvases[s];
  CanvasLoc C;
  C.W = K.W; C.H = K.H; C.ntx = K.ntx; C.bin_base = K.bin_base; C.px_base = K.px_base;
  return C;
}
__device__ __forceinline__ CanvasLoc canvas_of_bin(const RasterArgs& A, uint64_t bin) {
  if (!A.seg_scene) return canvas_one(A);
  uint32_t lo = 0, hi = A.n_scenes;  // the last scene whose first bin is <= bin
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (A.canvases[mid].bin_base <= bin) lo = mid; else hi = mid;
  }
  return canvas_at(A, lo);
}

// ------------------------------------------------------------------ binning
// The tiles that tile column tm (major-axis tiles) of a segment touches: the minor range is
// bounded by the samples at the column's two ends, since v(i) is monotone in i, and with
// |slope| <= 1 it spans at most two tiles.
template <class F>
__device__ __forceinline__ void column_tiles(const RSetup& R, const CanvasLoc& A, int tm, F&& f) {
  const int nmin = (int)(R.xmajor ? A.H : A.W);
  const int a = max(R.lo, tm * TILE), b = min(R.hi, tm * TILE + TILE) - 1;
  const int ja = raster_minor(R, a), jb = raster_minor(R, b);
  int jlo = min(ja, jb), jhi = max(ja, jb);
  if (jhi < 0 || jlo >= nmin) return;
  jlo = max(jlo, 0);
  jhi = min(jhi, nmin - 1);
  for (int tn = jlo / TILE; tn <= jhi / TILE; ++tn) {
    // bin id = 2 * tile + orientation: x-major and y-major segments of a tile are
    // rasterised in separate units, each with a bank-conflict-free layout
    const uint32_t tile = R.xmajor ? (uint32_t)tn * A.ntx + (uint32_t)tm : (uint32_t)tm * A.ntx + (uint32_t)tn;
    f((uint32_t)(A.bin_base + 2u * tile + (R.xmajor ? 0u : 1u)));
  }
}

// Visits every tile that holds at least one pixel of the segment.
template <class F>
__device__ __forceinline__ void for_each_tile(const RSetup& R, const CanvasLoc& A, F&& f) {
  const int tlo = R.lo / TILE, thi = (R.hi - 1) / TILE;
  for (int tm = tlo; tm <= thi; ++tm) column_tiles(R, A, tm, f);
}

__device__ __forceinline__ uint64_t n_segments(const RasterArgs& A) {
  const unsigned long long n = A.ctr->seg_count;
  return n < A.seg_cap ? n : A.seg_cap;
}

// Every (segment, bin) pair of the calling warp's share of the segments (32 consecutive
// segments per warp step, warp-strided over the grid), with the lanes spread densely over
// the step's tile columns: the 32 segments are set up lane-parallel, their column counts
// prefix-summed, and lane L takes columns L, L + 32, ... of the step, finding each column's
// segment by a binary search over the prefix sums with shuffles.  A segment that crosses
// many tiles is shared by the warp instead of keeping 31 lanes waiting.  f(segment, bin).
// Every lane of the warp calls it (the loops are warp-uniform).
template <class F>
__device__ __forceinline__ void for_each_pair_dense(const RasterArgs& A, uint64_t n, F&& f) {
  const unsigned lane = lane_id();
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = ((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) * 32; base < n; base += nw * 32) {
    const uint64_t i = base + lane;
    RSetup R;
    R.xmajor = 0; R.ua = 0.0f; R.va = 0.0f; R.slope = 0.0f; R.lo = 0; R.hi = 0;
    uint32_t sc = 0;
    int cnt = 0;
    if (i < n) {
      const float4 g = __ldg(reinterpret_cast<const float4*>(A.segs + i));
      if (A.seg_scene) sc = A.seg_scene[i];
      const CanvasLoc C = A.seg_scene ? canvas_at(A, sc) : canvas_one(A);
      lg_segment sg;
      sg.x0 = g.x; sg.y0 = g.y; sg.x1 = g.z; sg.y1 = g.w;
      if (raster_setup(sg, C.W, C.H, R)) cnt = (R.hi - 1) / TILE - R.lo / TILE + 1;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    const int excl = incl - cnt;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    for (int p0 = 0; p0 < total; p0 += 32) {
      const int p = p0 + (int)lane;
      // owner: the last lane whose exclusive prefix is <= p (a lane without columns shares
      // its prefix with the next lane and loses the search to it)
      int k = 0;
#pragma unroll
      for (int st = 16; st > 0; st >>= 1)
        if (__shfl_sync(0xffffffffu, excl, k + st) <= p) k += st;
      RSetup Q;
      Q.xmajor = __shfl_sync(0xffffffffu, R.xmajor, k);
      Q.ua = __shfl_sync(0xffffffffu, R.ua, k);
      Q.va = __shfl_sync(0xffffffffu, R.va, k);
      Q.slope = __shfl_sync(0xffffffffu, R.slope, k);
      Q.lo = __shfl_sync(0xffffffffu, R.lo, k);
      Q.hi = __shfl_sync(0xffffffffu, R.hi, k);
      const uint32_t qsc = __shfl_sync(0xffffffffu, sc, k);
      const int qexcl = __shfl_sync(0xffffffffu, excl, k);
      if (p < total) {
        const CanvasLoc C = A.seg_scene ? canvas_at(A, qsc) : canvas_one(A);
        const uint64_t seg = base + (uint64_t)k;
        column_tiles(Q, C, Q.lo / TILE + (p - qexcl), [&](uint32_t bin) { f(seg, bin); });
      }
    }
  }
}

// Per-CTA tile histogram in shared memory (native 32-bit shared atomics), one global
// atomic per touched tile per CTA.  Falls back to warp-aggregated global atomics when the
// tile count does not fit (smem_tiles == 0).
__global__ void __launch_bounds__(SCATTER_THREADS) k_bin_count(RasterArgs A, int smem_tiles) {
  if (A.ctr->skip_raster) return;
  extern __shared__ unsigned hist[];
  const uint64_t n = n_segments(A);
  if (smem_tiles) {
    for (uint32_t t = threadIdx.x; t < A.n_tiles; t += blockDim.x) hist[t] = 0;
    __syncthreads();
  }
  for_each_pair_dense(A, n, [&](uint64_t, uint32_t tile) {
    if (smem_tiles) {
      atomicAdd(&hist[tile], 1u);
    } else {
      const unsigned act = __activemask();
      const unsigned grp = __match_any_sync(act, tile);
      const int leader = __ffs(grp) - 1;
      if ((int)lane_id() == leader) atomicAdd(&A.tile_count[tile], (unsigned)__popc(grp));
    }
  });
  if (smem_tiles) {
    __syncthreads();
    uint32_t* mine = A.cta_hist ? A.cta_hist + (uint64_t)blockIdx.x * A.n_tiles : nullptr;
    for (uint32_t t = threadIdx.x; t < A.n_tiles; t += blockDim.x) {
      const unsigned c = hist[t];
      if (mine) mine[t] = c;
      if (c) atomicAdd(&A.tile_count[t], c);
    }
  }
}

// single-CTA exclusive scan of refs and units per tile
__global__ void __launch_bounds__(1024) k_scan_tiles(RasterArgs A) {
  if (A.ctr->skip_raster) return;
  __shared__ unsigned long long wsum_r[32], wsum_u[32];
  __shared__ unsigned long long carry_r, carry_u;
  if (threadIdx.x == 0) { carry_r = 0; carry_u = 0; }
  __syncthreads();
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (uint32_t base = 0; base < A.n_tiles; base += blockDim.x) {
    const uint32_t t = base + threadIdx.x;
    const unsigned long long c = t < A.n_tiles ? A.tile_count[t] : 0ull;
    const unsigned long long u = (c + A.unit_refs - 1) / A.unit_refs;
    unsigned long long ir = c, iu = u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long yr = __shfl_up_sync(0xffffffffu, ir, o), yu = __shfl_up_sync(0xffffffffu, iu, o);
      if ((int)lane >= o) { ir += yr; iu += yu; }
    }
    if (lane == 31) { wsum_r[wid] = ir; wsum_u[wid] = iu; }
    __syncthreads();
    if (wid == 0) {
      unsigned long long sr = lane < (blockDim.x >> 5) ? wsum_r[lane] : 0ull;
      unsigned long long su = lane < (blockDim.x >> 5) ? wsum_u[lane] : 0ull;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long yr = __shfl_up_sync(0xffffffffu, sr, o), yu = __shfl_up_sync(0xffffffffu, su, o);
        if ((int)lane >= o) { sr += yr; su += yu; }
      }
      wsum_r[lane] = sr;
      wsum_u[lane] = su;
    }
    __syncthreads();
    const unsigned long long pr = (wid ? wsum_r[wid - 1] : 0ull) + ir - c + carry_r;
    const unsigned long long pu = (wid ? wsum_u[wid - 1] : 0ull) + iu - u + carry_u;
    if (t < A.n_tiles) {
      A.tile_off[t] = pr;
      A.tile_cursor[t] = pr;
      A.unit_off[t] = pu;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) {
      carry_r = pr + c;
      carry_u = pu + u;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    A.ctr->tile_refs = carry_r;
    A.ctr->units = carry_u;
    A.ctr->unit_cursor = 0;
  }
}

// Multi-block version of k_scan_tiles for the many bins of a multi-scene accumulation:
// per-CTA sums of refs and units, one scan of the CTA sums, then each CTA scans its own
// chunk from its offset.  part holds 2 values per CTA (refs, units).
__device__ __forceinline__ void tile_counts(const RasterArgs& A, uint32_t t, unsigned long long& c,
                                            unsigned long long& u) {
  c = t < A.n_tiles ? A.tile_count[t] : 0ull;
  u = (c + A.unit_refs - 1) / A.unit_refs;
}

// inclusive block scan of (r, u) over 1024 threads; returns the block totals in tr, tu
__device__ __forceinline__ void block_scan2(unsigned long long& r, unsigned long long& u, unsigned long long& tr,
                                            unsigned long long& tu) {
  __shared__ unsigned long long wr[32], wu[32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long yr = __shfl_up_sync(0xffffffffu, r, o), yu = __shfl_up_sync(0xffffffffu, u, o);
    if ((int)lane >= o) { r += yr; u += yu; }
  }
  if (lane == 31) { wr[wid] = r; wu[wid] = u; }
  __syncthreads();
  if (wid == 0) {
    unsigned long long sr = lane < (blockDim.x >> 5) ? wr[lane] : 0ull;
    unsigned long long su = lane < (blockDim.x >> 5) ? wu[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long yr = __shfl_up_sync(0xffffffffu, sr, o), yu = __shfl_up_sync(0xffffffffu, su, o);
      if ((int)lane >= o) { sr += yr; su += yu; }
    }
    wr[lane] = sr;
    wu[lane] = su;
  }
  __syncthreads();
  if (wid) { r += wr[wid - 1]; u += wu[wid - 1]; }
  tr = wr[(blockDim.x >> 5) - 1];
  tu = wu[(blockDim.x >> 5) - 1];
  __syncthreads();
}

__global__ void __launch_bounds__(1024) k_tiles_partial(RasterArgs A, unsigned long long* part) {
  if (A.ctr->skip_raster) return;
  const uint32_t b0 = blockIdx.x * (uint32_t)TILE_SCAN_CHUNK;
  unsigned long long r = 0, u = 0;
  for (uint32_t k = threadIdx.x; k < (uint32_t)TILE_SCAN_CHUNK; k += blockDim.x) {
    unsigned long long c, v;
    tile_counts(A, b0 + k, c, v);
    r += c;
    u += v;
  }
  unsigned long long tr, tu;
  block_scan2(r, u, tr, tu);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = tr; part[2 * blockIdx.x + 1] = tu; }
}

__global__ void __launch_bounds__(1024) k_tiles_scan_partials(RasterArgs A, unsigned long long* part, uint32_t n_part) {
  if (A.ctr->skip_raster) return;
  __shared__ unsigned long long carry_r, carry_u;
  if (threadIdx.x == 0) { carry_r = 0; carry_u = 0; }
  __syncthreads();
  for (uint32_t base = 0; base < n_part; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const unsigned long long c = i < n_part ? part[2 * i] : 0ull, v = i < n_part ? part[2 * i + 1] : 0ull;
    unsigned long long r = c, u = v, tr, tu;
    block_scan2(r, u, tr, tu);
    const unsigned long long cr = carry_r, cu = carry_u;
    if (i < n_part) { part[2 * i] = cr + r - c; part[2 * i + 1] = cu + u - v; }
    __syncthreads();
    if (threadIdx.x == 0) { carry_r = cr + tr; carry_u = cu + tu; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    A.ctr->tile_refs = carry_r;
    A.ctr->units = carry_u;
    A.ctr->unit_cursor = 0;
  }
}

__global__ void __launch_bounds__(1024) k_tiles_apply(RasterArgs A, const unsigned long long* part) {
  if (A.ctr->skip_raster) return;
  __shared__ unsigned long long carry_r, carry_u;
  if (threadIdx.x == 0) { carry_r = part[2 * blockIdx.x]; carry_u = part[2 * blockIdx.x + 1]; }
  __syncthreads();
  const uint32_t b0 = blockIdx.x * (uint32_t)TILE_SCAN_CHUNK;
  for (uint32_t k = 0; k < (uint32_t)TILE_SCAN_CHUNK; k += blockDim.x) {
    const uint32_t t = b0 + k + threadIdx.x;
    unsigned long long c, v;
    tile_counts(A, t, c, v);
    unsigned long long r = c, u = v, tr, tu;
    block_scan2(r, u, tr, tu);
    const unsigned long long cr = carry_r, cu = carry_u;
    if (t < A.n_tiles) {
      A.tile_off[t] = cr + r - c;
      A.tile_cursor[t] = cr + r - c;
      A.unit_off[t] = cu + u - v;
    }
    __syncthreads();
    if (threadIdx.x == 0) { carry_r = cr + tr; carry_u = cu + tu; }
    __syncthreads();
  }
}

// After each generation of a streaming accumulation: accumulate now only if the ring could
// not take the next generation (one segment per queued ray at most), or nothing follows.
__global__ void k_stream_decide(Counters* ctr, uint32_t gen, uint64_t seg_cap, uint64_t queue_cap, int last) {
  const unsigned long long next = ctr->queue_count[gen + 1];
  const unsigned long long nxt = next < queue_cap ? next : queue_cap;
  const bool go = last || next == 0 || ctr->seg_count + nxt > seg_cap;
  ctr->skip_raster = go ? 0u : 1u;
}

__global__ void k_clear_counts(RasterArgs A) {
  if (A.ctr->skip_raster) return;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < A.n_tiles; t += gridDim.x * blockDim.x) A.tile_count[t] = 0u;
}

// End of one generation of a streaming accumulation: totals, largest demands, and the
// segment ring emptied for the next generation.
__global__ void k_stream_rotate(Counters* ctr, uint64_t seg_cap) {
  if (ctr->skip_raster) return;
  const unsigned long long s = ctr->seg_count, r = ctr->tile_refs;
  ctr->seg_total += s < seg_cap ? s : seg_cap;
  if (s > ctr->seg_max) ctr->seg_max = s;
  ctr->refs_total += r;
  if (r > ctr->refs_max) ctr->refs_max = r;
  ctr->seg_count = 0;
}

__global__ void k_build_units(RasterArgs A) {
  if (A.ctr->skip_raster) return;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < A.n_tiles; t += gridDim.x * blockDim.x) {
    const uint64_t c = A.tile_count[t], off = A.tile_off[t];
    uint64_t u = A.unit_off[t];
    for (uint64_t b = 0; b < c; b += A.unit_refs, ++u) {
      if (u >= A.units_cap) return;
      Unit U;
      U.tile = t;
      U.begin = off + b;
      U.n = (uint32_t)(c - b < A.unit_refs ? c - b : A.unit_refs);
      A.units[u] = U;
    }
  }
}

// Scatter of segment ids into the per-tile lists.  With shared-memory tiles a CTA counts
// its own segments per tile, reserves one range per touched tile with a single global
// atomic, and fills the ranges through shared-memory cursors.
__global__ void __launch_bounds__(SCATTER_THREADS) k_bin_scatter(RasterArgs A, int smem_tiles) {
  if (A.ctr->skip_raster) return;
  extern __shared__ unsigned cur[];  // slots are < refs_cap < 2^32
  const uint64_t n = n_segments(A);
  if (smem_tiles) {
    if (A.cta_hist) {  // this CTA's counts, left by k_bin_count with the same launch shape
      const uint32_t* mine = A.cta_hist + (uint64_t)blockIdx.x * A.n_tiles;
      for (uint32_t t = threadIdx.x; t < A.n_tiles; t += blockDim.x) cur[t] = mine[t];
    } else {
      for (uint32_t t = threadIdx.x; t < A.n_tiles; t += blockDim.x) cur[t] = 0;
      __syncthreads();
      for_each_pair_dense(A, n, [&](uint64_t, uint32_t tile) { atomicAdd(&cur[tile], 1u); });
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < A.n_tiles; t += blockDim.x) {
      const unsigned c = cur[t];
      cur[t] = c ? (unsigned)atomicAdd(&A.tile_cursor[t], (unsigned long long)c) : 0u;
    }
    __syncthreads();
    for_each_pair_dense(A, n, [&](uint64_t i, uint32_t tile) {
      const unsigned slot = atomicAdd(&cur[tile], 1u);
      if (slot < A.refs_cap) A.refs[slot] = (uint32_t)i;
    });
    return;
  }
  for_each_pair_dense(A, n, [&](uint64_t i, uint32_t tile) {
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, tile);
    const int leader = __ffs(grp) - 1;
    unsigned long long base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(&A.tile_cursor[tile], (unsigned long long)__popc(grp));
    base = __shfl_sync(grp, base, leader);
    const unsigned long long slot = base + __popc(grp & lanemask_lt());
    if (slot < A.refs_cap) A.refs[slot] = (uint32_t)i;
  });
}

// ------------------------------------------------------------------ tile raster
constexpr int TILE_PX = TILE * TILE;  // cells per channel plane

// Layout of a unit's shared-memory tile: x-major units index cells [row][col] and their
// 32 lanes own 32 columns; y-major units index [col][row] and their lanes own 32 rows.
// Either way one warp's 32 accesses fall in 32 distinct banks.
//
// Fixed-point sums use exact split accumulation in native 32-bit shared atomics: a
// contribution |q| < 2^34 (a colour term below 4) is split as q = b * 2^17 + c with an
// unsigned 17-bit c and a signed b (|b| <= 2^17).  A unit holds at most SPLIT_UNIT_REFS =
// 16384 segments and a segment adds at most once to a pixel, so both plane sums stay within
// 2^31 and B * 2^17 + C is exact.  (Sixteen times fewer units than 1024-segment units with
// a 21-bit split: each unit ends with a flush of its 32 KB tile by global atomics.)  A
// segment with a larger term (up to the clamp, 2^52) skips the tile and adds its 64-bit
// terms to the image with global atomics, which is just as exact.
constexpr int SPLIT_BITS = 17;   // c = q mod 2^17
constexpr int SPLIT_LIMIT = 34;  // |q| < 2^34 takes the split planes
static_assert((1ll << (SPLIT_LIMIT - SPLIT_BITS)) * SPLIT_UNIT_REFS <= (1ll << 31) &&
                  (1ll << SPLIT_BITS) * SPLIT_UNIT_REFS <= (1ll << 31), "split plane sums must fit 32 bits");
enum RasterMode { RM_FIXED_SPLIT = 0, RM_FIXED_MINMAX = 1, RM_F32 = 2 };

template <int MODE>
struct RasterSmem {
  static constexpr int acc_words = MODE == RM_F32 ? 4 * TILE_PX : 8 * TILE_PX;
  static constexpr int stage_words = 8 * 32 * 12;  // 8 warps x 32 staged segments x 48 B
  static constexpr int owner_words = 8 * 32 * 32 / 4;  // 8 warps x 1024 (segment, column) pairs, 1 B each
  static constexpr int pref_words = 8 * 33;
  static constexpr int bytes = (acc_words + stage_words + owner_words + pref_words) * 4;
};

// one staged segment: raster setup restricted to the unit's tile and the per-channel
// source terms, 48 B
constexpr int SPAN_BIG = 1 << 30;  // FIXED_SPLIT: terms too large for the split planes
struct __align__(16) Staged {
  float ua, va, slope;
  int span;             // first tile-local major-axis pixel | count << 16 | SPAN_BIG
  unsigned q[8];        // FIXED_SPLIT: (c, b) per channel, or 4 x int64 with SPAN_BIG;
                        // FIXED_MINMAX: 4 x int64; F32: 4 x float
};

template <int MODE>
__global__ void __launch_bounds__(256, 4) k_raster(RasterArgs A) {
  if (A.ctr->skip_raster) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned* acc32 = reinterpret_cast<unsigned*>(smem_raw);
  long long* acc64 = reinterpret_cast<long long*>(smem_raw);
  float* accf = reinterpret_cast<float*>(smem_raw);
  Staged* stage_all = reinterpret_cast<Staged*>(smem_raw + RasterSmem<MODE>::acc_words * 4);
  uint8_t* owner_all = reinterpret_cast<uint8_t*>(stage_all + 8 * 32);
  int* pref_all = reinterpret_cast<int*>(owner_all + 8 * 1024);
  __shared__ unsigned long long s_unit, s_pixels;
  if (threadIdx.x == 0) s_pixels = 0;
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  Staged* stage = stage_all + warp * 32;
  uint8_t* owner = owner_all + warp * 1024;
  int* pref = pref_all + warp * 33;
  const BlendDev& B = A.blend;
  unsigned long long my_pixels = 0;
  unsigned long long n_units = A.ctr->units;
  if (n_units > A.units_cap) n_units = A.units_cap;
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(&A.ctr->unit_cursor, 1ull);
    __syncthreads();
    const unsigned long long u = s_unit;
    if (u >= n_units) break;
    const Unit U = A.units[u];
    const CanvasLoc C = canvas_of_bin(A, U.tile);
    const uint32_t lbin = (uint32_t)(U.tile - C.bin_base);
    const uint32_t tile = lbin >> 1;
    const bool xmajor = (lbin & 1u) == 0;
    const uint32_t tx = tile % C.ntx, ty = tile / C.ntx;
    const int tm = xmajor ? (int)tx : (int)ty, tn = xmajor ? (int)ty : (int)tx;
    const int nmin = (int)(xmajor ? C.H : C.W);
    if (MODE == RM_FIXED_SPLIT) {
      uint4* z = reinterpret_cast<uint4*>(acc32);
      for (int k = threadIdx.x; k < RasterSmem<MODE>::acc_words / 4; k += blockDim.x) z[k] = make_uint4(0, 0, 0, 0);
    } else if (MODE == RM_FIXED_MINMAX) {
      for (int k = threadIdx.x; k < 4 * TILE_PX; k += blockDim.x) acc64[k] = ident64(B.op[k / TILE_PX]);
    } else {
      for (int k = threadIdx.x; k < 4 * TILE_PX; k += blockDim.x) accf[k] = ident32(B.op[k / TILE_PX]);
    }
    __syncthreads();
    const uint64_t end = min(U.begin + U.n, A.refs_cap);
    for (uint64_t base = U.begin + (uint64_t)warp * 32; base < end; base += (uint64_t)nwarps * 32) {
      // lane-parallel: fetch 32 segments, set them up and clip them to this tile
      const uint64_t r = base + lane;
      Staged st;
      int cnt = 0;
      if (r < end) {
        const uint32_t si = A.refs[r];
        const float4* sp = reinterpret_cast<const float4*>(A.segs + si);
        const float4 g = __ldg(sp), cc = __ldg(sp + 1);
        lg_segment sg;
        sg.x0 = g.x; sg.y0 = g.y; sg.x1 = g.z; sg.y1 = g.w;
        sg.color[0] = cc.x; sg.color[1] = cc.y; sg.color[2] = cc.z; sg.color[3] = cc.w;
        RSetup R;
        if (raster_setup(sg, C.W, C.H, R)) {
          const int c0 = max(R.lo - tm * TILE, 0), c1 = min(R.hi - tm * TILE, TILE);
          cnt = max(c1 - c0, 0);
          st.ua = R.ua; st.va = R.va; st.slope = R.slope;
          st.span = c0 | (cnt << 16);
          long long qv[4];
          bool big = false;
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const float v = contribution(B, ch, sg.color);
            if (MODE == RM_FIXED_SPLIT) {
              long long q = to_fixed(v);
              if (B.op[ch] == LG_BO_REVERSE_SUBTRACT) q = -q;
              qv[ch] = q;
              big = big || q >= (1ll << SPLIT_LIMIT) || q < -(1ll << SPLIT_LIMIT);
            } else if (MODE == RM_FIXED_MINMAX) {
              long long q = to_fixed(v);
              if (B.op[ch] == LG_BO_REVERSE_SUBTRACT) q = -q;
              st.q[2 * ch] = (unsigned)(q & 0xffffffffll);
              st.q[2 * ch + 1] = (unsigned)(q >> 32);
            } else {
              st.q[ch] = __float_as_uint(B.op[ch] == LG_BO_REVERSE_SUBTRACT ? -v : v);
            }
          }
          if (MODE == RM_FIXED_SPLIT) {
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) {
              const long long q = qv[ch];
              st.q[2 * ch] = big ? (unsigned)(q & 0xffffffffll) : (unsigned)(q & ((1ll << SPLIT_BITS) - 1));
              st.q[2 * ch + 1] = big ? (unsigned)(q >> 32) : (unsigned)(int)(q >> SPLIT_BITS);
            }
            if (big) st.span |= SPAN_BIG;
          }
        }
      }
      stage[lane] = st;
      // pack every (segment, pixel column) pair of the batch densely over the lanes
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += y;
      }
      pref[lane] = incl - cnt;
      for (int k = 0; k < cnt; ++k) owner[incl - cnt + k] = (uint8_t)lane;
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      __syncwarp();
      for (int pi = (int)lane; pi < total; pi += 32) {
        const int k = owner[pi];
        const Staged& sk = stage[k];
        const int i = tm * TILE + (sk.span & 0xffff) + (pi - pref[k]);  // SPAN_BIG is above bit 16
        RSetup R;
        R.ua = sk.ua; R.va = sk.va; R.slope = sk.slope;
        const int j = raster_minor(R, i);
        const int jl = j - tn * TILE;
        if (jl < 0 || jl >= TILE || j >= nmin) continue;
        const int cell = jl * TILE + (i - tm * TILE);  // [row][col] for x-major, [col][row] for y-major
        if (MODE == RM_FIXED_SPLIT) {
          const uint4 q0 = *reinterpret_cast<const uint4*>(&sk.q[0]);
          const uint4 q1 = *reinterpret_cast<const uint4*>(&sk.q[4]);
          const unsigned qs[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
          if (sk.span & SPAN_BIG) {  // rare: the 64-bit terms straight into the image
            const uint32_t x = xmajor ? (uint32_t)i : (uint32_t)j, y = xmajor ? (uint32_t)j : (uint32_t)i;
            unsigned long long* g = reinterpret_cast<unsigned long long*>(A.accum) + (C.px_base + (uint64_t)y * C.W + x) * 4;
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) {
              const unsigned long long q = ((unsigned long long)qs[2 * ch + 1] << 32) | qs[2 * ch];
              if (q) atomicAdd(g + ch, q);
            }
          } else {
#pragma unroll
            for (int w = 0; w < 8; ++w)
              if (qs[w]) atomicAdd(acc32 + w * TILE_PX + cell, qs[w]);
          }
        } else if (MODE == RM_FIXED_MINMAX) {
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const long long q = (long long)(((unsigned long long)sk.q[2 * ch + 1] << 32) | sk.q[2 * ch]);
            long long* p = acc64 + ch * TILE_PX + cell;
            const int op = B.op[ch];
            if (op == LG_BO_MIN) atomicMin(p, q);
            else if (op == LG_BO_MAX) atomicMax(p, q);
            else atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)q);
          }
        } else {
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const float v = __uint_as_float(sk.q[ch]);
            float* pf = accf + ch * TILE_PX + cell;
            const int op = B.op[ch];
            if (op == LG_BO_ADD || op == LG_BO_REVERSE_SUBTRACT) atomicAdd(pf, v);
            else {
              float o = *pf;
              while (op == LG_BO_MIN ? v < o : v > o) {
                const float w = __int_as_float(atomicCAS(reinterpret_cast<int*>(pf), __float_as_int(o), __float_as_int(v)));
                if (w == o) break;
                o = w;
              }
            }
          }
        }
        ++my_pixels;
      }
      __syncwarp();
    }
    __syncthreads();
    // flush: one global atomic per touched pixel channel
    for (int k = threadIdx.x; k < TILE_PX; k += blockDim.x) {
      const int row = k / TILE, col = k % TILE;
      const uint32_t x = tx * TILE + col, y = ty * TILE + row;
      if (x >= C.W || y >= C.H) continue;
      const uint64_t px = (C.px_base + (uint64_t)y * C.W + x) * 4;
      const int cell = xmajor ? row * TILE + col : col * TILE + row;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const int op = B.op[ch];
        if (MODE == RM_FIXED_SPLIT) {
          const unsigned* base = acc32 + 2 * ch * TILE_PX + cell;
          const long long q = (long long)(int)base[TILE_PX] * (1ll << SPLIT_BITS) + (long long)base[0];
          if (q == 0) continue;
          atomicAdd(reinterpret_cast<unsigned long long*>(A.accum) + px + ch, (unsigned long long)q);
        } else if (MODE == RM_FIXED_MINMAX) {
          const long long v = acc64[ch * TILE_PX + cell];
          if (v == ident64(op)) continue;
          long long* g = reinterpret_cast<long long*>(A.accum) + px + ch;
          if (op == LG_BO_MIN) atomicMin(g, v);
          else if (op == LG_BO_MAX) atomicMax(g, v);
          else atomicAdd(reinterpret_cast<unsigned long long*>(g), (unsigned long long)v);
        } else {
          const float v = accf[ch * TILE_PX + cell];
          if (v == ident32(op)) continue;
          float* g = reinterpret_cast<float*>(A.accum) + px + ch;
          if (op == LG_BO_MIN || op == LG_BO_MAX) {
            float o = *g;
            while (op == LG_BO_MIN ? v < o : v > o) {
              const float w = __int_as_float(atomicCAS(reinterpret_cast<int*>(g), __float_as_int(o), __float_as_int(v)));
              if (w == o) break;
              o = w;
            }
          } else {
            atomicAdd(g, v);
          }
        }
      }
    }
    __syncthreads();
  }
  atomicAdd(&s_pixels, my_pixels);
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(&A.ctr->pixels, s_pixels);
}

// One warp per unit with a private tile: lane L owns pixel column L of the tile (x-major
// units) or pixel row L (y-major units), and every segment of an x-major unit touches a
// column at most once, so no two lanes or warps ever update the same accumulator and
// plain 64-bit read-modify-write replaces atomics.  Units can therefore hold any number
// of segments (fewer flushes); occupancy is bounded by the 32 KB tile per warp.
template <int MODE>
__global__ void __launch_bounds__(32) k_raster_warp(RasterArgs A) {
  if (A.ctr->skip_raster) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long* acc64 = reinterpret_cast<long long*>(smem_raw);      // [ch][minor][lane]
  float* accf = reinterpret_cast<float*>(smem_raw);
  struct __align__(16) St {
    float ua, va, slope;
    int lohi;
    long long q[4];
  };
  St* stage = reinterpret_cast<St*>(smem_raw + 4 * TILE_PX * 8);
  const unsigned lane = lane_id();
  const BlendDev& B = A.blend;
  unsigned long long my_pixels = 0;
  unsigned long long n_units = A.ctr->units;
  if (n_units > A.units_cap) n_units = A.units_cap;
  for (;;) {
    unsigned long long u = 0;
    if (lane == 0) u = atomicAdd(&A.ctr->unit_cursor, 1ull);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= n_units) break;
    const Unit U = A.units[u];
    const CanvasLoc C = canvas_of_bin(A, U.tile);
    const uint32_t lbin = (uint32_t)(U.tile - C.bin_base);
    const uint32_t tile = lbin >> 1;
    const bool xmajor = (lbin & 1u) == 0;
    const uint32_t tx = tile % C.ntx, ty = tile / C.ntx;
    const int tm = xmajor ? (int)tx : (int)ty, tn = xmajor ? (int)ty : (int)tx;
    const int nmin = (int)(xmajor ? C.H : C.W);
    const int i = tm * TILE + (int)lane;
    for (int k = (int)lane; k < 4 * TILE_PX; k += 32) {
      if (MODE == RM_F32) accf[k] = ident32(B.op[k / TILE_PX]);
      else acc64[k] = ident64(B.op[k / TILE_PX]);
    }
    __syncwarp();
    const uint64_t end = min(U.begin + U.n, A.refs_cap);
    for (uint64_t base = U.begin; base < end; base += 32) {
      const uint64_t r = base + lane;
      St st;
      st.lohi = -1;
      if (r < end) {
        const uint32_t si = A.refs[r];
        const float4* sp = reinterpret_cast<const float4*>(A.segs + si);
        const float4 g = __ldg(sp), cc = __ldg(sp + 1);
        lg_segment sg;
        sg.x0 = g.x; sg.y0 = g.y; sg.x1 = g.z; sg.y1 = g.w;
        sg.color[0] = cc.x; sg.color[1] = cc.y; sg.color[2] = cc.z; sg.color[3] = cc.w;
        RSetup R;
        if (raster_setup(sg, C.W, C.H, R)) {
          st.ua = R.ua; st.va = R.va; st.slope = R.slope;
          st.lohi = R.lo | (R.hi << 16);
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const float v = contribution(B, ch, sg.color);
            if (MODE == RM_F32) {
              st.q[ch] = (long long)__float_as_uint(B.op[ch] == LG_BO_REVERSE_SUBTRACT ? -v : v);
            } else {
              const long long q = to_fixed(v);
              st.q[ch] = B.op[ch] == LG_BO_REVERSE_SUBTRACT ? -q : q;
            }
          }
        }
      }
      stage[lane] = st;
      __syncwarp();
      const int n = (int)min((uint64_t)32, end - base);
      for (int k = 0; k < n; ++k) {
        const int lohi = stage[k].lohi;
        if (lohi < 0 || i < (lohi & 0xffff) || i >= (lohi >> 16)) continue;
        RSetup R;
        R.ua = stage[k].ua; R.va = stage[k].va; R.slope = stage[k].slope;
        const int j = raster_minor(R, i);
        const int jl = j - tn * TILE;
        if (jl < 0 || jl >= TILE || j >= nmin) continue;
        const int cell = jl * TILE + (int)lane;
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          const int op = B.op[ch];
          const long long q = stage[k].q[ch];
          if (MODE == RM_F32) {
            float& a = accf[ch * TILE_PX + cell];
            const float v = __uint_as_float((unsigned)q);
            a = op == LG_BO_MIN ? fminf(a, v) : op == LG_BO_MAX ? fmaxf(a, v) : a + v;
          } else {
            long long& a = acc64[ch * TILE_PX + cell];
            a = op == LG_BO_MIN ? min(a, q) : op == LG_BO_MAX ? max(a, q) : a + q;
          }
        }
        ++my_pixels;
      }
      __syncwarp();
    }
    // flush the private tile: one global atomic per touched pixel channel
    for (int k = (int)lane; k < TILE_PX; k += 32) {
      const int jl = k / TILE, c = k % TILE;  // cell k = [minor][lane]
      const uint32_t x = xmajor ? tx * TILE + c : tx * TILE + jl;
      const uint32_t y = xmajor ? ty * TILE + jl : ty * TILE + c;
      if (x >= C.W || y >= C.H) continue;
      const uint64_t px = (C.px_base + (uint64_t)y * C.W + x) * 4;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const int op = B.op[ch];
        if (MODE == RM_F32) {
          const float v = accf[ch * TILE_PX + k];
          if (v == ident32(op)) continue;
          float* g = reinterpret_cast<float*>(A.accum) + px + ch;
          if (op == LG_BO_MIN || op == LG_BO_MAX) {
            float o = *g;
            while (op == LG_BO_MIN ? v < o : v > o) {
              const float w = __int_as_float(atomicCAS(reinterpret_cast<int*>(g), __float_as_int(o), __float_as_int(v)));
              if (w == o) break;
              o = w;
            }
          } else {
            atomicAdd(g, v);
          }
        } else {
          const long long v = acc64[ch * TILE_PX + k];
          if (v == ident64(op)) continue;
          long long* g = reinterpret_cast<long long*>(A.accum) + px + ch;
          if (op == LG_BO_MIN) atomicMin(g, v);
          else if (op == LG_BO_MAX) atomicMax(g, v);
          else atomicAdd(reinterpret_cast<unsigned long long*>(g), (unsigned long long)v);
        }
      }
    }
    __syncwarp();
  }
  if (my_pixels) atomicAdd(&A.ctr->pixels, my_pixels);
}

template __global__ void k_raster_warp<RM_FIXED_SPLIT>(RasterArgs A);
template __global__ void k_raster_warp<RM_F32>(RasterArgs A);
int raster_warp_smem_bytes() { return 4 * TILE_PX * 8 + 32 * 48; }

// ------------------------------------------------------------------ string-mod lines
// A few thousand lines per frame: one warp per line, one lane per major-axis pixel, and
// each pixel's terms go straight into the image with global atomics (int64 sums and
// min / max are order-independent, so the image stays bit-reproducible in fixed point).
template <bool FIXED>
__global__ void __launch_bounds__(256) k_raster_chords(RasterArgs A, const lg_chord* chords, uint64_t n) {
  const unsigned lane = lane_id();
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const BlendDev& B = A.blend;
  const float sc = (float)A.H * 0.5f, cx = (float)A.W * 0.5f;
  unsigned long long my_pixels = 0;
  for (uint64_t k = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; k < n; k += nw) {
    const lg_chord c = chords[k];
    lg_segment sg;
    sg.x0 = c.x0; sg.y0 = c.y0; sg.x1 = c.x1; sg.y1 = c.y1;
    RSetup R;
    if (!raster_setup(sg, A.W, A.H, R)) continue;
    // the vertices' major coordinates before raster_setup orders them
    const float U0 = R.xmajor ? __fmaf_rn(c.x0, sc, cx) : __fmaf_rn(-c.y0, sc, sc);
    const float dU = __fsub_rn(R.xmajor ? __fmaf_rn(c.x1, sc, cx) : __fmaf_rn(-c.y1, sc, sc), U0);
    float dc[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) dc[ch] = __fsub_rn(c.color1[ch], c.color0[ch]);
    const int nmin = (int)(R.xmajor ? A.H : A.W);
    for (int i = R.lo + (int)lane; i < R.hi; i += 32) {
      const int j = raster_minor(R, i);
      if (j < 0 || j >= nmin) continue;
      float f = __fdiv_rn(__fsub_rn(__fadd_rn((float)i, 0.5f), U0), dU);
      f = fminf(fmaxf(f, 0.0f), 1.0f);
      float src[4];
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) src[ch] = __fmaf_rn(f, dc[ch], c.color0[ch]);
      const uint32_t x = R.xmajor ? (uint32_t)i : (uint32_t)j, y = R.xmajor ? (uint32_t)j : (uint32_t)i;
      const uint64_t px = ((uint64_t)y * A.W + x) * 4;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const int op = B.op[ch];
        const float v = contribution(B, ch, src);
        if (FIXED) {
          long long q = to_fixed(v);
          long long* g = reinterpret_cast<long long*>(A.accum) + px + ch;
          if (op == LG_BO_MIN) atomicMin(g, q);
          else if (op == LG_BO_MAX) atomicMax(g, q);
          else {
            if (op == LG_BO_REVERSE_SUBTRACT) q = -q;
            if (q) atomicAdd(reinterpret_cast<unsigned long long*>(g), (unsigned long long)q);
          }
        } else {
          float* g = reinterpret_cast<float*>(A.accum) + px + ch;
          if (op == LG_BO_MIN || op == LG_BO_MAX) {
            float o = *g;
            while (op == LG_BO_MIN ? v < o : v > o) {
              const float w = __int_as_float(atomicCAS(reinterpret_cast<int*>(g), __float_as_int(o), __float_as_int(v)));
              if (w == o) break;
              o = w;
            }
          } else {
            atomicAdd(g, op == LG_BO_REVERSE_SUBTRACT ? -v : v);
          }
        }
      }
      ++my_pixels;
    }
  }
  if (my_pixels) atomicAdd(&A.ctr->pixels, my_pixels);
}

template __global__ void k_raster_chords<true>(RasterArgs A, const lg_chord* chords, uint64_t n);
template __global__ void k_raster_chords<false>(RasterArgs A, const lg_chord* chords, uint64_t n);

template __global__ void k_raster<RM_FIXED_SPLIT>(RasterArgs A);
template __global__ void k_raster<RM_FIXED_MINMAX>(RasterArgs A);
template __global__ void k_raster<RM_F32>(RasterArgs A);

int raster_smem_bytes(int mode) {
  return mode == RM_FIXED_SPLIT ? RasterSmem<RM_FIXED_SPLIT>::bytes
                                : mode == RM_FIXED_MINMAX ? RasterSmem<RM_FIXED_MINMAX>::bytes : RasterSmem<RM_F32>::bytes;
}

// ------------------------------------------------------------------ resolve
__device__ __forceinline__ float4 load_px(const void* acc, int fixed, uint64_t i) {
  if (fixed) {
    const longlong4_32a v = reinterpret_cast<const longlong4_32a*>(acc)[i];
    const float s = 2.3283064365386963e-10f;  // 2^-32
    return make_float4(__fmul_rn(__ll2float_rn(v.x), s), __fmul_rn(__ll2float_rn(v.y), s),
                       __fmul_rn(__ll2float_rn(v.z), s), __fmul_rn(__ll2float_rn(v.w), s));
  }
  return reinterpret_cast<const float4*>(acc)[i];
}

__global__ void k_resolve_f16(const void* acc, int fixed, uint32_t W, uint32_t H, uint16_t* dst, size_t pitch) {
  const uint64_t n = (uint64_t)W * H;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 f = load_px(acc, fixed, i);
    const uint32_t y = (uint32_t)(i / W), x = (uint32_t)(i % W);
    ushort4 h;
    h.x = __half_as_ushort(__float2half_rn(f.x));
    h.y = __half_as_ushort(__float2half_rn(f.y));
    h.z = __half_as_ushort(__float2half_rn(f.z));
    h.w = __half_as_ushort(__float2half_rn(f.w));
    *reinterpret_cast<ushort4*>(reinterpret_cast<char*>(dst) + y * pitch + (uint64_t)x * 8) = h;
  }
}

// renderer.rs:313-328: u8 = (f16 value ^ (1 / 2.2) * 255) as u8 (saturating, truncating)
__global__ void k_resolve_rgba8(const void* acc, int fixed, uint32_t W, uint32_t H, uint8_t* dst, size_t pitch) {
  const uint64_t n = (uint64_t)W * H;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 f = load_px(acc, fixed, i);
    const uint32_t y = (uint32_t)(i / W), x = (uint32_t)(i % W);
    const float c[4] = {f.x, f.y, f.z, f.w};
    uchar4 o;
    unsigned char* po = &o.x;
    for (int k = 0; k < 4; ++k) {
      const float h = __half2float(__float2half_rn(c[k]));
      const float g = __fmul_rn(powf(h, __fdiv_rn(1.0f, 2.2f)), 255.0f);
      po[k] = (g != g || g <= 0.0f) ? 0 : (g >= 255.0f ? 255 : (unsigned char)g);
    }
    *reinterpret_cast<uchar4*>(dst + y * pitch + (uint64_t)x * 4) = o;
  }
}

}  // namespace lgd
