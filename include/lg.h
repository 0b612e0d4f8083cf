/*
 * lg.h — C ABI of the GB300 trace-and-accumulate library (liblightgarden_cuda.so).
 *
 * This is the drop-in boundary for light_garden's per-frame hot path:
 *
 *   Tracer::trace_all            src/light_garden/tracer.rs:276-358   -> lg_trace
 *   Tracer::trace                src/light_garden/tracer.rs:360-493   -> (inside lg_trace)
 *   {Point,Spot,Directional}Light::set_num_rays
 *                                src/light_garden/light.rs:103-115,163-174,225-249 -> (inside lg_trace)
 *   StringMod::draw              src/light_garden/string_mod.rs:33-158 -> lg_params.string_mod overlay
 *   SubRenderPass::update_vertex_buffer
 *                                src/sub_render_pass.rs:188-203       -> segments stay on the device
 *   Renderer::render_to_texture  src/renderer.rs:164-188 (LineList, blend src/light_garden/mod.rs:57-73)
 *                                                                      -> lg_accumulate
 *   Renderer::render_texture     src/renderer.rs:330-418, src/render_to_texture.wgsl:17-28
 *                                                                      -> lg_resolve_f16
 *   Tracer::{push_object, push_light, clear, ...} src/light_garden/tracer.rs:48-116,
 *   pub fields max_bounce / cutoff_color       src/light_garden/tracer.rs:9-11
 *                                                                      -> lg_scene_upload
 *
 * The reference has no FFI; its Rust `Tracer` owns Vec<Object>/Vec<Light> and returns a
 * Vec<(P2, Color)>.  Here the caller owns the scene description (flat arrays of the
 * structs below), the library copies it to the device, owns every device buffer, and the
 * caller owns every output buffer.  A context is used by one host thread at a time;
 * several contexts may share a device.  Every entry point returns an lg_status and never
 * aborts the process; lg_last_error() describes the last failure of a context.
 *
 * World coordinates follow the reference: the canvas is the rectangle
 * [-aspect, aspect] x [-1, 1] with aspect = width / height (src/sub_render_pass.rs:146-158).
 * Geometry is FP64 (collision2d's Float = f64), colours are FP32 RGBA (light.rs:7).
 */
#ifndef LIGHT_GARDEN_GB300_LG_H
#define LIGHT_GARDEN_GB300_LG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: lg_device_opts gained culling and grid_density, lg_trace_stats bound_tests and
 * object_tests (both structs grew).
 * 3: lg_device_opts gained wait_polls; lg_params.precision (was padding), ray_stride and
 *    ray_offset (lg_params grew); lg_trace_stats scan_ms, solve_ms, bounce_ms (grew).
 * 4: lg_string_mod gained the curve parameters and the modulo-colour table (lg_params
 *    grew); string-mod lines are lg_chord records (lg_chords_download), no longer
 *    segments; lg_device_opts.scan_pairs (was padding); LG_PATH_ILL_CONDITIONED split from
 *    LG_PATH_NEAR_DEGENERATE, lg_trace_stats.ill_conditioned (grew).
 * 5: lg_string_mod.nested (lg_string_mod and lg_params grew). */
#define LG_ABI_VERSION 5

typedef enum lg_status {
  LG_OK = 0,
  LG_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad index, out-of-range parameter */
  LG_ERR_UNSUPPORTED = 2,      /* a shape kind, blend mode or option this path does not implement */
  LG_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed */
  LG_ERR_CUDA = 4,             /* a CUDA runtime call failed (message in lg_last_error) */
  LG_ERR_NO_SCENE = 5,         /* lg_trace/lg_render before lg_scene_upload */
  LG_ERR_TRUNCATED = 6,        /* caller buffer too small; *n_out holds the size needed */
  LG_ERR_TIMEOUT = 7,          /* a bounded device-side wait expired (no hang, no trap) */
  LG_ERR_BUDGET = 8,           /* admission refused: request does not fit the HBM budget */
  LG_ERR_NOT_READY = 9,        /* serving: result not finished yet */
  LG_ERR_NOT_FOUND = 10        /* serving: unknown request id */
} lg_status;

/* ---- geometry nodes: the collision2d `Geo` variants on the path ----------------------- */
enum lg_geo_kind {
  LG_GEO_CIRCLE = 0,  /* GeoCircle  { origin, radius }                              */
  LG_GEO_RECT = 1,    /* GeoRect    { origin (centre), rotation, width, height }    */
  LG_GEO_SEGMENT = 2, /* GeoLineSegment a -> b (straight mirror)                    */
  LG_GEO_CUBIC = 3,   /* GeoCubicBezier P0..P3 (curved mirror)                      */
  LG_GEO_LOGIC = 4,   /* GeoLogic   { op, a, b, origin, rotation } (CSG)            */
  LG_GEO_POLYGON = 5, /* convex polygon { points } (ConvexPolygon, object.rs:13,34-36) */
  LG_GEO_ELLIPSE = 6, /* Ellipse { origin, a, b, rot } (object.rs:14,37-44)         */
  LG_GEO_VERTICES = 7 /* continuation of a POLYGON's vertex list                   */
};

/* Logic / LogicOp (src/light_garden/mod.rs:366-372: geo_a & geo_b, |, and_not) */
enum lg_logic_op { LG_OP_AND = 0, LG_OP_OR = 1, LG_OP_AND_NOT = 2 };

/* One node of a geometry tree.  Trees are stored as a flat array; LOGIC nodes name their
 * two children by index into the same array.  LOGIC children are expressed in the
 * node's local frame: world = origin + R(rot) * local, R = [[c, -s], [s, c]]. */
typedef struct lg_geo {
  int32_t kind;     /* enum lg_geo_kind */
  int32_t op;       /* LOGIC: enum lg_logic_op */
  int32_t a, b;     /* LOGIC: child node indices.  POLYGON: a = vertex count (3..63),
                       b = index of the VERTICES node holding vertices 4.. (-1: none);
                       VERTICES: b = the next VERTICES node (-1: none) */
  double origin[2]; /* CIRCLE centre | RECT centre | LOGIC / POLYGON origin | ELLIPSE centre */
  double rot[2];    /* RECT / LOGIC / POLYGON / ELLIPSE rotation as (cos, sin); (1, 0) = identity */
  double v[8];      /* CIRCLE: v[0] = radius
                       RECT:   v[0] = width, v[1] = height
                       SEGMENT: (v[0], v[1]) -> (v[2], v[3])
                       CUBIC:  P0 = (v[0], v[1]) ... P3 = (v[6], v[7])
                       POLYGON / VERTICES: up to 4 vertices (x, y), in the node's frame, in
                               order around a convex polygon (either orientation)
                       ELLIPSE: v[0] = a (semi-axis along the rotated x), v[1] = b */
} lg_geo;

/* ---- objects: ObjectE + Option<Material> (src/light_garden/object.rs:7-16,51-55) ------ */
enum lg_object_kind {
  LG_OBJ_STRAIGHT_MIRROR = 0, /* root must be a SEGMENT */
  LG_OBJ_CURVED_MIRROR = 1,   /* root must be a CUBIC   */
  LG_OBJ_CIRCLE = 2,
  LG_OBJ_RECT = 3,
  LG_OBJ_LENS = 4,            /* Logic(And, circle, circle), object.rs:387-415 */
  LG_OBJ_CONVEX_POLYGON = 5,  /* root must be a POLYGON */
  LG_OBJ_ELLIPSE = 6,         /* root must be an ELLIPSE */
  LG_OBJ_GEO = 7              /* any geometry tree (CSG results, object.rs:107-113) */
};

typedef struct lg_object {
  int32_t kind;            /* enum lg_object_kind */
  int32_t geo;             /* index of the root node in the geo array */
  int32_t has_material;    /* 0: material_opt = None -> perfect mirror (tracer.rs:473-481) */
  int32_t _pad;
  double refractive_index; /* Material::refractive_index; default 1.2 (object.rs:441-447) */
} lg_object;

/* ---- lights (src/light_garden/light.rs:10-14) ----------------------------------------- */
enum lg_light_kind { LG_LIGHT_POINT = 0, LG_LIGHT_DIRECTIONAL = 1, LG_LIGHT_SPOT = 2 };

typedef struct lg_light {
  int32_t kind;      /* enum lg_light_kind */
  uint32_t num_rays; /* rays generated per frame (set_num_rays) */
  float color[4];    /* RGBA of every primary ray */
  double origin[2];  /* POINT/SPOT: position.  DIRECTIONAL: segment start a */
  double v[2];       /* SPOT: spot_direction.   DIRECTIONAL: segment end b  */
  double spot_angle; /* SPOT: full opening angle in radians */
} lg_light;

/* ---- blend state (wgpu::BlendComponent, src/light_garden/mod.rs:57-73) --------------- *
 * Only order-independent blends are accepted (dst_factor One with Add / ReverseSubtract,
 * or Min / Max); anything that reads the destination is order-dependent under
 * concurrent accumulation and is rejected with LG_ERR_UNSUPPORTED. */
enum lg_blend_factor {
  LG_BF_ZERO = 0, LG_BF_ONE = 1, LG_BF_SRC = 2, LG_BF_ONE_MINUS_SRC = 3,
  LG_BF_SRC_ALPHA = 4, LG_BF_ONE_MINUS_SRC_ALPHA = 5, LG_BF_DST = 6,
  LG_BF_ONE_MINUS_DST = 7, LG_BF_DST_ALPHA = 8, LG_BF_ONE_MINUS_DST_ALPHA = 9,
  LG_BF_SRC_ALPHA_SATURATED = 10, LG_BF_CONSTANT = 11, LG_BF_ONE_MINUS_CONSTANT = 12
};
enum lg_blend_op { LG_BO_ADD = 0, LG_BO_SUBTRACT = 1, LG_BO_REVERSE_SUBTRACT = 2, LG_BO_MIN = 3, LG_BO_MAX = 4 };

typedef struct lg_blend_component {
  int32_t src_factor, dst_factor, op;
} lg_blend_component;

enum lg_accum_mode {
  LG_ACCUM_FIXED64 = 0, /* signed Q31.32 fixed point in int64: order-independent, bit-reproducible */
  LG_ACCUM_F32 = 1      /* FP32 atomics: faster to reason about, not bit-reproducible */
};

/* ---- string-mod overlay (src/light_garden/string_mod.rs) ------------------------------- */
enum lg_string_mod_mode { LG_SM_ADD = 0, LG_SM_MUL = 1, LG_SM_POW = 2, LG_SM_BASE = 3 };

/* StringMod::init_curve (string_mod.rs:182-188, points init_points 33-85).  With
 * a(n) = turns * n * 2 pi / m:
 *   CIRCLE        (cos a, sin a)
 *   COMPLEX_EXP   c^(u32)(turns * n), c = curve_f[0] + i curve_f[1] (binary powering)
 *   HYPOTROCHOID  r, s, d = curve_u[0..2], k = s - r:
 *                 (k cos a + d cos(a k / r), k sin a - d sin(a k / r)) / (k + d)
 *   LISSAJOUS     a_, b_ = curve_u[0..1], delta = curve_f[0]: (sin(a_ a + delta), sin(b_ a)) */
enum lg_string_mod_curve {
  LG_CURVE_CIRCLE = 0,
  LG_CURVE_COMPLEX_EXP = 1,
  LG_CURVE_HYPOTROCHOID = 2,
  LG_CURVE_LISSAJOUS = 3
};

/* ModRemColor (string_mod.rs:167-172): point n takes `color` when n % modulo == rem.  A
 * point that several entries match takes their mean (f32 sums in table order, then one
 * division by the count); a point that none matches takes lg_string_mod.color
 * (StringMod::get_color, string_mod.rs:124-150). */
typedef struct lg_mod_color {
  uint64_t modulo; /* >= 1 */
  uint64_t rem;
  float color[4];
} lg_mod_color;

/* StringMod::nested (string_mod.rs:14, 87-102, 152-158).  When `nested` is not NULL the
 * lines drawn are the nested mod's, and its points are the crossings of this mod's m lines:
 * for diff = 1 .. m-1, for a = 0 .. m-1, the crossing of line a with line (a + diff) % m,
 * if they cross, in that order (so every crossing appears twice).  Two lines cross when the
 * 2x2 parametric solve of the segments, in FP64 with each operation rounded on its own, has
 * a non-zero determinant and both parameters in [0, 1]; the point is a + t (b - a) on the
 * first.  Nested line k joins crossing k % n and crossing ix(k) % n of the nested mode,
 * with the nested mod's colours; no crossings, no lines.  The nested mod's curve, turns,
 * curve parameters and its own `nested` are not used.  This mod's modulo is then at most
 * LG_STRING_MOD_NESTED_MAX. */
#define LG_STRING_MOD_NESTED_MAX 4096u

typedef struct lg_string_mod {
  uint64_t modulo;  /* number of points m; 0 disables the overlay */
  uint64_t num;
  uint64_t turns;
  uint32_t mode;    /* enum lg_string_mod_mode */
  uint32_t curve;   /* enum lg_string_mod_curve */
  float color[4];   /* StringMod::color */
  double curve_f[2];    /* curve parameters, see lg_string_mod_curve */
  uint64_t curve_u[3];
  uint32_t n_colors;    /* entries of `colors` (StringMod::modulo_colors), 0..4096 */
  uint32_t _pad;
  const lg_mod_color* colors; /* host array, copied by lg_scene_upload (not kept) */
  const struct lg_string_mod* nested; /* NULL, or the mod drawn between this one's line
                                         crossings; copied by lg_scene_upload (not kept) */
} lg_string_mod;

/* ---- trace precision ----------------------------------------------------------------- *
 * EXACT: every hit, membership test and bounce is evaluated in IEEE-754 double with each
 * operation rounded on its own (no fused multiply-add), in the order of the restated
 * collision2d formulas, so the trace equals the FP64 CPU trace of the same formulas bit for
 * bit; an FP32 search only prunes the candidates.  Geometry trees may hold up to 8 levels
 * of Logic nodes.
 * FAST: the hit and the bounce are refined in double-float (~2^-47 relative) on the FP32
 * pipe; decisions within the rounding of the ray's own error bound are flagged
 * LG_PATH_NEAR_DEGENERATE and may differ from an FP64 trace. */
enum lg_precision { LG_PRECISION_EXACT = 0, LG_PRECISION_FAST = 1 };

/* ---- per-scene parameters ------------------------------------------------------------- */
typedef struct lg_params {
  uint32_t max_bounce;          /* Tracer::max_bounce (default 5, GUI 1..=20); here 1..=64 */
  uint32_t width, height;       /* accumulation canvas in pixels */
  float cutoff_color[4];        /* Tracer::cutoff_color (default 0.001) */
  float clear_color[4];         /* render-texture clear; wgpu::Color::BLACK = (0,0,0,1) */
  float blend_constant[4];      /* for LG_BF_CONSTANT */
  lg_blend_component color_blend; /* default One / One / Add */
  lg_blend_component alpha_blend; /* default SrcAlpha / One / Add */
  int32_t accum;                /* enum lg_accum_mode */
  int32_t emit_control_lines;   /* append curved-mirror control polygons (tracer.rs:341-346) */
  int32_t record_paths;         /* also write one lg_path_record per segment (parity tooling) */
  int32_t precision;            /* enum lg_precision of the trace */
  lg_string_mod string_mod;     /* overlay lines (lg_chord), drawn with the same raster */
  uint32_t ray_stride;          /* trace only the primaries i = ray_offset + k * ray_stride of each
                                   light (0 or 1: all), as a sampled frame; the overlays are drawn
                                   only when ray_offset == 0.  One scene only (not batches/serving) */
  uint32_t ray_offset;
} lg_params;

/* Fills *p with the reference defaults (tracer.rs:37-39, mod.rs:57-73). */
void lg_params_default(lg_params* p);

/* ---- outputs -------------------------------------------------------------------------- */
/* One emitted line segment: two (P2, Color) vertices of the reference's line list,
 * positions narrowed to f32 exactly like update_vertex_buffer (sub_render_pass.rs:188-203). */
typedef struct lg_segment {
  float x0, y0, x1, y1;
  float color[4];
} lg_segment;

/* One string-mod line (StringMod::draw_init_points, string_mod.rs:104-122): the two
 * (P2, Color) vertices of the reference's line list with their own colours.  The raster
 * interpolates the colour along the major axis: at the sample of major-axis pixel i,
 * f = clamp((i + 1/2 - U0) / (U1 - U0), 0, 1) with U0, U1 the vertices' major pixel
 * coordinates, and colour = fma(f, color1 - color0, color0), each an f32 operation
 * rounded once. */
typedef struct lg_chord {
  float x0, y0, x1, y1;
  float color0[4];
  float color1[4];
} lg_chord;

enum lg_path_flags {
  LG_PATH_NEAR_DEGENERATE = 1, /* a decision on this path fell inside the FP64 epsilon band */
  LG_PATH_TIR = 2,             /* this segment ends in total internal reflection */
  LG_PATH_FALLBACK = 4,        /* candidate list overflowed: every object re-solved in FP64 */
  LG_PATH_ILL_CONDITIONED = 8  /* double-float mode: the ray's rounding bound passed 1e-6 (chaotic
                                  amplification along the path), so the path may part from an
                                  FP64 trace although no decision fell in a band */
};
/* LG_SRC_STRING_MOD is kept for numbering; string-mod lines are lg_chord records. */
enum lg_path_source { LG_SRC_TRACE = 0, LG_SRC_CONTROL_LINE = 1, LG_SRC_STRING_MOD = 2 };

/* Identity of a segment in the ray tree, for parity checks against a CPU trace. */
typedef struct lg_path_record {
  uint64_t path;    /* bit k = branch taken at generation k+1: 0 reflected/mirror, 1 refracted */
  uint32_t primary; /* primary ray index within its light */
  uint16_t light;   /* light index */
  uint8_t gen;      /* generation (0 = primary ray) */
  uint8_t flags;    /* enum lg_path_flags, inherited by descendants */
  int32_t hit;      /* object index hit, -1 = canvas exit */
  uint32_t source;  /* enum lg_path_source */
} lg_path_record;

typedef struct lg_trace_stats {
  uint64_t primary_rays;   /* rays generated by all lights */
  uint64_t ray_visits;     /* queue entries traced (after the cutoff) */
  uint64_t segments;       /* segments written (traced + control lines) */
  uint64_t fp64_solves;    /* object intersections re-solved in FP64 */
  uint64_t fp64_fallbacks; /* rays whose FP32 candidate list overflowed */
  uint64_t near_degenerate;/* segments carrying LG_PATH_NEAR_DEGENERATE (a decision in its band) */
  uint64_t pixels;         /* pixel updates made by lg_accumulate */
  uint64_t tile_refs;      /* (segment, tile) pairs binned by lg_accumulate */
  uint64_t bound_tests;    /* FP32 ray / bounding-circle tests of the nearest-hit search */
  uint64_t object_tests;   /* FP32 ray / object classifications (bounding test passed) */
  uint32_t retries;        /* re-launches after a ring/queue overflow */
  uint32_t _pad;
  /* device time from CUDA events on the library's stream; lg_render splits accumulate
     into bin (count, scan, scatter) and raster (tile accumulation) */
  float trace_ms, accumulate_ms, resolve_ms, total_ms, bin_ms, raster_ms;
  /* lg_render: the trace's kernels summed over the generations: the FP32 nearest-hit search,
     the precise solve (k_solve_x, or k_refine + k_full), the bounce */
  float scan_ms, solve_ms, bounce_ms;
  float _pad2;
  uint64_t ill_conditioned; /* segments carrying LG_PATH_ILL_CONDITIONED (double-float mode) */
} lg_trace_stats;

typedef struct lg_device_opts {
  int32_t device;             /* CUDA device ordinal */
  int32_t raster_variant;     /* 0: autotune on the first accumulation; 1: shared-atomic tile
                                 raster; 2: warp-private tile raster (results are identical) */
  uint64_t segment_capacity;  /* initial segment ring size (0 = automatic); grows on overflow */
  uint64_t queue_capacity;    /* initial per-generation ray queue size (0 = automatic) */
  uint64_t stream_segments;   /* lg_render accumulates while tracing, with a ring of this many
                                 segments, once a frame has more (0 = 2^28) */
  int32_t culling;            /* lg_culling: spatial culling of the nearest-hit search */
  float grid_density;         /* culling grid cells per object (0 = 2) */
  int32_t wait_polls;         /* polls of each bounded device-side wait before it gives up with
                                 LG_ERR_TIMEOUT: 0 = default (2^22); a negative value gives up
                                 at once (exercises the timeout path in tests) */
  int32_t scan_pairs;         /* pair slots per lane of the FP32 nearest-hit scan, 8 or 16; 0 =
                                 autotune: the second lg_render / lg_batch_render of each scene or
                                 batch renders with both and keeps the faster (results are
                                 identical either way; a scene rendered once is not tuned) */
} lg_device_opts;

/* Nearest-hit culling (replaces the reference's approximate tile map, tile_map.rs:18-146).
 * The culled search visits objects in ray order through a uniform grid and returns the
 * same hits as the full scan. */
typedef enum lg_culling {
  LG_CULL_AUTO = 0,  /* grid for scenes of LG_CULL_AUTO_MIN objects or more; the bounce's medium
                        test uses it, and the nearest-hit scan walks it from LG_CULL_WALK_MIN
                        objects (batches: always) or as the scene's second lg_render measured
                        faster (lg_device_opts.scan_pairs = 0) */
  LG_CULL_OFF = 1,   /* every ray tests every object's bounding circle */
  LG_CULL_ON = 2     /* grid for every scene, walked by the scan */
} lg_culling;
#define LG_CULL_AUTO_MIN 16
#define LG_CULL_WALK_MIN 96

typedef struct lg_ctx lg_ctx;

/* ---- context --------------------------------------------------------------------------- */
lg_status lg_create(lg_ctx** out, const lg_device_opts* opts_or_null);
lg_status lg_destroy(lg_ctx* ctx);
const char* lg_last_error(const lg_ctx* ctx_or_null);
uint32_t lg_abi_version(void);

/* ---- one scene ------------------------------------------------------------------------ */
/* Copies a scene (geometry trees, objects, lights, parameters) to the device.  Replaces
 * the whole object/light list, like Tracer::clear + push_object/push_light
 * (tracer.rs:54-94) followed by Light::set_num_rays (light.rs:45-51).  A call rejected by
 * its argument checks keeps the previous scene; one that fails later (device memory) leaves
 * no scene (LG_ERR_NO_SCENE until the next successful upload). */
lg_status lg_scene_upload(lg_ctx* ctx, const lg_geo* geos, uint32_t n_geo,
                          const lg_object* objects, uint32_t n_objects,
                          const lg_light* lights, uint32_t n_lights, const lg_params* params);

/* Traces every light (Tracer::trace_all, tracer.rs:276-358) into the device segment ring.
 * If the ring or a generation queue overflows, the library grows it and traces again
 * (stats->retries counts this). */
lg_status lg_trace(lg_ctx* ctx, lg_trace_stats* stats_or_null);

/* Clears the accumulation image to params.clear_color and rasterises every segment in the
 * ring into it: aliased 1-px lines, one sample per pixel column (x-major) or row
 * (y-major) at the pixel centre, half-open at the far end, blended per lg_params. */
lg_status lg_accumulate(lg_ctx* ctx, lg_trace_stats* stats_or_null);

/* Rasterises caller-provided segments (host memory) into the accumulation image after
 * clearing it.  Same raster rule and blend as lg_accumulate. */
lg_status lg_accumulate_segments(lg_ctx* ctx, const lg_segment* segments, uint64_t n,
                                 lg_trace_stats* stats_or_null);

/* Converts the accumulation image to RGBA16F (IEEE binary16, round to nearest even),
 * row 0 = top of the canvas.  dst is host memory unless dst_is_device != 0.
 * pitch_bytes >= width * 8. */
lg_status lg_resolve_f16(lg_ctx* ctx, uint16_t* dst, size_t pitch_bytes, int32_t dst_is_device);

/* Optional export tonemap (renderer.rs:313-328): u8 = sat(f^(1/2.2) * 255), truncating
 * like Rust `as u8`; RGBA8, pitch_bytes >= width * 4. */
lg_status lg_resolve_rgba8(lg_ctx* ctx, uint8_t* dst, size_t pitch_bytes, int32_t dst_is_device);

/* trace + accumulate + resolve_f16 as one captured CUDA graph launch. */
lg_status lg_render(lg_ctx* ctx, uint16_t* dst, size_t pitch_bytes, int32_t dst_is_device,
                    lg_trace_stats* stats_or_null);

/* Copies segments (and optionally their path records) out of the ring.  If cap is too
 * small, returns LG_ERR_TRUNCATED with *n_out = segments available. */
lg_status lg_segments_download(lg_ctx* ctx, lg_segment* out, lg_path_record* paths_or_null,
                               uint64_t cap, uint64_t* n_out);

/* Copies the raw accumulation image: width*height*4 values, int64 (FIXED64) or float (F32). */
lg_status lg_accum_download(lg_ctx* ctx, void* out, uint64_t cap_bytes);

/* Copies the string-mod lines of the last lg_trace / lg_render (lg_params.string_mod.modulo
 * of them, or with a nested mod its modulo, or none when the lines do not cross; none in a
 * sampled frame with ray_offset != 0, or after lg_accumulate_segments).
 * *n_out receives the count; LG_ERR_TRUNCATED when cap is smaller.  lg_accumulate draws
 * them together with the segments. */
lg_status lg_chords_download(lg_ctx* ctx, lg_chord* out, uint64_t cap, uint64_t* n_out);

/* ---- batches: many scenes in one trace ----------------------------------------------- *
 * No counterpart in the reference, which traces one scene per Tracer (tracer.rs:276-358).
 * A batch concatenates the scenes' tables and traces all rays of all scenes together, one
 * wavefront per generation, accumulating each generation into the scenes' own images. */
typedef struct lg_scene_desc {
  const lg_geo* geos;
  const lg_object* objects;
  const lg_light* lights;
  const lg_params* params;
  uint32_t n_geo, n_objects, n_lights, _pad;
} lg_scene_desc;

/* Uploads k scenes (replacing the context's scene or batch; lg_trace / lg_render then need
 * lg_scene_upload again).  Scenes may differ in objects, lights, canvas size, max_bounce and
 * cutoff; they must share the accum mode, blend state, blend constant and clear colour, and
 * may not use the string-mod overlay (LG_ERR_UNSUPPORTED).  At most 65535 scenes, 65535
 * objects per scene and 65535 lights in all. */
lg_status lg_batch_upload(lg_ctx* ctx, const lg_scene_desc* scenes, uint32_t k);

/* Traces, accumulates and resolves every scene of the batch (one captured CUDA graph).
 * dst receives the RGBA16F images one after another in scene order, each width*height*4
 * binary16 values with rows top-down and no padding; dst_bytes >= 8 * sum(width*height).
 * Each image is bit-identical to lg_render of that scene alone.  The first call of a
 * context also picks the faster tile-raster kernel for the batch (autotune). */
lg_status lg_batch_render(lg_ctx* ctx, uint16_t* dst, uint64_t dst_bytes, int32_t dst_is_device,
                          lg_trace_stats* stats_or_null);

/* First pixel of scene `scene`'s image in lg_batch_render's output (in pixels, 4 values each). */
lg_status lg_batch_image_offset(const lg_ctx* ctx, uint32_t scene, uint64_t* px_offset);

/* ---- serving: continuous batching of scene requests ---------------------------------- *
 * No counterpart in the reference.  lg_serve_step runs one generation of the multi-scene
 * wavefront over every request in flight and admits waiting requests at every step (their
 * primaries join the same launch as the older requests' deeper generations).  Admission is
 * bounded by the HBM budget (ray queues, segment ring, image pools); a finished request is
 * resolved to RGBA16F and kept until lg_serve_poll copies it out (which frees its memory).
 * Every image is bit-identical to lg_render of the scene alone.  Requests share blend state
 * and clear colour, accumulate in LG_ACCUM_FIXED64 and may not use the string-mod overlay.
 * While serving, lg_scene_upload and lg_batch_upload return LG_ERR_INVALID_ARGUMENT. */
typedef struct lg_serve_opts {
  uint64_t hbm_budget_bytes; /* device memory the server may hold (0: 80 % of free memory) */
  uint32_t max_slots;        /* requests in flight at once, 1..65535 */
  uint32_t _pad;
} lg_serve_opts;

typedef struct lg_serve_step_stats {
  uint32_t admitted, finished, in_flight, pending;
  uint32_t rasterised;      /* 1 if the step accumulated the segment ring */
  uint32_t restarted;       /* 1 if the step overflowed its queue and restarted the requests in flight */
  uint64_t live_rays;       /* rays queued for the next step */
  uint64_t segments;        /* segments accumulated so far */
  float step_ms;            /* host wall time of the step */
  uint32_t _pad;
} lg_serve_step_stats;

lg_status lg_serve_begin(lg_ctx* ctx, const lg_serve_opts* opts);
/* Validates and queues one scene; *id_out identifies it.  LG_ERR_BUDGET if the scene could
 * never be admitted under the budget (too many primaries or too large a canvas). */
lg_status lg_serve_submit(lg_ctx* ctx, const lg_scene_desc* scene, uint64_t* id_out);
lg_status lg_serve_step(lg_ctx* ctx, lg_serve_step_stats* stats_or_null);
/* LG_OK: the finished image (width*height*4 binary16, rows top-down) was copied to dst and
 * the request forgotten; LG_ERR_NOT_READY: still queued or in flight; LG_ERR_NOT_FOUND. */
lg_status lg_serve_poll(lg_ctx* ctx, uint64_t id, uint16_t* dst, uint64_t dst_bytes, int32_t dst_is_device);
lg_status lg_serve_end(lg_ctx* ctx);

/* No counterpart in the reference.  For callers that may not allocate device memory
 * (plug-ins whose host owns every allocation, real-time loops that must not take the
 * allocator's locks or risk the implicit synchronisation of cudaMalloc / cudaFree, code
 * under a fixed memory budget): clears `accum` to params->clear_color and rasterises the
 * n segments into it exactly like lg_accumulate_segments, on the calling thread's current
 * device and the given stream (NULL = default stream), without a context and without
 * allocating.  `segments` and `accum` must be device-accessible (accum: width*height*4
 * int64 for LG_ACCUM_FIXED64, float for LG_ACCUM_F32).  Canvas sides, accumulation mode
 * and blend state follow lg_params' rules (LG_ERR_INVALID_ARGUMENT / LG_ERR_UNSUPPORTED).
 * Binning scratch lives in one 32 MiB array per device, resident until the process exits;
 * limits per call: at most 4096 tiles of 32x32 pixels (e.g. 2048x2048) and 8,000,000
 * (segment, tile) pairs, else LG_ERR_BUDGET (and the image is not valid; the next call
 * starts afresh).  The first call on a device sets the array up; make it before any
 * stream capture.  Calls share the array, so calls that overlap on the GPU race:
 * serialise them.  Every call reads two counters back and waits for its stream before
 * returning; *pixels_out (optional) receives the number of pixel updates. */
lg_status lg_accumulate_segments_noalloc(const lg_segment* segments, uint64_t n, const lg_params* params,
                                         void* accum, void* stream, uint64_t* pixels_out);

#ifdef __cplusplus
}
#endif
#endif /* LIGHT_GARDEN_GB300_LG_H */
