/*
 * lg_oracle.h — CPU FP64 restatement of light_garden's trace-and-accumulate path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load this library, and only as the checker or as the timed CPU
 * baseline.  The product path (liblightgarden_cuda.so) never links or calls it.
 *
 * PARITY UNPINNED: the reference is Rust (no toolchain here) and its geometry crate
 * collision2d (git rev a7b471b54a940622f658a16177d63925536f16c3, Cargo.lock:880-887) is
 * not vendored, and the reference ships no tests or golden outputs.  This oracle follows
 * the reference's own control flow line by line (tracer.rs, light.rs, object.rs,
 * string_mod.rs) and restates the collision2d primitives from their mathematics; the
 * definitions it has to choose are listed at the top of lg_oracle.c.
 */
#ifndef LG_ORACLE_H
#define LG_ORACLE_H
#include <stdint.h>
#include "../include/lg.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  LGO_OK = 0,
  LGO_ERR_INVALID = -1,
  LGO_ERR_UNSUPPORTED = -2,
  LGO_ERR_OOM = -3,
  LGO_ERR_TRUNCATED = -6
};

typedef struct lgo_stats {
  uint64_t primary_rays;
  uint64_t ray_visits;
  uint64_t segments;
  uint64_t near_degenerate;
  uint64_t pixels;
  double seconds;
} lgo_stats;

typedef struct lgo_hit {
  double t, px, py, nx, ny;
} lgo_hit;

/* Trace every light (tracer.rs:276-358).  Only primaries with i % ray_stride == ray_offset
 * are traced (ray_stride = 1 traces all).  The curved-mirror control lines are appended
 * when ray_offset == 0 and the params ask for them (string-mod lines: lgo_string_mod_chords).  seg64 (optional) receives
 * x0,y0,x1,y1 in FP64 per segment.  n_threads <= 0 uses all online cores. */
int lgo_trace(const lg_geo* geos, uint32_t n_geo, const lg_object* objs, uint32_t n_obj,
              const lg_light* lights, uint32_t n_lights, const lg_params* prm,
              uint32_t ray_stride, uint32_t ray_offset, int n_threads,
              lg_segment* segs, lg_path_record* paths, double* seg64, uint64_t cap,
              uint64_t* n_out, lgo_stats* stats);

/* String-mod lines of prm->string_mod (string_mod.rs:33-158): modulo of them, or with a
 * nested mod the nested modulo (none when the lines do not cross), written to out[0..n).
 * *n_out receives the count; LGO_ERR_TRUNCATED when cap is smaller. */
int lgo_string_mod_chords(const lg_params* prm, lg_chord* out, uint64_t cap, uint64_t* n_out);
/* Crossing points of the mod's lines in the order of StringMod::line_crossings_as_points
 * (string_mod.rs:87-102), as (x, y) pairs: up to cap of them to xy (NULL: count only);
 * *n_out receives the count, LGO_ERR_TRUNCATED when cap is smaller. */
int lgo_string_mod_crossings(const lg_string_mod* sm, double* xy, uint64_t cap, uint64_t* n_out);
/* The crossing of segments ab and cd that lgo_string_mod_crossings uses (include/lg.h states it
 * for lg_string_mod.nested): 1 and the point when they cross, else 0. */
int lgo_seg_cross(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy,
                  double* px, double* py);
/* Raster of string-mod lines (the segment raster rule, colour interpolated along the major
 * axis as include/lg.h states for lg_chord), into the same images as lgo_raster(_f64). */
int lgo_raster_chords(const lg_chord* chords, uint64_t n, const lg_params* prm, int64_t* accum,
                      uint64_t* pixels);
int lgo_raster_chords_f64(const lg_chord* chords, uint64_t n, const lg_params* prm, double* accum,
                          uint64_t* pixels);

/* The ray generators' sin / cos / atan (see lg_oracle.c: plain IEEE double operations,
 * within a few ulp of the C library). */
void lgo_sincos(double x, double* s, double* c);
double lgo_atan(double x);

/* Primary rays of one light (light.rs set_num_rays): out[4*i..] = ox, oy, dx, dy. */
int lgo_light_rays(const lg_light* light, double* out, uint64_t cap);

/* All hits (t > T_MIN) of one ray with geometry node `root`, in collision2d order. */
int lgo_geo_hits(const lg_geo* geos, uint32_t n_geo, int32_t root, double ox, double oy,
                 double dx, double dy, lgo_hit* out, int cap, uint32_t* flags);
int lgo_geo_contains(const lg_geo* geos, uint32_t n_geo, int32_t root, double px, double py);

/* Ray::refract restated: returns 1 if a refracted ray exists (no TIR). */
int lgo_refract(double dx, double dy, double nx, double ny, double n1, double n2,
                double* refl_dir, double* refr_dir, double* reflectance);

/* Start medium of a light (tracer.rs:280-287). */
double lgo_light_medium(const lg_geo* geos, uint32_t n_geo, const lg_object* objs,
                        uint32_t n_obj, const lg_light* light);

/* Raster (the raster rule of lg_accumulate) into an int64 Q31.32 RGBA image that the
 * caller initialised (lgo_clear).  Returns pixel updates.  n_threads as above. */
int lgo_clear(int64_t* accum, uint32_t w, uint32_t h, const lg_params* prm);
int lgo_raster(const lg_segment* segs, uint64_t n, const lg_params* prm, int64_t* accum,
               int n_threads, uint64_t* pixels);
/* Same raster into a double image (reference for LG_ACCUM_F32 within tolerance). */
int lgo_raster_f64(const lg_segment* segs, uint64_t n, const lg_params* prm, double* accum,
                   uint64_t* pixels);
/* Q31.32 -> f32 -> binary16 (round to nearest even); rows top-down like lg_resolve_f16. */
void lgo_resolve_f16(const int64_t* accum, uint32_t w, uint32_t h, uint16_t* out);
void lgo_resolve_rgba8(const int64_t* accum, uint32_t w, uint32_t h, uint8_t* out);
uint16_t lgo_f32_to_f16(float f);
float lgo_f16_to_f32(uint16_t h);
int64_t lgo_fixed(float v);

#ifdef __cplusplus
}
#endif
#endif
