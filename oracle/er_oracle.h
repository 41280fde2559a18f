/*
 * er_oracle.h - CPU oracle for the Exposure Render transport path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: a plain-C restatement of
 * the reference's single-scattering path and post-processing, used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The
 * product (libexposurerender.so) never links or calls it.
 *
 * Pinning: every function here is compared bit-for-bit with the reference's
 * own code compiled for the host (oracle/ref_harness.cpp, built by
 * oracle/Makefile into oracle/_ref/) and with the golden vectors that
 * tests/golden/make_golden.py generated from that build.
 *
 * The same entry points are exported by both libraries with the prefixes
 * or_ (this restatement, oracle/_build/liberoracle.so) and ref_ (the
 * reference, oracle/_ref/liberref.so), so a test can run both on one input.
 *
 * FP64 oracle: er_oracle.c compiled with -DER_ORACLE_FP64 (prefix fp64_,
 * oracle/_build/liberfp64.so) evaluates the same estimators in binary64
 * with the C library's double functions; every `float` of this header is a
 * `double` there.  It is the converged reference of the image-RMSE
 * measurements, not a bit-exact checker.
 */
#ifndef ER_ORACLE_H
#define ER_ORACLE_H

#include <stdint.h>
#include "er_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ER_ORACLE_PREFIX
#define ER_ORACLE_PREFIX or_
#endif
#define ER_OR_CAT2(a, b) a##b
#define ER_OR_CAT(a, b) ER_OR_CAT2(a, b)
#define ER_OR(name) ER_OR_CAT(ER_ORACLE_PREFIX, name)

typedef struct or_scene or_scene;

/* Builds the scene the way BindVolume/BindLight/BindTexture/BindTracer do:
   light i of `lights` has light ID i, texture i has texture ID i. */
or_scene* ER_OR(scene_create)(const er_tracer_desc* tracer, const er_volume_desc* volume,
                              const er_light_desc* lights, int32_t n_lights,
                              const er_texture_desc* textures, int32_t n_textures);
void ER_OR(scene_destroy)(or_scene* scene);
/* BindObject for the scene: object i of `objects` is the i-th bound object
   (gpObjects[i]); the tracer's object_count says how many are intersected */
void ER_OR(scene_set_objects)(or_scene* scene, const er_object_desc* objects, int32_t n);
/* BindClippingObject for the scene: clipping object i has ID i; the
   tracer's clipping_object_ids name the ones applied to the volume */
void ER_OR(scene_set_clipping_objects)(or_scene* scene, const er_clipping_object_desc* clips, int32_t n);
/* BindBitmap for the scene: bitmap i is gpBitmaps[i] (ErTexture::BitmapID) */
void ER_OR(scene_set_bitmaps)(or_scene* scene, const er_bitmap_desc* bitmaps, int32_t n);

/* KrnlSingleScattering over the whole film with stateful lanes
   (lanes[0..W*H) = RandomSeeds1, lanes[W*H..2W*H) = RandomSeeds2, advanced in
   place); frame receives W*H XYZA float4. */
void ER_OR(render_frame)(or_scene* scene, uint32_t* lanes, float* frame, int32_t nthreads);

/* Counter-seeded samples: sum over s in [first, first+spp) of SingleScattering
   with lanes er_seed_lanes(seed, view, pixel, s), for the pixel rectangle
   [x0, x0+w) x [y0, y0+h); sum receives w*h float4. */
void ER_OR(render_sum)(or_scene* scene, int32_t spp, uint32_t view, uint32_t first_sample,
                       int32_t x0, int32_t y0, int32_t w, int32_t h, float* sum, int32_t nthreads);
/* render_sum plus the per-pixel sums of squares of the four components
   (sum2 receives w*h float4) */
void ER_OR(render_moments)(or_scene* scene, int32_t spp, uint32_t view, uint32_t first_sample,
                           int32_t x0, int32_t y0, int32_t w, int32_t h, float* sum, float* sum2, int32_t nthreads);

/* KrnlComputeAutoFocusDistance (Source/autofocus.cuh:26-62) for film
   pixel (u, v) with RNG lanes (lane0, lane1) */
float ER_OR(autofocus)(or_scene* scene, int32_t u, int32_t v, uint32_t lane0, uint32_t lane1);

/* Work counters per sample of the last render_frame / render_sum /
   render_moments, in the order of the OR_STAT_* indices: volume lookups
   (GetIntensity calls) in the primary free flight (with the event normal),
   majorant-grid reads (all rays), shadow-segment lookups, shadow-segment
   majorant reads, volume scatter events, shadow segments, lookups of the
   event normals (all normals). */
enum { OR_STAT_FREE_FLIGHT_LOOKUPS = 0, OR_STAT_MAJORANT = 1, OR_STAT_SHADOW_LOOKUPS = 2, OR_STAT_SHADOW_MAJORANT = 3,
       OR_STAT_EVENTS = 4, OR_STAT_SHADOW_RAYS = 5, OR_STAT_NORMAL_LOOKUPS = 6, OR_NSTATS = 7 };
void ER_OR(render_stats)(double* out);

/* Differentiable medium (extension): a float density grid (the scene
   volume's resolution and placement), n cubic B-spline opacity values over
   density, sigma = scale * opacity, albedo, NEE probability q and a fixed
   majorant grid of brick^3 voxels (copied).  dm_render writes per-pixel
   sums (W*H*3) and optionally every sample ((s*H*W + pixel)*3);
   dm_adjoint adds dLoss/d(density) and dLoss/d(opacity values) given
   dLoss/d(pixel sum) and the forward samples.  In the FP64 build every
   float buffer is double. */
void ER_OR(dm_attach)(or_scene* scene, const float* rho, const float* tf_val, int32_t tf_n, float scale, const float* albedo,
                      float q, const float* majorant, int32_t brick);
/* Model of the medium (after dm_attach): 0 the B-spline opacity and
   isotropic albedo; 1 the tracer's transfer functions - the opacity PLF at
   the tracer's node positions with the node values tf_val (tf_n = the
   tracer's opacity node count), Diffuse/Specular/Glossiness/Emission of the
   tracer at the grid's float intensity - and its BRDF / phase / hybrid
   shading (the hybrid as the expected value over its shader choice); gm_inv
   is the hybrid's 1 / gradient-magnitude range, a constant. */
void ER_OR(dm_set_model)(or_scene* scene, int32_t model, float gm_inv);
void ER_OR(dm_render)(or_scene* scene, int32_t spp, uint32_t view, uint32_t first, float* sum, float* samples, int32_t nthreads);
void ER_OR(dm_adjoint)(or_scene* scene, int32_t spp, uint32_t view, uint32_t first, const float* dimg, const float* fwd,
                       float* g_rho, float* g_tf, int32_t nthreads);

/* The reference pipeline of RenderEstimate after the transport kernel
   (Source/core.cu:130-135): 3x3 Gaussian frame filter, running estimate
   update with divisor max(no_iterations,1), tone map.  frame is filtered in
   place (the reference copies FrameEstimateTemp back, :71-73). */
void ER_OR(post_frame)(float* frame, float* running, uint8_t* rgba, int32_t width, int32_t height,
                       int32_t no_iterations, float exposure);

/* mean lookups per sample of the last render call (restatement only; the
   reference harness returns 0) */
double ER_OR(lookups_per_sample)(void);

/* ---- known-answer helpers ---- */
void ER_OR(rng_draws)(uint32_t lane0, uint32_t lane1, int32_t n, float* out);
void ER_OR(rng_get2_get3)(uint32_t lane0, uint32_t lane1, float* out5);
void ER_OR(plf_evaluate)(const er_plf* plf, int32_t n, const float* x, float* y);
/* volume lookups (GetIntensity) at n world points */
void ER_OR(get_intensity)(or_scene* scene, int32_t n, const float* p, float* out);
void ER_OR(normalized_gradient)(or_scene* scene, int32_t n, const float* p, float* out);
void ER_OR(gradient_magnitude)(or_scene* scene, int32_t n, const float* p, float* out);
/* IntersectBox against the volume box: out = {valid, near, far} per ray (o, d, mint, maxt) */
void ER_OR(intersect_volume_box)(or_scene* scene, int32_t n, const float* rays8, float* out3);
void ER_OR(concentric_sample_disk)(int32_t n, const float* u2, float* out2);
/* tone map of n XYZA values with the given exposure -> RGBA8 */
void ER_OR(tonemap)(int32_t n, const float* xyza, float exposure, uint8_t* rgba);
/* primary camera ray of pixel (x, y) with film jitter (fu, fv) and lens (lu, lv): out = {o, d} */
void ER_OR(camera_ray)(or_scene* scene, int32_t x, int32_t y, const float* uv4, float* out6);
/* derived camera frame {N, U, V, screen00, screen01, screen10, screen11, inv0, inv1} */
void ER_OR(camera_frame)(or_scene* scene, float* out15);
/* derived volume geometry {minp(3), inv_size(3), min_step, spacing(3), size(3)} */
void ER_OR(volume_frame)(or_scene* scene, float* out13);

/* restatement only (no live reference code exists for these): */
/* separable bilateral filter on RGBA8 (design of Source/filterrunningestimate.cuh:35-200) */
void ER_OR(bilateral)(const uint8_t* in, uint8_t* tmp, uint8_t* out, int32_t width, int32_t height, int32_t radius,
                      float sigma_d, float sigma_r);
/* gradient magnitude at voxel centres (Source/gradientmagnitude.cuh:28-71 design); returns the maximum */
float ER_OR(gradient_magnitude_volume)(or_scene* scene, uint16_t* gm);
/* include/er_math.h on the host: fn 0 log, 1 exp, 2 sin, 3 cos, 4 tan, 5 pow, 6 acos, 7 atan2 */
void ER_OR(math_eval)(int32_t fn, int32_t n, const float* x, const float* y, float* out);
/* IntersectsLight of one shape for n segments (O, D, MinT, MaxT: 8 floats each) */
void ER_OR(segments_hit_shape)(const er_shape* shape, int32_t n, const float* seg, int32_t* hit);
/* majorant grid of the delta tracker: ds * max sigma over each brick plus a one-voxel apron */
void ER_OR(majorant_grid)(const uint16_t* vox, const int32_t* res, int32_t brick, const float* sigma, int32_t n, float ds, float* out);

#ifdef __cplusplus
}
#endif

#endif
