/*
 * er_capi.h - C ABI of the GB300 Exposure Render transport library
 * (libexposurerender.so).
 *
 * Plain C: POD descriptors, integer status codes, no C++ types and no
 * exceptions across the boundary.  Every entry point names the reference
 * interface it replaces (paths are relative to the reference project).
 *
 * Semantics follow the reference's global-singleton API
 * (Source/exposurerender.h:32-42, Source/core.cu:50-155):
 *   - one library-wide context per process (per CUDA device 0 .. n-1 chosen by
 *     er_set_device); bind lists hold at most ER_MAX_ITEMS_PER_LIST items each,
 *     like List<D,H,32> (Source/list.cuh:27,63);
 *   - Bind assigns ID = counter++ on first bind and writes it back through the
 *     `id` pointer (the reference writes the caller's `mutable int ID`,
 *     Source/erbindable.h:65, Source/list.cuh:69-76); binding an existing ID
 *     updates the item in place; IDs are never reused;
 *   - lights referenced by a tracer are addressed by light ID (the reference's
 *     packed-array index equals the ID while nothing is unbound,
 *     Source/list.cuh:115-126, Source/lights.h:96);
 *   - errors: the reference throws ExposureRender::Exception
 *     (Source/exception.h:27-55) or refuses silently (Source/list.cuh:63-67);
 *     here every call returns an er_status and er_last_error_message() holds
 *     the text of the last failure on the calling thread.
 */
#ifndef ER_CAPI_H
#define ER_CAPI_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define ER_API __declspec(dllexport)
#else
#define ER_API __attribute__((visibility("default")))
#endif

#define ER_ABI_VERSION 1

/* Source/defines.h:76 (MAX_NO_TF_NODES); AddNode keeps Count < 128 (Source/plf.h:53) */
#define ER_MAX_TF_NODES 128
/* Source/list.cuh:27,63: List<D,H,MaxSize=32> accepts Map.size()+1 < 32 */
#define ER_MAX_ITEMS_PER_LIST 31
/* Source/vector.h:554-579: Indices holds 256 ints */
#define ER_MAX_INDICES 256

typedef enum er_status {
    ER_OK = 0,
    ER_ERR_INVALID_ID = 1,        /* Source/list.cuh:154-161 throws Warning */
    ER_ERR_INVALID_ARGUMENT = 2,
    ER_ERR_LIST_FULL = 3,         /* Source/list.cuh:63-67 refuses silently */
    ER_ERR_CUDA = 4,              /* Source/wrapper.cuh:38-46 throws Error */
    ER_ERR_OUT_OF_MEMORY = 5,
    ER_ERR_UNSUPPORTED = 6,       /* a scene feature the selected kernel does not implement */
    ER_ERR_NO_DEVICE = 7,
    ER_ERR_TIMEOUT = 8            /* a device-side bounded wait gave up */
} er_status;

/* Source/enums.h:52-61 */
enum { ER_SHAPE_PLANE = 0, ER_SHAPE_DISK = 1, ER_SHAPE_RING = 2, ER_SHAPE_BOX = 3, ER_SHAPE_SPHERE = 4,
       ER_SHAPE_CYLINDER = 5, ER_SHAPE_CONE = 6 };
/* Source/enums.h:39-50 */
enum { ER_PROCEDURAL_UNIFORM = 0, ER_PROCEDURAL_CHECKER = 1, ER_PROCEDURAL_GRADIENT = 2 };
enum { ER_TEXTURE_PROCEDURAL = 0, ER_TEXTURE_BITMAP = 1 };
/* Source/enums.h:63-71 */
enum { ER_SHADING_BRDF_ONLY = 0, ER_SHADING_PHASE_ONLY = 1, ER_SHADING_HYBRID = 2,
       ER_SHADING_MODULATION = 3, ER_SHADING_THRESHOLD = 4, ER_SHADING_GRADIENT_MAGNITUDE = 5 };
/* Source/enums.h:73-78 */
enum { ER_GRADIENT_FORWARD = 0, ER_GRADIENT_CENTRAL = 1, ER_GRADIENT_FILTERED = 2 };
/* Source/enums.h:88-93 */
enum { ER_UNIT_POWER = 0, ER_UNIT_LUX = 1, ER_UNIT_INTENSITY = 2 };

/* Free-flight estimator (extension; 0 keeps the reference's fixed-step
   marcher of Source/raymarching.h:30-113). */
enum { ER_FREE_FLIGHT_MARCH = 0, ER_FREE_FLIGHT_DELTA = 1 };
/* Direct-light estimator (extension; 0 keeps the live light-sampling half of
   Source/transport.h:58-84, 1 adds the BSDF-sampling half :86-112). */
enum { ER_MIS_LIGHT_ONLY = 0, ER_MIS_FULL = 1 };

/* PiecewiseLinearFunction<128> (Source/plf.h:26-92, Source/pf.h:35-71).
   node_range starts at {FLT_MAX, FLT_MIN} and is widened by every AddNode. */
typedef struct er_plf {
    int32_t count;
    float node_range[2];
    float position[ER_MAX_TF_NODES];
    float value[ER_MAX_TF_NODES];
} er_plf;

/* ColorTransferFunction1D (Source/transferfunction.h:118-154) */
typedef struct er_color_tf {
    er_plf plf[3];
} er_color_tf;

/* Shape (Source/shape.h:57-113); area is recomputed by the library the way
   Shape::Update does (Source/shape.h:92-103), the field is ignored on input. */
typedef struct er_shape {
    float tm[4][4];
    float inv_tm[4][4];
    int32_t one_sided;
    int32_t type;
    float size[3];
    float area;
    float inner_radius;
    float outer_radius;
} er_shape;

/* ErLight (Source/erlight.h:27-66) */
typedef struct er_light_desc {
    int32_t visible;
    er_shape shape;
    int32_t texture_id;
    float multiplier;
    int32_t unit;
} er_light_desc;

/* Procedural (Source/procedural.h:27-60) */
typedef struct er_procedural {
    int32_t type;
    float uniform_color[3];
    float checker_color1[3];
    float checker_color2[3];
    er_color_tf gradient;
} er_procedural;

/* ErTexture (Source/ertexture.h:27-82) */
typedef struct er_texture_desc {
    int32_t type;
    float output_level;
    int32_t bitmap_id;
    er_procedural procedural;
    float offset[2];
    float repeat[2];
    int32_t flip[2];
} er_texture_desc;

/* ErVolume (Source/ervolume.h:28-74): voxels are x-fastest
   (z*Rx*Ry + y*Rx + x, Source/buffer3d.h:212-213) and are deep-copied at bind
   time like BindVoxels does (Source/buffer3d.h:166-198). */
typedef struct er_volume_desc {
    int32_t resolution[3];
    float spacing[3];
    int32_t normalize_size;
    const uint16_t* voxels;       /* host pointer, resolution[0]*[1]*[2] values */
} er_volume_desc;

/* ErBitmap (Source/erbitmap.h:28-61): RGBA8, row-major */
typedef struct er_bitmap_desc {
    int32_t resolution[2];
    const uint8_t* pixels;        /* host pointer, 4*resolution[0]*resolution[1] bytes */
} er_bitmap_desc;

/* ErObject (Source/erobject.h:27-67) */
typedef struct er_object_desc {
    er_shape shape;
    int32_t diffuse_texture_id;
    int32_t specular_texture_id;
    int32_t glossiness_texture_id;
    float ior;
} er_object_desc;

/* ErClippingObject (Source/erclippingobject.h:27-58) */
typedef struct er_clipping_object_desc {
    er_shape shape;
    int32_t invert;
} er_clipping_object_desc;

/* Camera inputs (Source/camera.h:98-108); the derived frame (N, U, V,
   screen window) is computed by the library as Camera::Update does
   (Source/camera.h:61-96). */
typedef struct er_camera_desc {
    int32_t film_size[2];
    float pos[3];
    float target[3];
    float up[3];
    float focal_distance;
    float aperture_size;
    float clip_near;
    float clip_far;
    float exposure;
    float gamma;
    float fov;
} er_camera_desc;

/* RenderSettings (Source/rendersettings.h:27-131) plus extension fields.
   er_default_render_settings() fills the reference defaults. */
typedef struct er_render_settings {
    /* TraversalSettings (Source/rendersettings.h:30-64) */
    float step_factor_primary;
    float step_factor_shadow;
    int32_t shadows;
    float max_shadow_distance;
    /* ShadingSettings (Source/rendersettings.h:66-106) */
    int32_t shading_type;
    float density_scale;
    int32_t opacity_modulated;
    int32_t gradient_computation;
    float gradient_threshold;
    float gradient_factor;
    /* extensions: zero-initialised values keep the reference's behaviour */
    int32_t apply_shading_type;   /* 0: every volume event uses the BRDF, as the live reference does
                                     (Source/transport.h:138 ignores Shading.Type); 1: shading_type
                                     selects BRDF / phase / hybrid per Source/scatterevent.h:155-212 */
    int32_t free_flight;          /* ER_FREE_FLIGHT_* */
    int32_t mis;                  /* ER_MIS_* */
    float volume_ior;             /* 15 in the reference (Source/transport.h:138); 0 means 15 */
    int32_t frame_filter;         /* 1: 3x3 Gaussian on each frame (Source/filterframeestimate.cuh:66-74); -1: off */
    int32_t bilateral;            /* 1: separable bilateral on the display image (Source/filterrunningestimate.cuh) */
    int32_t bilateral_radius;     /* KernelRadius of BilateralFilter (Source/filter.h:34-40) */
    float bilateral_sigma_d;      /* spatial sigma in pixels for KernelD[] */
    float bilateral_sigma_r;      /* range sigma in 0..255 luminance units for GaussSimilarity[] */
    uint32_t seed;                /* counter-based seed of the per-pixel RNG lanes */
    int32_t majorant_brick;       /* delta tracking: edge of the cubic voxel bricks of the majorant grid (0 means 8) */
    int32_t engine;               /* multi-sample launches: 0 auto (wavefront), 1 one-kernel path, 2 wavefront stages */
    int32_t tune_primary;         /* wavefront: resident 256-thread blocks per SM the free-flight stage is compiled for:
                                     2, 3, 4, 6 or 8 (0 or other values: 4) */
    int32_t tune_shadow;          /* wavefront: same for the shadow stage (0 or other values: 4) */
    int32_t tune_shade;           /* wavefront: resident 128-thread blocks per SM of the shade stage
                                     (2, 3, 4 or 6; 0 or other values: 2) */
    int32_t stratify;             /* 1: multi-sample renders (er_render_spp, er_trace_sum_device, batches) take
                                     each sample's point on the light, light choice, BSDF sample and first
                                     delta-tracking draw from per-pixel shifted rank-1 lattices over the
                                     sample index (er_stratified_sample in er_math.h) instead of the random
                                     stream; 0: the reference's draws */
    int32_t tune_stages;          /* delta tracking: bits 0-1 which wavefront tracking stages run persistent
                                     lanes (ER_PERSISTENT_*; 0: the shadow stage only); bits 2 and 3
                                     (ER_TUNE_NO_SKIP_*) are accepted and ignored */
} er_render_settings;

/* tune_stages bits 0-1: the persistent-lane stages keep every warp's lanes
   busy by handing a lane whose ray ended the next ray of the window; the
   per-thread stages keep neighbouring pixels' rays together in a warp */
enum {
    ER_PERSISTENT_SHADOW = 0,     /* persistent shadow stage, per-thread primary stage */
    ER_PERSISTENT_BOTH = 1,
    ER_PERSISTENT_NONE = 2,
    ER_PERSISTENT_PRIMARY = 3
};
/* tune_stages bits 2, 3: accepted for compatibility, no effect.  Each
   empty majorant brick stores its Chebyshev distance k to the nearest
   non-empty brick, and every delta/ratio tracker jumps in one step to the
   exit of the cube of empty bricks of half-width k-1 around it; the jump
   sets the face times the tracker continues from, so it is not optional. */
#define ER_TUNE_NO_SKIP_PRIMARY 4
#define ER_TUNE_NO_SKIP_SHADOW 8
#define ER_TUNE_NO_SKIP (ER_TUNE_NO_SKIP_PRIMARY | ER_TUNE_NO_SKIP_SHADOW)

/* ErTracer (Source/ertracer.h:33-117).  light_ids/object_ids/clipping_ids are
   item IDs returned by the bind calls. */
typedef struct er_tracer_desc {
    er_plf opacity;
    er_color_tf diffuse;
    er_color_tf specular;
    er_plf glossiness;
    er_color_tf emission;
    er_camera_desc camera;
    er_render_settings settings;
    int32_t volume_id;
    int32_t light_count;
    int32_t light_ids[ER_MAX_INDICES];
    int32_t object_count;
    int32_t object_ids[ER_MAX_INDICES];
    int32_t clipping_object_count;
    int32_t clipping_object_ids[ER_MAX_INDICES];
} er_tracer_desc;

/* ---------------------------------------------------------------------- */
/* library                                                                 */
/* ---------------------------------------------------------------------- */

ER_API int er_abi_version(void);
/* Text of the last error on this thread (never NULL). */
ER_API const char* er_last_error_message(void);
/* Selects the CUDA device used by subsequent calls of this thread's context
   (the reference always used the current device). */
ER_API er_status er_set_device(int device);
/* Stream for all asynchronous work (cudaStream_t passed as void*; NULL is the
   legacy default stream used by the reference, Source/macros.cuh:41-65). */
ER_API er_status er_set_stream(void* stream);
ER_API er_status er_synchronize(void);
/* Releases every bound item and device buffer. */
ER_API er_status er_reset(void);
ER_API void er_default_render_settings(er_render_settings* settings);
/* Appends a node the way PiecewiseLinearFunction::AddNode does
   (Source/plf.h:51-66), including the silent cap at 127 nodes. */
ER_API void er_plf_init(er_plf* plf);
ER_API void er_plf_add_node(er_plf* plf, float position, float value);

/* ---------------------------------------------------------------------- */
/* bind lists: Source/exposurerender.h:32-38, Source/core.cu:50-124        */
/* ---------------------------------------------------------------------- */

/* BindTracer(const ErTracer&, true) - Source/exposurerender.h:32 */
ER_API er_status er_bind_tracer(const er_tracer_desc* desc, int32_t* id);
/* BindTracer(const ErTracer&, false) */
ER_API er_status er_unbind_tracer(int32_t id);
/* BindVolume - Source/exposurerender.h:33 */
ER_API er_status er_bind_volume(const er_volume_desc* desc, int32_t* id);
ER_API er_status er_unbind_volume(int32_t id);
/* Partial re-upload of a bound volume (no counterpart in the reference, which
   re-uploads every voxel of every bound volume on each bind,
   Source/list.cuh:115-133): the box [offset, offset + size) of the volume
   (voxel units, x fastest) receives `voxels`, size[0]*size[1]*size[2] values
   packed x fastest.  The corner quads of the edited voxels, the maximum
   voxel, the gradient-magnitude range and every tracer's sigma table and
   majorant grid over this volume are refreshed; renders afterwards equal
   those of a fresh bind of the edited volume.  Waits for work queued on the
   volume.  ER_ERR_INVALID_ARGUMENT when the box leaves the volume. */
ER_API er_status er_update_volume_region(int32_t volume_id, const int32_t offset[3], const int32_t size[3], const uint16_t* voxels);
/* The same with the box's voxels in device memory, copied on `stream`
   (NULL: the library's stream). */
ER_API er_status er_update_volume_region_device(int32_t volume_id, const int32_t offset[3], const int32_t size[3],
                                                const uint16_t* d_voxels, void* stream);
/* BindLight - Source/exposurerender.h:34 */
ER_API er_status er_bind_light(const er_light_desc* desc, int32_t* id);
ER_API er_status er_unbind_light(int32_t id);
/* BindObject - Source/exposurerender.h:35 */
ER_API er_status er_bind_object(const er_object_desc* desc, int32_t* id);
ER_API er_status er_unbind_object(int32_t id);
/* BindClippingObject - Source/exposurerender.h:36 */
ER_API er_status er_bind_clipping_object(const er_clipping_object_desc* desc, int32_t* id);
ER_API er_status er_unbind_clipping_object(int32_t id);
/* BindTexture - Source/exposurerender.h:37 */
ER_API er_status er_bind_texture(const er_texture_desc* desc, int32_t* id);
ER_API er_status er_unbind_texture(int32_t id);
/* BindBitmap - Source/exposurerender.h:38 */
ER_API er_status er_bind_bitmap(const er_bitmap_desc* desc, int32_t* id);
ER_API er_status er_unbind_bitmap(int32_t id);

/* ---------------------------------------------------------------------- */
/* rendering                                                               */
/* ---------------------------------------------------------------------- */

/* RenderEstimate(int TracerID) - Source/exposurerender.h:39, Source/core.cu:126-136.
   One frame: one sample per pixel, 3x3 Gaussian frame filter, running
   cumulative moving average with divisor max(NoIterations,1), tone map,
   NoIterations++.  Asynchronous on the library stream. */
ER_API er_status er_render_estimate(int32_t tracer_id);
/* GetEstimate(int TracerID, unsigned char*) - Source/exposurerender.h:40,
   Source/core.cu:138-143.  Blocking copy of W*H RGBA8 into a host buffer of
   at least 4*W*H bytes (the bilateral-filtered image when the tracer's
   settings enable the bilateral filter). */
ER_API er_status er_get_estimate(int32_t tracer_id, uint8_t* rgba);
/* GetAutoFocusDistance - Source/exposurerender.h:41 (a stub at
   Source/core.cu:145-148) computed as Source/autofocus.cuh:26-62 designs it:
   the mean distance from the camera to the fixed-step march's scatter event
   over 100 rays jittered around the screen point of film pixel
   (film_u, film_v).  Its random lanes are er_seed_lanes(seed,
   ER_AUTOFOCUS_VIEW, film_v * W + film_u, 0) with the tracer's seed (the
   reference draws rand()).  Synchronous. */
#define ER_AUTOFOCUS_VIEW 0x41F0C05Eu
ER_API er_status er_get_auto_focus_distance(int32_t tracer_id, int32_t film_u, int32_t film_v, float* distance);
/* GetNoIterations - Source/exposurerender.h:42 (a stub at Source/core.cu:150-153) */
ER_API er_status er_get_no_iterations(int32_t tracer_id, int32_t* no_iterations);

/* Extension: `spp` samples per pixel in one launch, accumulated as a plain
   sample mean into the running estimate (no per-frame filter), followed by
   the frame filter on the mean, the tone map and the optional bilateral
   filter.  NoIterations grows by spp.  Asynchronous. */
ER_API er_status er_render_spp(int32_t tracer_id, int32_t spp);
/* Restarts progressive accumulation: running estimate, NoIterations and the
   per-pixel RNG lanes (FrameBuffer::Reset, Source/framebuffer.h:70-74). */
ER_API er_status er_reset_accumulation(int32_t tracer_id);
/* Blocking copies of the float XYZA buffers (W*H*4 floats each). */
ER_API er_status er_get_frame_estimate(int32_t tracer_id, float* xyza);
ER_API er_status er_get_running_estimate(int32_t tracer_id, float* xyza);
/* Per-pixel RNG lanes (2*W*H uint32: all lane-0 values then all lane-1 values). */
ER_API er_status er_get_seeds(int32_t tracer_id, uint32_t* lanes);
ER_API er_status er_set_seeds(int32_t tracer_id, const uint32_t* lanes);
/* Film size of a bound tracer. */
ER_API er_status er_get_film_size(int32_t tracer_id, int32_t* width, int32_t* height);

/* ---------------------------------------------------------------------- */
/* device-pointer entry points (caller owns all buffers; cudaStream_t as   */
/* void*; no allocation, no synchronisation)                               */
/* ---------------------------------------------------------------------- */

/* Renders `spp` counter-seeded samples per pixel of a bound tracer into a
   caller-owned float4 sum buffer (XYZ sum, alpha sum) of W*H*4 floats.
   Sample s of pixel p uses lanes er_seed_lanes(seed, view, p, first_sample+s)
   (include/er_math.h).  `accumulate` = 0 overwrites, 1 adds. */
ER_API er_status er_trace_sum_device(int32_t tracer_id, int32_t spp, uint32_t view, uint32_t first_sample,
                                     float* d_sum_xyza, int32_t accumulate, void* stream);

/* ---------------------------------------------------------------------- */
/* batched multi-view transport (no reference counterpart: the reference   */
/* renders one tracer per call, Source/core.cu:126-136 RenderEstimate)     */
/* ---------------------------------------------------------------------- */

/* One view of a batch: a bound tracer (its camera, film, volume, transfer
   functions and lights) and the samples to render into its sum buffer. */
typedef struct er_batch_view {
    int32_t tracer_id;
    int32_t spp;             /* samples per pixel per launch, > 0 */
    uint32_t view;           /* view index of the counter-based RNG stream */
    uint32_t first_sample;   /* stream index of the first sample (er_batch_advance moves it) */
    float* d_sum_xyza;       /* device, W*H*4 floats; NULL: the tracer's own sum buffer */
    int32_t accumulate;      /* 0 overwrites the sums, 1 adds to them */
    int32_t display;         /* 1: tone-map the mean into the tracer's display (er_get_estimate) */
    const er_camera_desc* camera;  /* NULL: the tracer's camera; else this camera and film
                                      (then d_sum_xyza is required and display must be 0) */
} er_batch_view;

#define ER_BATCH_GRAPH 1     /* er_batch_launch replays one captured CUDA graph */

/* Plans a batch: the samples of all views form one index space cut into
   windows of at most window_items samples (0: 8M), each window one pass of
   the wavefront stages over many views.  Every view's sums are bit-identical
   to er_trace_sum_device with the same tracer, spp, view, first_sample and
   accumulate.  With display set, the view's mean sum / n (n = first_sample +
   spp for an accumulating view, spp otherwise) goes through the frame
   filter, tone map and bilateral filter of the tracer's settings into the
   tracer's running estimate and display.  Binding or unbinding any resource
   re-plans the batch at its next launch.  Views share no output buffers. */
ER_API er_status er_batch_create(const er_batch_view* views, int32_t n_views, int32_t flags, int32_t window_items,
                                 int32_t* batch_id);
/* Enqueues one render of every view on `stream` (asynchronous). */
ER_API er_status er_batch_launch(int32_t batch_id, void* stream);
/* Enqueues on `stream` an update that adds `samples` to every view's
   first_sample, for progressive accumulation (first launch at 0, then
   advance by spp before each further launch). */
ER_API er_status er_batch_advance(int32_t batch_id, uint32_t samples, void* stream);
/* Resource-occupancy variants of the primary and shadow stages (2, 3, 4, 6
   or 8 resident blocks of 256 threads per SM; 0 keeps the current value).
   Without this call a batch uses the settings of its first view's tracer. */
ER_API er_status er_batch_set_tuning(int32_t batch_id, int32_t tune_primary, int32_t tune_shadow);
/* The tracking stages' persistent-lane mode of a batch (tune_stages of
   er_render_settings: ER_PERSISTENT_*; ER_TUNE_NO_SKIP_* bits ignored).
   Without this call (or er_batch_autotune) a batch uses its first view's
   tracer's value. */
ER_API er_status er_batch_set_stages(int32_t batch_id, int32_t tune_stages);
/* Tunes a batch on its own launches (a one-view probe misjudges a batch):
   times one launch of the whole batch per candidate, first each
   delta-tracking tracer's majorant brick in {1, 2, 4, 8} in turn (written
   into that tracer's settings, as er_autotune_tracer does), then eight
   tune_stages candidates, then six occupancy pairs of the tracking stages
   (as er_batch_set_tuning), keeping the fastest of each.  The views' sums are
   rendered into (accumulating views accumulate), so reset them afterwards.
   Synchronous. */
ER_API er_status er_batch_autotune(int32_t batch_id, void* stream, int32_t* tune_stages, float* msamples_per_s);
/* Windows, segments and queue bytes of the plan. */
ER_API er_status er_batch_info(int32_t batch_id, int32_t* n_windows, int32_t* n_segments, int64_t* queue_bytes);
ER_API er_status er_batch_destroy(int32_t batch_id);

/* ---------------------------------------------------------------------- */
/* differentiable medium (no reference counterpart)                        */
/* ---------------------------------------------------------------------- */

/* A float density grid in place of the tracer volume's intensities (same
   resolution and placement; the tracer supplies camera, lights and
   settings).  sigma(x) = scale * opacity(rho(x)), rho the trilinear
   interpolation of the grid, opacity a uniform cubic B-spline of the
   n_opacity values over u = 2 + rho * (n_opacity - 5) (control i at density
   (i - 2) / (n_opacity - 5)); isotropic phase function with `albedo`.
   The estimator (per sample: tentative collisions from the fixed majorant
   grid, next-event estimation with probability nee_probability and a
   ratio-tracked shadow segment, ratio-tracked throughput) draws random
   numbers independently of the medium, so for fixed seeds its samples are
   smooth functions of density and opacity values.  The majorant must bound
   sigma (er_medium_majorant with a margin); a violation sets the tracer's
   error word (ER_ERR_TIMEOUT at the next synchronising call). */
typedef struct er_medium_desc {
    const float* d_density;       /* device, the tracer volume's resolution, x fastest */
    const float* d_opacity;       /* device, n_opacity B-spline values (ER_MEDIUM_SPLINE) or the values of
                                     the tracer's opacity nodes (ER_MEDIUM_TRACER) */
    int32_t n_opacity;            /* 6 .. ER_MAX_TF_NODES (spline); the tracer's opacity node count (tracer) */
    float scale;                  /* sigma = scale * opacity */
    float albedo[3];              /* ER_MEDIUM_SPLINE only */
    float nee_probability;        /* (0, 1] */
    const float* d_majorant;      /* device, one float per brick of brick^3 voxels (x fastest) */
    int32_t brick;                /* 1 .. 64 */
    int32_t model;                /* ER_MEDIUM_SPLINE (0) or ER_MEDIUM_TRACER (1) */
    float gradient_magnitude_inv; /* ER_MEDIUM_TRACER with the hybrid shader: 1 / the gradient-magnitude range
                                     that normalises the shader switch (a constant of the estimator) */
} er_medium_desc;

/* Models of the differentiable medium.  ER_MEDIUM_SPLINE: the B-spline
   opacity and isotropic albedo above.  ER_MEDIUM_TRACER: the bound tracer's
   own transfer functions and shading over the float grid, read as
   intensities - sigma = scale * Opacity1D(I) with the tracer's opacity node
   positions and d_opacity's node values (the parameters), and at each
   next-event estimate Diffuse1D/Specular1D/Glossiness1D(I) with the BRDF
   (normal from central differences of the grid), the isotropic phase
   function, or the hybrid switch of the settings (Source/scatterevent.h:
   155-212) as the expected value over its random choice; Emission1D(I) at
   every collision.  The tracer's gradient_computation must be central
   differences; shading types other than BRDF, phase and hybrid are
   refused (ER_ERR_UNSUPPORTED). */
enum { ER_MEDIUM_SPLINE = 0, ER_MEDIUM_TRACER = 1 };

/* Per-brick majorant of a medium into d_majorant: scale * (max opacity
   control value over the spline segments of the brick's density range with
   a 1-voxel apron * margin + floor). */
ER_API er_status er_medium_majorant(int32_t tracer_id, const er_medium_desc* medium, float margin, float floor_, float* d_majorant,
                                    void* stream);
/* Renders spp samples per pixel: d_samples receives every sample
   ((s * H * W + pixel) * 3 floats, RGB of the phase-function albedo times
   light), d_sum_rgb (optional) the per-pixel sums in sample order. */
ER_API er_status er_medium_render(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                  uint32_t first_sample, float* d_samples, float* d_sum_rgb, void* stream);
/* The same samples with every medium-dependent quantity (density, opacity,
   collision weights, transmittances, sums) in binary64; the geometry, which
   does not depend on the medium, stays float.  For finite-difference checks
   of the adjoint: d_samples64 (spp*W*H*3 doubles) and d_sum64 (W*H*3). */
ER_API er_status er_medium_render_f64(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                      uint32_t first_sample, double* d_samples64, double* d_sum64, void* stream);
/* Path-replay adjoint: given dLoss/d(pixel sum) (W*H*3) and the forward
   samples (NULL: each thread recomputes its sample first), adds
   dLoss/d(density) (grid) and dLoss/d(opacity values) to the gradient
   buffers (either may be NULL).  d_samples must hold the forward of the
   parameter values the buffers hold now.  When the last er_medium_render or
   er_medium_adjoint call on this device was on the same stream with the
   same tracer (not rebuilt since), medium descriptor, spp, view, first
   sample and samples buffer, and covered at most 2^21 samples, the adjoint
   replays against the shadow jobs that call kept instead of walking and
   shadowing every path again. */
ER_API er_status er_medium_adjoint(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                   uint32_t first_sample, const float* d_dloss_dsum, const float* d_samples,
                                   float* d_grad_density, float* d_grad_opacity, void* stream);

/* ---------------------------------------------------------------------- */
/* autotuner (no reference counterpart)                                    */
/* ---------------------------------------------------------------------- */

typedef struct er_tune_result {
    int32_t majorant_brick;   /* edge of the delta tracker's majorant bricks */
    int32_t tune_primary;     /* occupancy variant of the primary stage */
    int32_t tune_shadow;      /* occupancy variant of the shadow stage */
    int32_t from_cache;       /* 1: read from the tuning cache, nothing measured */
    float msamples_per_s;     /* probe throughput of the chosen configuration */
    int32_t candidates;       /* configurations timed */
    int32_t tune_shade;       /* occupancy variant of the shade stage */
    int32_t tune_stages;      /* tune_stages of the chosen configuration (ER_PERSISTENT_*) */
} er_tune_result;

/* Times probe renders of a bound tracer (probe_spp samples per pixel of its
   film, raised to at least 2^21 samples per probe, one warm-up each) over
   majorant bricks {1, 2, 4, 8, 16} with empty-space skipping in both
   tracking stages, the free-flight stage only or neither (delta tracking
   only), then the occupancy
   variants of the wavefront stages under each persistent-lane mode
   (ER_PERSISTENT_*, delta tracking only), and last the shade stage's
   variants, and writes the fastest configuration into the bound tracer's
   settings (the caller's descriptor is not changed; re-binding it restores
   its values).
   Results are cached per device, volume and shading configuration in the
   file named by the environment variable ER_TUNE_CACHE (default
   $HOME/.cache/exposurerender_gb300/autotune.txt; "off" disables the
   cache).  Brick and occupancy change which random numbers a sample draws,
   not the estimator: the tuned tracer stays bit-exact with the CPU oracle
   given the same settings.  Synchronous. */
ER_API er_status er_autotune_tracer(int32_t tracer_id, int32_t probe_spp, er_tune_result* result);
/* Stage timing of the wavefront transport (no reference counterpart): while
   enabled, every launch outside a CUDA-graph capture records CUDA events
   around its stages on the launching stream.  er_profile_read waits for them
   and returns, per stage (0 primary: camera ray, free flight, visible lights;
   1 shade; 2 shadow segments; 3 per-pixel reduction), the milliseconds and
   launch counts accumulated since the previous read. */
ER_API er_status er_profile_enable(int32_t enable);
ER_API er_status er_profile_read(double* ms4, int64_t* launches4);
/* The settings the bound tracer renders with (after er_autotune_tracer). */
ER_API er_status er_get_render_settings(int32_t tracer_id, er_render_settings* settings);

/* One reference frame with explicit per-pixel lanes: d_lanes holds 2*W*H
   uint32 (lane 0 block then lane 1 block) and is advanced in place exactly as
   KrnlSingleScattering advances RandomSeeds1/2 (Source/singlescattering.cuh:27-32);
   d_frame_xyza receives W*H float4. */
ER_API er_status er_trace_frame_device(int32_t tracer_id, uint32_t* d_lanes, float* d_frame_xyza, void* stream);

/* Post-process stages on caller buffers (W*H pixels):
   3x3 Gaussian of a float4 image (Source/filterframeestimate.cuh:33-64) fused
   with the running average R += (F-R)/max(n,1) (Source/estimate.cuh:27-38)
   and the tone map (Source/tonemap.cuh:30-59). */
ER_API er_status er_post_frame_device(const float* d_frame_xyza, float* d_running_xyza, uint8_t* d_rgba,
                                      int32_t width, int32_t height, int32_t no_iterations, float exposure,
                                      int32_t frame_filter, void* stream);
/* Tone map only (Source/tonemap.cuh:30-59): float4 XYZA scaled by `scale` -> RGBA8. */
ER_API er_status er_tonemap_device(const float* d_xyza, float scale, uint8_t* d_rgba, int32_t width, int32_t height,
                                   float exposure, void* stream);
/* Separable bilateral filter on RGBA8 (design of Source/filterrunningestimate.cuh:35-200):
   horizontal pass into d_tmp, vertical pass into d_out. */
ER_API er_status er_bilateral_device(const uint8_t* d_in, uint8_t* d_tmp, uint8_t* d_out, int32_t width, int32_t height,
                                     int32_t radius, float sigma_d, float sigma_r, void* stream);

/* Gradient-magnitude pre-pass of a bound volume (Source/gradientmagnitude.cuh:28-71
   with the per-voxel magnitude of Source/volumes.h:93-114 at voxel centres):
   optional u16 magnitude volume (saturating) and the maximum magnitude. */
ER_API er_status er_gradient_magnitude(int32_t volume_id, uint16_t* d_gm_or_null, float* max_gradient_magnitude);

/* Majorant grid of the delta tracker for caller-owned device buffers:
   d_voxels (x-fastest uint16, resolution[0]*[1]*[2]), d_sigma (sigma_count
   floats, sigma[I] = density_scale * Opacity(I), covering every voxel value),
   d_majorant receives ceil(res/brick) per axis floats, x fastest:
   density_scale * max sigma[lo - 1 .. hi], lo and hi the smallest and largest
   voxel of the brick's footprint (voxels b*brick .. (b+1)*brick per axis,
   the corners a lookup clamped to the brick blends; lo - 1 because the
   truncated blend can round to one below its smallest corner).
   The design precedent is the commented macrocell tracker of
   Source/raymarching.h:115-273 (per-cell maximum extinction).  Scratch space
   (per-brick min/max, range-max table) is allocated by the library. */
ER_API er_status er_build_majorant_device(const uint16_t* d_voxels, const int32_t resolution[3], int32_t brick, const float* d_sigma,
                                          int32_t sigma_count, float density_scale, float* d_majorant, void* stream);

/* Allocation-free variant of er_build_majorant_device, for callers that
   cannot allocate device memory where they rebuild the grid (inside a frame
   loop, where cudaMalloc/cudaFree would synchronise the device, or under a
   host-owned pool allocator).  Same arguments and result; the scratch lives
   in static device arrays sized for at most 2^20 bricks and 65536 sigma
   entries (8.25 MiB per GPU, held until exit); larger inputs are rejected
   with ER_ERR_INVALID_ARGUMENT.  The first call on a device resolves the
   arrays' addresses (make it before any stream capture), and the first call
   after the device's context was replaced (cudaDeviceReset) resolves them
   again; calls that overlap on the GPU share the arrays and race.  No
   counterpart in the reference. */
ER_API er_status er_build_majorant_device_noalloc(const uint16_t* d_voxels, const int32_t resolution[3], int32_t brick,
                                                  const float* d_sigma, int32_t sigma_count, float density_scale, float* d_majorant,
                                                  void* stream);

/* Diagnostics: evaluates one include/er_math.h function on the GPU for n
   arguments (fn 0 log, 1 exp, 2 sin, 3 cos, 4 tan, 5 pow(x,y), 6 acos,
   7 atan2(x,y)); used to check that device and host produce the same bits.
   No reference counterpart. */
ER_API er_status er_math_eval_device(int32_t fn, int32_t n, const float* d_x, const float* d_y, float* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ER_CAPI_H */
