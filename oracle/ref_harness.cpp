/*
 * ref_harness.cpp - runs the reference's own transport and post-processing
 * code on the host (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/Makefile against the unmodified headers in the reference's
 * Source/ directory (with oracle/ref_shim/er_ref_prelude.h force-included)
 * into oracle/_ref/liberref.so.  It exports the oracle API of
 * oracle/er_oracle.h with the prefix ref_, so the tests can run the
 * restatement (or_) and the reference (ref_) on the same input.
 *
 * Kernels: the .cuh files define their kernels with KERNEL (empty on the
 * host) and index pixels through blockIdx/blockDim/threadIdx (KERNEL_2D,
 * Source/macros.cuh:83-90).  This file provides host stand-ins for those
 * three variables and neutralises the launch macros, so KrnlSingleScattering,
 * KrnlFilterFrameEstimate, KrnlComputeEstimate and KrnlToneMap run as plain
 * functions, one call per pixel.
 *
 * Scene set-up follows the reference's bind path: ErVolume::BindVoxels
 * (Source/ervolume.h:63-69) then Volume = ErVolume (Source/volume.h:100-129),
 * Light = ErLight (Source/light.h:39-45), Texture = ErTexture, Tracer =
 * ErTracer (Source/tracer.h:45-52).  Buffers whose MemoryType the reference
 * sets to Device are switched to Host before they are sized, because the host
 * build never allocates device memory (Source/buffer2d.h:155-161).
 */
#include "er_oracle.h"

#include <pthread.h>
#include <vector>

struct er_ref_dim3 { unsigned int x, y, z; };
static thread_local er_ref_dim3 blockIdx, blockDim, threadIdx;

#include "macros.cuh"
#undef LAUNCH_CUDA_KERNEL_TIMED
#define LAUNCH_CUDA_KERNEL_TIMED(call, title)
#undef LAUNCH_CUDA_KERNEL
#define LAUNCH_CUDA_KERNEL(call)

#include "tracer.h"
#include "volume.h"
#include "light.h"
#include "object.h"
#include "clippingobject.h"
#include "texture.h"
#include "bitmap.h"

/* Source/core.cu:30-36 without DEVICE */
ExposureRender::Tracer* gpTracer = NULL;
ExposureRender::Volume* gpVolumes = NULL;
ExposureRender::Light* gpLights = NULL;
ExposureRender::Object* gpObjects = NULL;
ExposureRender::ClippingObject* gpClippingObjects = NULL;
ExposureRender::Texture* gpTextures = NULL;
ExposureRender::Bitmap* gpBitmaps = NULL;

#include "singlescattering.cuh"
#include "filterframeestimate.cuh"
#include "estimate.cuh"
#include "tonemap.cuh"

using namespace ExposureRender;

#define MAX_NO_INDICES_HARNESS 256

struct or_scene {
    ErVolume* ervolume;
    Volume* volume;
    std::vector<Light> lights;
    std::vector<Texture> textures;
    std::vector<Object> objects;
    std::vector<Bitmap> bitmaps;
    Tracer* tracer;
    int W, H;
    uint32_t seed;
};

static void set_plf(PiecewiseLinearFunction<MAX_NO_TF_NODES>& plf, const er_plf& d)
{
    for (int i = 0; i < d.count; i++) plf.AddNode(d.position[i], d.value[i]);
}

static void set_ctf(ColorTransferFunction1D& tf, const er_color_tf& d)
{
    for (int c = 0; c < 3; c++) set_plf(tf.PLF[c], d.plf[c]);
}

static void set_shape(Shape& s, const er_shape& d)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            s.TM.NN[i][j] = d.tm[i][j];
            s.InvTM.NN[i][j] = d.inv_tm[i][j];
        }
    s.OneSided = d.one_sided != 0;
    s.Type = (Enums::ShapeType)d.type;
    s.Size = Vec3f(d.size[0], d.size[1], d.size[2]);
    s.InnerRadius = d.inner_radius;
    s.OuterRadius = d.outer_radius;
    s.Area = d.area;
}

extern "C" or_scene* ref_scene_create(const er_tracer_desc* t, const er_volume_desc* vd, const er_light_desc* lights,
                                      int32_t n_lights, const er_texture_desc* textures, int32_t n_textures)
{
    or_scene* s = new or_scene();
    /* BindVolume */
    s->ervolume = new ErVolume();
    s->ervolume->BindVoxels(Vec3i(vd->resolution[0], vd->resolution[1], vd->resolution[2]),
                            Vec3f(vd->spacing[0], vd->spacing[1], vd->spacing[2]),
                            (unsigned short*)vd->voxels, vd->normalize_size != 0);
    s->volume = new Volume();
    s->volume->Voxels.MemoryType = Enums::Host;
    *s->volume = *s->ervolume;
    /* BindLight */
    for (int i = 0; i < n_lights; i++) {
        ErLight el;
        el.Visible = lights[i].visible != 0;
        set_shape(el.Shape, lights[i].shape);
        el.TextureID = lights[i].texture_id;
        el.Multiplier = lights[i].multiplier;
        el.Unit = (Enums::EmissionUnit)lights[i].unit;
        s->lights.push_back(Light(el));
    }
    /* BindTexture */
    for (int i = 0; i < n_textures; i++) {
        ErTexture et;
        et.Type = (Enums::TextureType)textures[i].type;
        et.OutputLevel = textures[i].output_level;
        et.BitmapID = textures[i].bitmap_id;
        et.Procedural.Type = (Enums::ProceduralType)textures[i].procedural.type;
        et.Procedural.UniformColor = ColorXYZf(textures[i].procedural.uniform_color[0], textures[i].procedural.uniform_color[1],
                                               textures[i].procedural.uniform_color[2]);
        et.Procedural.CheckerColor1 = ColorXYZf(textures[i].procedural.checker_color1[0], textures[i].procedural.checker_color1[1],
                                                textures[i].procedural.checker_color1[2]);
        et.Procedural.CheckerColor2 = ColorXYZf(textures[i].procedural.checker_color2[0], textures[i].procedural.checker_color2[1],
                                                textures[i].procedural.checker_color2[2]);
        set_ctf(et.Procedural.Gradient, textures[i].procedural.gradient);
        et.Offset = Vec2f(textures[i].offset[0], textures[i].offset[1]);
        et.Repeat = Vec2f(textures[i].repeat[0], textures[i].repeat[1]);
        et.Flip = Vec2i(textures[i].flip[0], textures[i].flip[1]);
        s->textures.push_back(Texture(et));
    }
    /* BindTracer */
    ErTracer et;
    set_plf(et.Opacity1D.PLF, t->opacity);
    set_ctf(et.Diffuse1D, t->diffuse);
    set_ctf(et.Specular1D, t->specular);
    set_plf(et.Glossiness1D.PLF, t->glossiness);
    set_ctf(et.Emission1D, t->emission);
    Camera cam;
    cam.FilmSize = Vec2i(t->camera.film_size[0], t->camera.film_size[1]);
    cam.Pos = Vec3f(t->camera.pos[0], t->camera.pos[1], t->camera.pos[2]);
    cam.Target = Vec3f(t->camera.target[0], t->camera.target[1], t->camera.target[2]);
    cam.Up = Vec3f(t->camera.up[0], t->camera.up[1], t->camera.up[2]);
    cam.FocalDistance = t->camera.focal_distance;
    cam.ApertureSize = t->camera.aperture_size;
    cam.ClipNear = t->camera.clip_near;
    cam.ClipFar = t->camera.clip_far;
    cam.Exposure = t->camera.exposure;
    cam.Gamma = t->camera.gamma;
    cam.FOV = t->camera.fov;
    et.Camera = cam;
    et.RenderSettings.Traversal.StepFactorPrimary = t->settings.step_factor_primary;
    et.RenderSettings.Traversal.StepFactorShadow = t->settings.step_factor_shadow;
    et.RenderSettings.Traversal.Shadows = t->settings.shadows != 0;
    et.RenderSettings.Traversal.MaxShadowDistance = t->settings.max_shadow_distance;
    et.RenderSettings.Shading.Type = t->settings.shading_type;
    et.RenderSettings.Shading.DensityScale = t->settings.density_scale;
    et.RenderSettings.Shading.OpacityModulated = t->settings.opacity_modulated != 0;
    et.RenderSettings.Shading.GradientComputation = t->settings.gradient_computation;
    et.RenderSettings.Shading.GradientThreshold = t->settings.gradient_threshold;
    et.RenderSettings.Shading.GradientFactor = t->settings.gradient_factor;
    et.NoIterations = 0;
    et.VolumeID = 0;
    for (int i = 0; i < t->light_count; i++) et.LightIDs[i] = t->light_ids[i];
    et.LightIDs.Count = t->light_count;
    for (int i = 0; i < t->object_count && i < MAX_NO_INDICES_HARNESS; i++) et.ObjectIDs[i] = t->object_ids[i];
    et.ObjectIDs.Count = t->object_count;
    et.ClippingObjectIDs.Count = 0;

    s->tracer = new Tracer();
    FrameBuffer& fb = s->tracer->FrameBuffer;
    fb.FrameEstimate.MemoryType = Enums::Host;
    fb.FrameEstimateTemp.MemoryType = Enums::Host;
    fb.RunningEstimateXyza.MemoryType = Enums::Host;
    fb.DisplayEstimate.MemoryType = Enums::Host;
    fb.DisplayEstimateTemp.MemoryType = Enums::Host;
    fb.DisplayEstimateFiltered.MemoryType = Enums::Host;
    fb.RandomSeeds1.MemoryType = Enums::Host;
    fb.RandomSeeds2.MemoryType = Enums::Host;
    fb.RandomSeedsCopy1.MemoryType = Enums::Host;
    fb.RandomSeedsCopy2.MemoryType = Enums::Host;
    *s->tracer = et;
    s->W = t->camera.film_size[0];
    s->H = t->camera.film_size[1];
    s->seed = t->settings.seed;

    gpTracer = s->tracer;
    gpVolumes = s->volume;
    gpLights = s->lights.empty() ? NULL : &s->lights[0];
    gpTextures = s->textures.empty() ? NULL : &s->textures[0];
    gpObjects = s->objects.empty() ? NULL : &s->objects[0];
    gpClippingObjects = NULL;
    gpBitmaps = NULL;
    return s;
}

extern "C" void ref_scene_destroy(or_scene* s)
{
    if (!s) return;
    if (gpTracer == s->tracer) {
        gpTracer = NULL; gpVolumes = NULL; gpLights = NULL; gpTextures = NULL; gpObjects = NULL; gpBitmaps = NULL;
    }
    delete s->tracer;
    delete s->volume;
    delete s->ervolume;
    delete s;
}

static void bind_scene(or_scene* s)
{
    gpTracer = s->tracer;
    gpVolumes = s->volume;
    gpLights = s->lights.empty() ? NULL : &s->lights[0];
    gpTextures = s->textures.empty() ? NULL : &s->textures[0];
    gpObjects = s->objects.empty() ? NULL : &s->objects[0];
    gpBitmaps = s->bitmaps.empty() ? NULL : &s->bitmaps[0];
}

/* BindBitmap: bitmap i is the i-th entry of gpBitmaps.  The Bitmap records
   are sized first and switched to host memory before the ErBitmap is
   assigned (device buffers are not allocated in a host build,
   Source/buffer2d.h:118-131). */
extern "C" void ref_scene_set_bitmaps(or_scene* s, const er_bitmap_desc* bitmaps, int32_t n)
{
    s->bitmaps.clear();
    s->bitmaps.resize((size_t)(n > 0 ? n : 0));
    for (int i = 0; i < n; i++) {
        ErBitmap eb;
        eb.BindPixels(Vec2i(bitmaps[i].resolution[0], bitmaps[i].resolution[1]), (ColorRGBAuc*)bitmaps[i].pixels);
        s->bitmaps[i].Pixels.MemoryType = Enums::Host;
        s->bitmaps[i] = eb;
    }
    bind_scene(s);
}

/* BindObject: object i is the i-th entry of gpObjects */
extern "C" void ref_scene_set_objects(or_scene* s, const er_object_desc* objects, int32_t n)
{
    s->objects.clear();
    for (int i = 0; i < n; i++) {
        ErObject eo;
        set_shape(eo.Shape, objects[i].shape);
        eo.DiffuseTextureID = objects[i].diffuse_texture_id;
        eo.SpecularTextureID = objects[i].specular_texture_id;
        eo.GlossinessTextureID = objects[i].glossiness_texture_id;
        eo.Ior = objects[i].ior;
        s->objects.push_back(Object(eo));
    }
    bind_scene(s);
}

/* one KERNEL_2D "thread" for pixel (x, y) with a 16x8 block, as the launch of
   SingleScattering(Tracer&) (Source/singlescattering.cuh:34-38) */
static inline void set_thread(int x, int y, int bw, int bh)
{
    blockDim.x = bw; blockDim.y = bh; blockDim.z = 1;
    blockIdx.x = x / bw; blockIdx.y = y / bh; blockIdx.z = 0;
    threadIdx.x = x % bw; threadIdx.y = y % bh; threadIdx.z = 0;
}

struct ref_job {
    or_scene* s;
    int mode;
    uint32_t* lanes;
    float* out;
    int spp;
    uint32_t view, first, seed;
    int x0, y0, w, h, row0, row1;
};

static void* ref_job_run(void* arg)
{
    ref_job* j = (ref_job*)arg;
    or_scene* s = j->s;
    FrameBuffer& fb = s->tracer->FrameBuffer;
    const int W = s->W, H = s->H;
    for (int r = j->row0; r < j->row1; r++) {
        if (j->mode == 0) {
            for (int x = 0; x < W; x++) {
                const size_t p = (size_t)r * W + x;
                fb.RandomSeeds1(x, r) = j->lanes[p];
                fb.RandomSeeds2(x, r) = j->lanes[(size_t)W * H + p];
                set_thread(x, r, 16, 8);
                KrnlSingleScattering();
                const ColorXYZAf& F = fb.FrameEstimate(x, r);
                for (int k = 0; k < 4; k++) j->out[4 * p + k] = F[k];
                j->lanes[p] = fb.RandomSeeds1(x, r);
                j->lanes[(size_t)W * H + p] = fb.RandomSeeds2(x, r);
            }
        } else {
            const int y = j->y0 + r;
            for (int xi = 0; xi < j->w; xi++) {
                const int x = j->x0 + xi;
                const uint32_t pix = (uint32_t)y * (uint32_t)W + (uint32_t)x;
                float acc[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
                for (int k = 0; k < j->spp; k++) {
                    uint32_t l0, l1;
                    er_seed_lanes(j->seed, j->view, pix, j->first + (uint32_t)k, &l0, &l1);
                    fb.RandomSeeds1(x, y) = l0;
                    fb.RandomSeeds2(x, y) = l1;
                    const ColorXYZAf o = SingleScattering(gpTracer, Vec2i(x, y));
                    for (int c = 0; c < 4; c++) acc[c] += o[c];
                }
                float* d = &j->out[4 * ((size_t)r * j->w + xi)];
                for (int c = 0; c < 4; c++) d[c] = acc[c];
            }
        }
    }
    return NULL;
}

static void ref_run(ref_job* proto, int rows, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > rows) nthreads = rows > 0 ? rows : 1;
    std::vector<ref_job> jobs(nthreads, *proto);
    std::vector<pthread_t> th(nthreads);
    for (int t = 0; t < nthreads; t++) {
        jobs[t].row0 = (int)((long long)rows * t / nthreads);
        jobs[t].row1 = (int)((long long)rows * (t + 1) / nthreads);
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, ref_job_run, &jobs[t]);
    ref_job_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
}

extern "C" void ref_render_frame(or_scene* s, uint32_t* lanes, float* frame, int32_t nthreads)
{
    bind_scene(s);
    ref_job proto = {};
    proto.s = s; proto.mode = 0; proto.lanes = lanes; proto.out = frame;
    ref_run(&proto, s->H, nthreads);
}

extern "C" void ref_render_sum(or_scene* s, int32_t spp, uint32_t view, uint32_t first_sample, int32_t x0, int32_t y0,
                               int32_t w, int32_t h, float* sum, int32_t nthreads)
{
    bind_scene(s);
    ref_job proto = {};
    proto.s = s; proto.mode = 1; proto.out = sum; proto.spp = spp; proto.view = view; proto.first = first_sample;
    /* the reference tracer has no seed field; the counter-based seed comes
       from the descriptor's settings.seed, as in the restatement */
    proto.seed = s->seed; proto.x0 = x0; proto.y0 = y0; proto.w = w; proto.h = h;
    ref_run(&proto, h, nthreads);
}

/* RenderEstimate after the transport kernel (Source/core.cu:130-135), on the
   caller's buffers: the reference kernels read/write the tracer's frame
   buffer, so the buffers are copied in and out around the per-pixel calls. */
extern "C" void ref_post_frame(float* frame, float* running, uint8_t* rgba, int32_t W, int32_t H, int32_t no_iterations,
                               float exposure)
{
    ErTracer et;
    Camera cam;
    cam.FilmSize = Vec2i(W, H);
    cam.Pos = Vec3f(0.0f, 0.0f, -1.0f);
    cam.Target = Vec3f(0.0f);
    cam.Up = Vec3f(0.0f, 1.0f, 0.0f);
    cam.FocalDistance = 1.0f; cam.ApertureSize = 0.0f; cam.ClipNear = 0.0f; cam.ClipFar = 1.0f;
    cam.Exposure = exposure; cam.Gamma = 2.2f; cam.FOV = 35.0f;
    et.Camera = cam;
    et.NoIterations = no_iterations;
    Tracer* T = new Tracer();
    FrameBuffer& fb = T->FrameBuffer;
    fb.FrameEstimate.MemoryType = Enums::Host;
    fb.FrameEstimateTemp.MemoryType = Enums::Host;
    fb.RunningEstimateXyza.MemoryType = Enums::Host;
    fb.DisplayEstimate.MemoryType = Enums::Host;
    fb.DisplayEstimateTemp.MemoryType = Enums::Host;
    fb.DisplayEstimateFiltered.MemoryType = Enums::Host;
    fb.RandomSeeds1.MemoryType = Enums::Host;
    fb.RandomSeeds2.MemoryType = Enums::Host;
    fb.RandomSeedsCopy1.MemoryType = Enums::Host;
    fb.RandomSeedsCopy2.MemoryType = Enums::Host;
    *T = et;
    Tracer* saved = gpTracer;
    gpTracer = T;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int k = 0; k < 4; k++) {
                fb.FrameEstimate(x, y)[k] = frame[4 * ((size_t)y * W + x) + k];
                fb.RunningEstimateXyza(x, y)[k] = running[4 * ((size_t)y * W + x) + k];
            }
    /* FilterFrameEstimate (Source/filterframeestimate.cuh:66-74), 8x8 blocks */
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) { set_thread(x, y, 8, 8); KrnlFilterFrameEstimate(1, 1.0f); }
    fb.FrameEstimateTemp.Dirty = true;
    fb.FrameEstimate = fb.FrameEstimateTemp;
    /* ComputeEstimate (Source/estimate.cuh:34-38) */
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) { set_thread(x, y, 16, 8); KrnlComputeEstimate(); }
    /* ToneMap (Source/tonemap.cuh:61-65) */
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) { set_thread(x, y, 16, 8); KrnlToneMap(); }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            for (int k = 0; k < 4; k++) {
                frame[4 * ((size_t)y * W + x) + k] = fb.FrameEstimate(x, y)[k];
                running[4 * ((size_t)y * W + x) + k] = fb.RunningEstimateXyza(x, y)[k];
                rgba[4 * ((size_t)y * W + x) + k] = fb.DisplayEstimate(x, y)[k];
            }
        }
    gpTracer = saved;
    delete T;
}

extern "C" double ref_lookups_per_sample(void) { return 0.0; }

extern "C" void ref_rng_draws(uint32_t lane0, uint32_t lane1, int32_t n, float* out)
{
    unsigned int a = lane0, b = lane1;
    CRNG r(&a, &b);
    for (int i = 0; i < n; i++) out[i] = r.Get1();
}

extern "C" void ref_rng_get2_get3(uint32_t lane0, uint32_t lane1, float* out5)
{
    unsigned int a = lane0, b = lane1;
    CRNG r(&a, &b);
    const Vec2f v2 = r.Get2();
    const Vec3f v3 = r.Get3();
    out5[0] = v2[0]; out5[1] = v2[1]; out5[2] = v3[0]; out5[3] = v3[1]; out5[4] = v3[2];
}

extern "C" void ref_plf_evaluate(const er_plf* plf, int32_t n, const float* x, float* y)
{
    ScalarTransferFunction1D tf;
    set_plf(tf.PLF, *plf);
    for (int i = 0; i < n; i++) y[i] = tf.Evaluate(x[i]);
}

extern "C" void ref_get_intensity(or_scene* s, int32_t n, const float* p, float* out)
{
    bind_scene(s);
    for (int i = 0; i < n; i++) out[i] = GetIntensity(0, Vec3f(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
}

extern "C" void ref_normalized_gradient(or_scene* s, int32_t n, const float* p, float* out)
{
    bind_scene(s);
    for (int i = 0; i < n; i++) {
        const Vec3f g = NormalizedGradient(0, Vec3f(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
        out[3 * i] = g[0]; out[3 * i + 1] = g[1]; out[3 * i + 2] = g[2];
    }
}

extern "C" void ref_gradient_magnitude(or_scene* s, int32_t n, const float* p, float* out)
{
    bind_scene(s);
    for (int i = 0; i < n; i++) out[i] = GradientMagnitude(0, Vec3f(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
}

extern "C" void ref_intersect_volume_box(or_scene* s, int32_t n, const float* r8, float* out3)
{
    bind_scene(s);
    for (int i = 0; i < n; i++) {
        Ray R(Vec3f(r8[8 * i], r8[8 * i + 1], r8[8 * i + 2]), Vec3f(r8[8 * i + 3], r8[8 * i + 4], r8[8 * i + 5]),
              r8[8 * i + 6], r8[8 * i + 7]);
        Intersection Int;
        IntersectBox(R, gpVolumes[0].BoundingBox.MinP, gpVolumes[0].BoundingBox.MaxP, Int);
        out3[3 * i] = Int.Valid ? 1.0f : 0.0f;
        out3[3 * i + 1] = Int.NearT;
        out3[3 * i + 2] = Int.FarT;
    }
}

extern "C" void ref_concentric_sample_disk(int32_t n, const float* u2, float* out2)
{
    for (int i = 0; i < n; i++) {
        const Vec2f d = ConcentricSampleDisk(Vec2f(u2[2 * i], u2[2 * i + 1]));
        out2[2 * i] = d[0]; out2[2 * i + 1] = d[1];
    }
}

extern "C" void ref_tonemap(int32_t n, const float* xyza, float exposure, uint8_t* rgba)
{
    ErTracer et;
    Camera cam;
    cam.FilmSize = Vec2i(1, 1);
    cam.Pos = Vec3f(0.0f, 0.0f, -1.0f); cam.Target = Vec3f(0.0f); cam.Up = Vec3f(0.0f, 1.0f, 0.0f);
    cam.FocalDistance = 1.0f; cam.ApertureSize = 0.0f; cam.ClipNear = 0.0f; cam.ClipFar = 1.0f;
    cam.Exposure = exposure; cam.Gamma = 2.2f; cam.FOV = 35.0f;
    et.Camera = cam;
    Tracer T;
    T.ErTracer::operator=(et);
    Tracer* saved = gpTracer;
    gpTracer = &T;
    for (int i = 0; i < n; i++) {
        const ColorRGBuc c = ToneMap(ColorXYZAf(xyza[4 * i], xyza[4 * i + 1], xyza[4 * i + 2], xyza[4 * i + 3]));
        rgba[4 * i] = c[0]; rgba[4 * i + 1] = c[1]; rgba[4 * i + 2] = c[2];
        rgba[4 * i + 3] = (unsigned char)(xyza[4 * i + 3] * 255.0f);
    }
    gpTracer = saved;
}

extern "C" void ref_camera_ray(or_scene* s, int32_t x, int32_t y, const float* uv4, float* out6)
{
    bind_scene(s);
    CameraSample cs;
    cs.FilmUV = Vec2f(uv4[0], uv4[1]);
    cs.LensUV = Vec2f(uv4[2], uv4[3]);
    Ray R;
    SampleCamera(gpTracer->Camera, R, x, y, cs);
    out6[0] = R.O[0]; out6[1] = R.O[1]; out6[2] = R.O[2]; out6[3] = R.D[0]; out6[4] = R.D[1]; out6[5] = R.D[2];
}

extern "C" void ref_camera_frame(or_scene* s, float* o)
{
    const Camera& c = s->tracer->Camera;
    o[0] = c.N[0]; o[1] = c.N[1]; o[2] = c.N[2];
    o[3] = c.U[0]; o[4] = c.U[1]; o[5] = c.U[2];
    o[6] = c.V[0]; o[7] = c.V[1]; o[8] = c.V[2];
    o[9] = c.Screen[0][0]; o[10] = c.Screen[0][1]; o[11] = c.Screen[1][0]; o[12] = c.Screen[1][1];
    o[13] = c.InvScreen[0]; o[14] = c.InvScreen[1];
}

extern "C" void ref_volume_frame(or_scene* s, float* o)
{
    const Volume& v = *s->volume;
    o[0] = v.BoundingBox.MinP[0]; o[1] = v.BoundingBox.MinP[1]; o[2] = v.BoundingBox.MinP[2];
    o[3] = v.InvSize[0]; o[4] = v.InvSize[1]; o[5] = v.InvSize[2];
    o[6] = v.MinStep;
    o[7] = v.Spacing[0]; o[8] = v.Spacing[1]; o[9] = v.Spacing[2];
    o[10] = v.Size[0]; o[11] = v.Size[1]; o[12] = v.Size[2];
}
