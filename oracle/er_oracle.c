/*
 * er_oracle.c - CPU oracle: a plain-C restatement of Exposure Render's
 * single-scattering transport path and post-processing.
 *
 * TEST INFRASTRUCTURE ONLY (see er_oracle.h).  The product never calls this.
 *
 * Every function cites the reference file:line it restates (paths relative
 * to the reference project).  Floating-point expressions keep the
 * reference's evaluation order (C++ operators are left-associative and the
 * Vec/Color operators of Source/vector.h and Source/color.h work
 * component-wise), and the file must be compiled with -ffp-contract=off so
 * that no multiply-add is fused.  Elementary functions come from
 * include/er_math.h; the reference build in oracle/_ref routes its
 * logf/expf/powf/sinf/cosf/tanf/acosf/atan2f calls to the same functions.
 *
 * std::min/std::max (the reference's `using namespace std`) are
 * (b < a) ? b : a and (a < b) ? b : a; ExposureRender::Min/Max/Clamp
 * (Source/vector.h:27-43) are A < B ? A : B, A > B ? A : B and
 * Max(lo, Min(v, hi)); fminf/fmaxf are the IEEE functions.
 */
#include "er_capi.h"
#include "er_math.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* a float field of an er_capi.h descriptor (stays float in the FP64 build) */
typedef float desc_f32;

#ifdef ER_ORACLE_FP64
/* FP64 oracle build: every float of the restatement (and of er_oracle.h,
   included below) is a double, and the elementary functions are the C
   library's double functions.  The descriptors of er_capi.h keep their
   float fields (included above); the RNG keeps its 23-bit uniforms. */
#define float double
#define sqrtf sqrt
#define fabsf fabs
#define floorf floor
#define ceilf ceil
#define fminf fmin
#define fmaxf fmax
#define er_logf log
#define er_expf exp
#define er_powf pow
#define er_sinf sin
#define er_cosf cos
#define er_tanf tan
#define er_acosf acos
#define er_atan2f atan2
#define er_sincosf(x, s, c) (*(s) = sin(x), *(c) = cos(x))
#endif

#include "er_oracle.h"

/* ------------------------------------------------------------------ */
/* small vector algebra (Source/vector.h:397-552)                       */
/* ------------------------------------------------------------------ */

typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;
typedef struct { float c[3]; } col3;   /* ColorXYZf */

static inline v3 V3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdivv(v3 a, v3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 vscale(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 vneg(v3 a) { return V3(-a.x, -a.y, -a.z); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }               /* :477-480 */
static inline float vlen2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }                     /* :459-462 */
static inline float vlen(v3 a) { return sqrtf(vlen2(a)); }                                        /* :464-467 */
static inline v3 vnorm(v3 a) { const float L = vlen(a); return V3(a.x / L, a.y / L, a.z / L); }   /* :469-475 */
static inline v3 vcross(v3 a, v3 b)                                                               /* :482-485 */
{
    return V3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
static inline float vabsdot(v3 a, v3 b) { return fabsf(vdot(a, b)); }                           /* :547 */
static inline float vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

static inline float smin(float a, float b) { return (b < a) ? b : a; }   /* std::min */
static inline float smax(float a, float b) { return (a < b) ? b : a; }   /* std::max */
static inline float emin(float a, float b) { return a < b ? a : b; }     /* ExposureRender::Min */
static inline float emax(float a, float b) { return a > b ? a : b; }     /* ExposureRender::Max */
static inline float eclamp(float v, float lo, float hi) { return emax(lo, emin(v, hi)); }
static inline int iclamp(int v, int lo, int hi) { int m = v < hi ? v : hi; return lo > m ? lo : m; }

static inline col3 C3(float a, float b, float c) { col3 r; r.c[0] = a; r.c[1] = b; r.c[2] = c; return r; }
static inline col3 cadd(col3 a, col3 b) { return C3(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
static inline col3 csub(col3 a, col3 b) { return C3(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]); }
static inline col3 cmul(col3 a, col3 b) { return C3(a.c[0] * b.c[0], a.c[1] * b.c[1], a.c[2] * b.c[2]); }
static inline col3 cdiv(col3 a, col3 b) { return C3(a.c[0] / b.c[0], a.c[1] / b.c[1], a.c[2] / b.c[2]); }
static inline col3 cscale(col3 a, float s) { return C3(a.c[0] * s, a.c[1] * s, a.c[2] * s); }
static inline col3 cdivs(col3 a, float s) { return C3(a.c[0] / s, a.c[1] / s, a.c[2] / s); }
static inline int cblack(col3 a) { return a.c[0] == 0.0f && a.c[1] == 0.0f && a.c[2] == 0.0f; }  /* Source/color.h:27-35 */

#define PI_F 3.141592654f                      /* Source/defines.h:58 */
#define INV_PI_F 0.31830988618379067154f       /* :62 */
#define INV_TWO_PI_F 0.15915494309189533577f   /* :63 */
#define RAY_EPS 0.0001f                        /* :71 */
/* INV_FOUR_PI_F expands to 1.0f / 4.0f * PI_F (:64-65), i.e. pi/4 */
#define INV_FOUR_PI_EXPANDED (1.0f / 4.0f * PI_F)

/* ------------------------------------------------------------------ */
/* scene                                                                */
/* ------------------------------------------------------------------ */

typedef struct {
    er_light_desc d;
    float area;
} or_light;

struct or_scene {
    /* Volume (Source/volume.h:100-149) */
    const uint16_t* vox;
    int res[3];
    v3 minp;
    v3 inv_size;
    v3 size;
    v3 spacing;
    float min_step;
    v3 gdx, gdy, gdz;
    /* Camera (Source/camera.h:61-116) */
    int film[2];
    v3 pos, N, U, V;
    float screen[2][2];
    float inv_screen[2];
    float clip_near, clip_far, aperture, focal_distance, exposure;
    /* tracer */
    er_render_settings st;
    er_plf opacity, glossiness;
    er_color_tf diffuse, specular, emission;
    int light_count;
    int light_idx[ER_MAX_INDICES];
    int n_lights;
    or_light* lights;
    int n_textures;
    er_texture_desc* textures;
    /* surface objects: the tracer's ObjectIDs.Count and the bound objects in
       device-array order (IntersectObjects indexes gpObjects[i] by the loop
       index, Source/objects.h:52) */
    int object_count;
    int n_objects;
    er_object_desc* objects;
    /* bitmaps (gpBitmaps in device-array order, ErTexture::BitmapID indexes
       it, Source/textures.h:101-107): RGBA8 row-major */
    int n_bitmaps;
    int* bitmap_res;            /* 2 per bitmap */
    uint8_t** bitmap_pixels;
    /* clipping objects named by the tracer's ClippingObjectIDs, resolved
       (scene_set_clipping_objects) */
    int n_clips;
    er_clipping_object_desc* clips;
    int clip_ids_count;
    int clip_ids[ER_MAX_INDICES];
    /* the stratified first free-flight draw of the current sample, or < 0 */
    float tau_u;
    /* statistics */
    uint64_t lookups;
    uint64_t stat[OR_NSTATS];   /* work counters of the last render (render_stats) */
    uint64_t samples;
    /* extension estimators (see er_capi.h): sigma table over integer
       intensities, majorant grid of the delta tracker, 1 / max |grad I| */
    uint16_t vmax;
    float* sigma;            /* DensityScale * Opacity(I), I in [0, vmax] */
    int brick;
    int nb[3];
    float* majorant;         /* per brick: DensityScale * max sigma over the brick footprint */
    float gm_inv_max;
    int gm_ready;
    /* differentiable medium (dm_attach): float density grid, cubic B-spline
       opacity over density, albedo, NEE probability; the majorant grid above
       is the caller's fixed grid */
    const float* rho;
    const float* tf_val;
    int tf_n;
    float dm_scale;
    col3 dm_albedo;
    float dm_q;
    /* dm_set_model: 0 the B-spline opacity and isotropic albedo above; 1 the
       tracer's transfer functions and shading, with tf_val the values of the
       tracer's opacity nodes (at its node positions) */
    int dm_model;
    int dm_emissive;          /* model 1: the emission TF is not zero everywhere */
    float dm_gm_inv;          /* model 1, hybrid shading: 1 / gradient-magnitude range (a fixed constant) */
};

static double g_lookups_per_sample = 0.0;
static double g_stats[OR_NSTATS];
static void prepare_extensions(or_scene* s);
static int clipped(const or_scene* s, v3 p);

/* Shape::Update (Source/shape.h:92-103) with the area helpers :27-55 */
static float shape_area(const er_shape* s)
{
    switch (s->type) {
    case ER_SHAPE_PLANE: return s->size[0] * s->size[1];
    case ER_SHAPE_DISK: return PI_F * (s->outer_radius * s->outer_radius);
    case ER_SHAPE_RING: return PI_F * (s->outer_radius * s->outer_radius) - PI_F * (s->inner_radius * s->inner_radius);
    case ER_SHAPE_BOX: return (2.0f * s->size[0] * s->size[1]) + (2.0f * s->size[0] * s->size[2]) + (2.0f * s->size[1] * s->size[2]);
    case ER_SHAPE_SPHERE: return 4.0f * PI_F * (s->outer_radius * s->outer_radius);
    case ER_SHAPE_CYLINDER: return (2.0f * PI_F * (s->outer_radius * s->outer_radius)) + (2.0f * PI_F * s->outer_radius * s->size[2]);
    default: return s->area;   /* Update() leaves Area untouched for other types */
    }
}

or_scene* ER_OR(scene_create)(const er_tracer_desc* t, const er_volume_desc* vol,
                              const er_light_desc* lights, int32_t n_lights,
                              const er_texture_desc* textures, int32_t n_textures)
{
    or_scene* s = (or_scene*)calloc(1, sizeof(or_scene));
    if (!s) return NULL;
    /* Volume::operator=(const ErVolume&) - Source/volume.h:100-129 */
    s->vox = vol->voxels;
    for (int i = 0; i < 3; i++) s->res[i] = vol->resolution[i];
    float scale = 0.0f;
    if (vol->normalize_size) {
        const v3 phys = V3((float)s->res[0] * vol->spacing[0], (float)s->res[1] * vol->spacing[1], (float)s->res[2] * vol->spacing[2]);
        scale = 1.0f / smax(phys.x, smax(phys.y, phys.z));
    }
    s->spacing = V3(vol->spacing[0] * scale, vol->spacing[1] * scale, vol->spacing[2] * scale);
    s->size = V3((float)s->res[0] * s->spacing.x, (float)s->res[1] * s->spacing.y, (float)s->res[2] * s->spacing.z);
    s->inv_size = V3(1.0f / s->size.x, 1.0f / s->size.y, 1.0f / s->size.z);
    s->minp = vscale(s->size, -0.5f);
    s->min_step = smin(s->spacing.x, smin(s->spacing.y, s->spacing.z));
    s->gdx = V3(s->min_step, 0.0f, 0.0f);
    s->gdy = V3(0.0f, s->min_step, 0.0f);
    s->gdz = V3(0.0f, 0.0f, s->min_step);

    /* Camera::Update - Source/camera.h:61-96 */
    const er_camera_desc* c = &t->camera;
    s->film[0] = c->film_size[0];
    s->film[1] = c->film_size[1];
    s->pos = V3(c->pos[0], c->pos[1], c->pos[2]);
    const v3 target = V3(c->target[0], c->target[1], c->target[2]);
    const v3 up = V3(c->up[0], c->up[1], c->up[2]);
    s->N = vnorm(vsub(target, s->pos));
    s->U = vnorm(vcross(s->N, up));
    s->V = vnorm(vcross(s->N, s->U));
    s->focal_distance = c->focal_distance;
    if (s->focal_distance == -1.0f) s->focal_distance = vlen(vsub(target, s->pos));
    const float sc = er_tanf((0.5f * c->fov / 57.29577951308232f));
    const float aspect = (float)c->film_size[1] / (float)c->film_size[0];
    if (aspect > 1.0f) {
        s->screen[0][0] = -sc; s->screen[0][1] = sc;
        s->screen[1][0] = -sc * aspect; s->screen[1][1] = sc * aspect;
    } else {
        s->screen[0][0] = -sc / aspect; s->screen[0][1] = sc / aspect;
        s->screen[1][0] = -sc; s->screen[1][1] = sc;
    }
    s->inv_screen[0] = (s->screen[0][1] - s->screen[0][0]) / (float)c->film_size[0];
    s->inv_screen[1] = (s->screen[1][1] - s->screen[1][0]) / (float)c->film_size[1];
    s->clip_near = c->clip_near;
    s->clip_far = c->clip_far;
    s->aperture = c->aperture_size;
    s->exposure = c->exposure;

    s->st = t->settings;
    s->opacity = t->opacity;
    s->glossiness = t->glossiness;
    s->diffuse = t->diffuse;
    s->specular = t->specular;
    s->emission = t->emission;
    s->light_count = t->light_count;
    s->object_count = t->object_count > 0 ? t->object_count : 0;
    s->tau_u = -1.0f;
    for (int i = 0; i < ER_MAX_INDICES; i++) s->light_idx[i] = t->light_ids[i];
    s->clip_ids_count = t->clipping_object_count < 0 ? 0 : (t->clipping_object_count > ER_MAX_INDICES ? ER_MAX_INDICES : t->clipping_object_count);
    for (int i = 0; i < ER_MAX_INDICES; i++) s->clip_ids[i] = t->clipping_object_ids[i];

    s->n_lights = n_lights;
    s->lights = (or_light*)calloc(n_lights > 0 ? (size_t)n_lights : 1u, sizeof(or_light));
    for (int i = 0; i < n_lights; i++) {
        s->lights[i].d = lights[i];
        s->lights[i].area = shape_area(&lights[i].shape);   /* Light::operator= - Source/light.h:39-45 */
    }
    s->n_textures = n_textures;
    s->textures = (er_texture_desc*)calloc(n_textures > 0 ? (size_t)n_textures : 1u, sizeof(er_texture_desc));
    if (n_textures > 0) memcpy(s->textures, textures, sizeof(er_texture_desc) * (size_t)n_textures);
    prepare_extensions(s);
    return s;
}

void ER_OR(scene_destroy)(or_scene* s)
{
    if (!s) return;
    free(s->lights);
    free(s->textures);
    free(s->objects);
    free(s->clips);
    for (int i = 0; i < s->n_bitmaps; i++) free(s->bitmap_pixels[i]);
    free(s->bitmap_pixels);
    free(s->bitmap_res);
    free(s->sigma);
    free(s->majorant);
    free(s);
}

/* ------------------------------------------------------------------ */
/* RNG - Source/rng.h:26-66                                             */
/* ------------------------------------------------------------------ */

typedef struct { uint32_t s0, s1; } rng_t;

static inline float rng_get1(rng_t* r)   /* :35-51 */
{
    r->s0 = 36969u * (r->s0 & 65535u) + (r->s0 >> 16);
    r->s1 = 18000u * (r->s1 & 65535u) + (r->s1 >> 16);
    const uint32_t ires = (r->s0 << 16) + r->s1;
    const float f = er_u2f((ires & 0x007fffffu) | 0x40000000u);
    return (f - 2.0f) / 2.0f;
}

/* Get2/Get3 (:53-61) construct Vec2f(Get1(), Get1()); the host compiler
   evaluates constructor arguments right to left, so the last component
   receives the first draw (checked by tests/test_oracle_ref.py). */
static inline v2 rng_get2(rng_t* r)
{
    v2 v;
    v.y = rng_get1(r);
    v.x = rng_get1(r);
    return v;
}
static inline v3 rng_get3(rng_t* r)
{
    v3 v;
    v.z = rng_get1(r);
    v.y = rng_get1(r);
    v.x = rng_get1(r);
    return v;
}

/* MetroSample::LargeStep - Source/sample.h:258-262 with :142-146, :101-104,
   :180-185, :221-225 */
typedef struct {
    float brdf_component;
    v2 brdf_dir;
    v3 light_uvw;
    float light_num;
    v2 film_uv;
    v2 lens_uv;
} metro_sample;

static inline void metro_large_step(metro_sample* m, rng_t* r)
{
    m->brdf_component = rng_get1(r);
    m->brdf_dir = rng_get2(r);
    m->light_uvw = rng_get3(r);
    m->light_num = rng_get1(r);
    m->film_uv = rng_get2(r);
    m->lens_uv = rng_get2(r);
}

/* ------------------------------------------------------------------ */
/* transfer functions - Source/plf.h:68-91                              */
/* ------------------------------------------------------------------ */

static inline float plf_eval(const er_plf* p, float x)
{
    if (p->count <= 0) return 0.0f;
    if (x < p->node_range[0]) return p->value[0];
    if (x > p->node_range[1]) return p->value[p->count - 1];
    for (int i = 1; i < p->count; i++) {
        const float P1 = p->position[i - 1];
        const float P2 = p->position[i];
        const float DeltaP = P2 - P1;
        const float LerpT = (x - P1) / DeltaP;
        if (x >= P1 && x < P2) return p->value[i - 1] + LerpT * (p->value[i] - p->value[i - 1]);
    }
    return 0.0f;
}

/* ColorTransferFunction1D::Evaluate - Source/transferfunction.h:148-151 */
static inline col3 ctf_eval(const er_color_tf* t, float x)
{
    return C3(plf_eval(&t->plf[0], x), plf_eval(&t->plf[1], x), plf_eval(&t->plf[2], x));
}

/* ------------------------------------------------------------------ */
/* volume access                                                        */
/* ------------------------------------------------------------------ */

/* Buffer3D<T>::operator()(const int&,const int&,const int&) - Source/buffer3d.h:210-214 */
static inline float voxel(const or_scene* s, int x, int y, int z)
{
    const int cx = iclamp(x, 0, s->res[0] - 1);
    const int cy = iclamp(y, 0, s->res[1] - 1);
    const int cz = iclamp(z, 0, s->res[2] - 1);
    return (float)s->vox[(size_t)cz * (size_t)s->res[0] * (size_t)s->res[1] + (size_t)cy * (size_t)s->res[0] + (size_t)cx];
}

/* Lerp(t, v1, v2) - Source/geometry.h:87-90; the result is stored in an
   unsigned short (T of Buffer3D<unsigned short>), i.e. truncated. */
static inline float lerp_u16(float t, float a, float b)
{
    const float r = (1.0f - t) * a + t * b;
    return (float)(unsigned short)r;
}

/* GetIntensity (Source/volumes.h:26-29) -> Volume::operator() (Source/volume.h:131-138)
   -> Buffer3D<unsigned short>::operator()(Vec3f) (Source/buffer3d.h:222-242) */
/* the trilinear lookup at local voxel coordinates L */
static inline float get_intensity_local(or_scene* s, v3 L)
{
    s->lookups++;
    const int vx = (int)floorf(L.x);
    const int vy = (int)floorf(L.y);
    const int vz = (int)floorf(L.z);
    const float dx = L.x - (float)vx;
    const float dy = L.y - (float)vy;
    const float dz = L.z - (float)vz;
    const float d00 = lerp_u16(dx, voxel(s, vx, vy, vz), voxel(s, vx + 1, vy, vz));
    const float d10 = lerp_u16(dx, voxel(s, vx, vy + 1, vz), voxel(s, vx + 1, vy + 1, vz));
    const float d01 = lerp_u16(dx, voxel(s, vx, vy, vz + 1), voxel(s, vx + 1, vy, vz + 1));
    const float d11 = lerp_u16(dx, voxel(s, vx, vy + 1, vz + 1), voxel(s, vx + 1, vy + 1, vz + 1));
    const float d0 = lerp_u16(dy, d00, d10);
    const float d1 = lerp_u16(dy, d01, d11);
    return lerp_u16(dz, d0, d1);
}

static inline v3 local_coords(const or_scene* s, v3 P)
{
    const v3 off = vsub(P, s->minp);
    return V3(off.x * s->inv_size.x * (float)s->res[0], off.y * s->inv_size.y * (float)s->res[1],
              off.z * s->inv_size.z * (float)s->res[2]);
}

static inline float get_intensity(or_scene* s, v3 P)
{
    return get_intensity_local(s, local_coords(s, P));
}

/* GradientCD / GradientFD / GradientFiltered / Gradient - Source/volumes.h:31-86 */
static v3 gradient_cd(or_scene* s, v3 P)
{
    const float i00 = get_intensity(s, vadd(P, s->gdx)), i01 = get_intensity(s, vsub(P, s->gdx));
    const float i10 = get_intensity(s, vadd(P, s->gdy)), i11 = get_intensity(s, vsub(P, s->gdy));
    const float i20 = get_intensity(s, vadd(P, s->gdz)), i21 = get_intensity(s, vsub(P, s->gdz));
    return V3(i01 - i00, i11 - i10, i21 - i20);
}

static v3 gradient_fd(or_scene* s, v3 P)
{
    const float i0 = get_intensity(s, P);
    const float i1 = get_intensity(s, vadd(P, s->gdx));
    const float i2 = get_intensity(s, vadd(P, s->gdy));
    const float i3 = get_intensity(s, vadd(P, s->gdz));
    return V3(i0 - i1, i0 - i2, i0 - i3);
}

/* Lerp(const Vec3f& A, const Vec3f& B, const float& c) = A + c*(B - A) - Source/vector.h:552 */
static inline v3 vlerp(v3 a, v3 b, float c) { return vadd(a, vscale(vsub(b, a), c)); }

static v3 gradient_filtered(or_scene* s, v3 P)
{
    const v3 o = V3(s->gdx.x, s->gdy.y, s->gdz.z);
    const v3 G0 = gradient_cd(s, P);
    const v3 G1 = gradient_cd(s, vadd(P, V3(-o.x, -o.y, -o.z)));
    const v3 G2 = gradient_cd(s, vadd(P, V3(o.x, o.y, o.z)));
    const v3 G3 = gradient_cd(s, vadd(P, V3(-o.x, o.y, -o.z)));
    const v3 G4 = gradient_cd(s, vadd(P, V3(o.x, -o.y, o.z)));
    const v3 G5 = gradient_cd(s, vadd(P, V3(-o.x, -o.y, o.z)));
    const v3 G6 = gradient_cd(s, vadd(P, V3(o.x, o.y, -o.z)));
    const v3 G7 = gradient_cd(s, vadd(P, V3(-o.x, o.y, o.z)));
    const v3 G8 = gradient_cd(s, vadd(P, V3(o.x, -o.y, -o.z)));
    const v3 L0 = vlerp(vlerp(G1, G2, 0.5f), vlerp(G3, G4, 0.5f), 0.5f);
    const v3 L1 = vlerp(vlerp(G5, G6, 0.5f), vlerp(G7, G8, 0.5f), 0.5f);
    return vlerp(G0, vlerp(L0, L1, 0.5f), 0.75f);
}

static v3 gradient(or_scene* s, v3 P)
{
    switch (s->st.gradient_computation) {
    case ER_GRADIENT_FORWARD: return gradient_fd(s, P);
    case ER_GRADIENT_CENTRAL: return gradient_cd(s, P);
    case ER_GRADIENT_FILTERED: return gradient_filtered(s, P);
    default: return gradient_fd(s, P);
    }
}

/* NormalizedGradient - Source/volumes.h:88-91 */
static v3 normalized_gradient(or_scene* s, v3 P)
{
    const uint64_t lk = s->lookups;
    const v3 g = vnorm(gradient(s, P));
    s->stat[OR_STAT_NORMAL_LOOKUPS] += s->lookups - lk;
    return g;
}

/* GradientMagnitude - Source/volumes.h:93-114 */
static float gradient_magnitude(or_scene* s, v3 P)
{
    v3 pts[3][2];
    pts[0][0] = vadd(P, s->gdx); pts[0][1] = vsub(P, s->gdx);
    pts[1][0] = vadd(P, s->gdy); pts[1][1] = vsub(P, s->gdy);
    pts[2][0] = vadd(P, s->gdz); pts[2][1] = vsub(P, s->gdz);
    float sum = 0.0f;
    for (int i = 0; i < 3; i++) {
        float D = get_intensity(s, pts[i][1]) - get_intensity(s, pts[i][0]);
        D *= 0.5f / vget(s->spacing, i);
        sum += D * D;
    }
    return sqrtf(sum);
}

/* ------------------------------------------------------------------ */
/* geometry                                                             */
/* ------------------------------------------------------------------ */

typedef struct { v3 O, D; float MinT, MaxT; } ray_t;   /* Source/ray.h:26-56 */

/* Ray::operator()(T) = O + Normalize(D)*T - Source/ray.h:47-50 */
static inline v3 ray_at(const ray_t* r, float t) { return vadd(r->O, vscale(vnorm(r->D), t)); }

typedef struct {                                         /* Source/intersection.h:30-78 */
    int valid, front;
    float near_t, far_t;
    v3 P, N;
    v2 UV;
} isect_t;

static inline void isect_invalid(isect_t* i)             /* :47-56 */
{
    i->valid = 0; i->front = 1; i->near_t = 0.0f; i->far_t = FLT_MAX;
    i->P = V3(0, 0, 0); i->N = V3(0, 0, 0); i->UV.x = 0.0f; i->UV.y = 0.0f;
}

/* TransformPoint / TransformVector / TransformRay - Source/geometry.h:30-68 */
static inline v3 xform_point(const desc_f32 m[4][4], v3 p)
{
    return V3(m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3],
              m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3],
              m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3]);
}
static inline v3 xform_vector(const desc_f32 m[4][4], v3 v)
{
    return V3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z,
              m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}
static inline ray_t xform_ray(const desc_f32 m[4][4], const ray_t* r)
{
    ray_t t;
    const v3 P = xform_point(m, r->O);
    const v3 MinP = xform_point(m, ray_at(r, r->MinT));
    const v3 MaxP = xform_point(m, ray_at(r, r->MaxT));
    t.O = P;
    t.D = vnorm(vsub(MaxP, t.O));
    t.MinT = vlen(vsub(MinP, t.O));
    t.MaxT = vlen(vsub(MaxP, t.O));
    return t;
}

/* SphericalTheta / SphericalPhi / SphericalToUV - Source/geometry.h:70-85 */
static inline float spherical_theta(v3 w) { return er_acosf(eclamp(w.y, -1.0f, 1.0f)); }
static inline float spherical_phi(v3 w)
{
    const float p = er_atan2f(w.z, w.x);
    return (p < 0.0f) ? p + 2.0f * PI_F : p;
}

/* IntersectBox(R, MinAABB, MaxAABB, Int) - Source/box.h:51-83 */
static void intersect_box(const ray_t* R, v3 mn, v3 mx, isect_t* I)
{
    const v3 InvR = V3(1.0f / R->D.x, 1.0f / R->D.y, 1.0f / R->D.z);
    const v3 B = vmul(InvR, vsub(mn, R->O));
    const v3 T = vmul(InvR, vsub(mx, R->O));
    const v3 MinT = V3(smin(T.x, B.x), smin(T.y, B.y), smin(T.z, B.z));
    const v3 MaxT = V3(smax(T.x, B.x), smax(T.y, B.y), smax(T.z, B.z));
    const float LargestMinT = fmaxf(fmaxf(MinT.x, MinT.y), fmaxf(MinT.x, MinT.z));
    const float LargestMaxT = fminf(fminf(MaxT.x, MaxT.y), fminf(MaxT.x, MaxT.z));
    if (LargestMaxT < LargestMinT) return;
    I->near_t = LargestMinT > 0.0f ? LargestMinT : 0.0f;
    I->far_t = LargestMaxT;
    if (I->near_t < R->MinT || I->near_t > R->MaxT) return;
    I->valid = 1;
    I->P = ray_at(R, I->near_t);
    I->N = V3(0, 0, 0);
    I->UV.x = 0.0f; I->UV.y = 0.0f;
    float n[3] = { 0.0f, 0.0f, 0.0f };
    for (int i = 0; i < 3; i++) {
        if (vget(I->P, i) <= vget(mn, i) + 0.0001f) n[i] = -1.0f;
        if (vget(I->P, i) >= vget(mx, i) - 0.0001f) n[i] = 1.0f;
    }
    I->N = V3(n[0], n[1], n[2]);
}

/* IntersectPlane(R, OneSided, Int) - Source/plane.h:41-62 */
static void intersect_plane_inf(const ray_t* R, int one_sided, isect_t* I)
{
    if (fabsf(R->O.z - R->D.z) < RAY_EPS) return;
    I->near_t = (0.0f - R->O.z) / R->D.z;
    if (I->near_t < R->MinT || I->near_t > R->MaxT) return;
    I->P = ray_at(R, I->near_t);
    I->UV.x = I->P.x; I->UV.y = I->P.y;
    I->N = V3(0.0f, 0.0f, 1.0f);
    if (one_sided && R->D.z >= 0.0f) {
        I->front = 0;
        I->N = V3(0.0f, 0.0f, -1.0f);
    }
    I->valid = 1;
}

/* IntersectPlane(R, OneSided, Size, Int) - Source/plane.h:76-88 */
static void intersect_plane(const ray_t* R, int one_sided, float sx, float sy, isect_t* I)
{
    intersect_plane_inf(R, one_sided, I);
    if (I->valid && (I->UV.x < -0.5f * sx || I->UV.x > 0.5f * sx || I->UV.y < -0.5f * sy || I->UV.y > 0.5f * sy))
        I->valid = 0;
    I->UV.x /= sx;
    I->UV.y /= sy;
    I->UV.x = I->UV.x + 0.5f;
    I->UV.y = I->UV.y + 0.5f;
    I->UV.x = 1.0f - I->UV.x;
}

static inline float v2len(v2 a) { return sqrtf(a.x * a.x + a.y * a.y); }   /* Source/vector.h:418-426 */

/* IntersectDisk - Source/disk.h:37-49 */
static void intersect_disk(const ray_t* R, int one_sided, float radius, isect_t* I)
{
    intersect_plane_inf(R, one_sided, I);
    if (I->valid && v2len(I->UV) > radius) I->valid = 0;
    const float diameter = 2.0f * radius;
    I->UV.x /= diameter; I->UV.y /= diameter;
    I->UV.x = I->UV.x + 0.5f; I->UV.y = I->UV.y + 0.5f;
    I->UV.x = 1.0f - I->UV.x;
}

/* IntersectRing - Source/ring.h:45-57 */
static void intersect_ring(const ray_t* R, int one_sided, float inner, float outer, isect_t* I)
{
    intersect_plane_inf(R, one_sided, I);
    if (I->valid && (v2len(I->UV) < inner || v2len(I->UV) > outer)) I->valid = 0;
    const float diameter = 2.0f * outer;
    I->UV.x /= diameter; I->UV.y /= diameter;
    I->UV.x = I->UV.x + 0.5f; I->UV.y = I->UV.y + 0.5f;
    I->UV.x = 1.0f - I->UV.x;
}

/* IntersectSphere - Source/sphere.h:84-140 */
static void intersect_sphere(const ray_t* R, float radius, isect_t* I)
{
    const float a = vdot(R->D, R->D);
    const float b = 2 * vdot(R->D, R->O);
    const float c = vdot(R->O, R->O) - (radius * radius);
    const float disc = b * b - 4 * a * c;
    if (disc < 0) return;
    const float distSqrt = sqrtf(disc);
    float q;
    if (b < 0) q = (-b - distSqrt) / 2.0f;
    else q = (-b + distSqrt) / 2.0f;
    float t0 = q / a;
    float t1 = c / q;
    if (t0 > t1) { const float tmp = t0; t0 = t1; t1 = tmp; }
    if (t0 >= R->MinT && t0 < R->MaxT) I->near_t = t0;
    else {
        if (t1 >= R->MinT && t1 < R->MaxT) I->near_t = t1;
        else return;
    }
    if (I->near_t < R->MinT || I->near_t > R->MaxT) return;
    I->valid = 1;
    I->P = ray_at(R, I->near_t);
    I->N = vnorm(I->P);
    const v3 Vn = vnorm(I->P);   /* SphericalToUV - Source/geometry.h:81-85 */
    I->UV.x = INV_TWO_PI_F * spherical_phi(Vn);
    I->UV.y = 1.0f - (INV_PI_F * spherical_theta(Vn));
}

/* IntersectShape / IntersectsShape - Source/shapes.h:44-72 (box lights use the
   3-component size, Source/box.h:85-88) */
static void intersect_shape(const er_shape* sh, const ray_t* R, isect_t* I)
{
    switch (sh->type) {
    case ER_SHAPE_PLANE: intersect_plane(R, sh->one_sided, sh->size[0], sh->size[1], I); break;
    case ER_SHAPE_DISK: intersect_disk(R, sh->one_sided, sh->outer_radius, I); break;
    case ER_SHAPE_RING: intersect_ring(R, sh->one_sided, sh->inner_radius, sh->outer_radius, I); break;
    case ER_SHAPE_BOX: {
        const v3 size = V3(sh->size[0], sh->size[1], sh->size[2]);
        intersect_box(R, vscale(size, -0.5f), vscale(size, 0.5f), I);
        break;
    }
    case ER_SHAPE_SPHERE: intersect_sphere(R, sh->outer_radius, I); break;
    default: break;
    }
}

/* ------------------------------------------------------------------ */
/* sampling - Source/montecarlo.h, shape samplers                       */
/* ------------------------------------------------------------------ */

/* ConcentricSampleDisk - Source/montecarlo.h:86-137 */
static v2 concentric_sample_disk(v2 U)
{
    float r, theta;
    const float sx = 2 * U.x - 1;
    const float sy = 2 * U.y - 1;
    v2 out;
    if (sx == 0.0 && sy == 0.0) { out.x = 0.0f; out.y = 0.0f; return out; }
    if (sx >= -sy) {
        if (sx > sy) {
            r = sx;
            if (sy > 0.0) theta = sy / r;
            else theta = 8.0f + sy / r;
        } else {
            r = sy;
            theta = 2.0f - sx / r;
        }
    } else {
        if (sx <= sy) {
            r = -sx;
            theta = 4.0f - sy / r;
        } else {
            r = -sy;
            theta = 6.0f + sx / r;
        }
    }
    theta *= PI_F / 4.f;
    float sn, cs;
    er_sincosf(theta, &sn, &cs);
    out.x = r * cs;
    out.y = r * sn;
    return out;
}

typedef struct { v3 P, N; v2 UV; } surf_sample;   /* Source/sample.h:57-79 */

/* SampleLightSurface - Source/lights.h:28-42 with the shape samplers
   Source/plane.h:95-107, Source/disk.h:59-74, Source/ring.h:59-75,
   Source/box.h:122-191, Source/sphere.h:152-170 */
static void sample_light_surface(const or_light* L, v3 UVW, surf_sample* SS)
{
    const er_shape* sh = &L->d.shape;
    SS->P = V3(0, 0, 0); SS->N = V3(0.0f, 0.0f, 1.0f); SS->UV.x = 0.0f; SS->UV.y = 0.0f;
    switch (sh->type) {
    case ER_SHAPE_PLANE:
        SS->P = V3(-0.5f + UVW.x, -0.5f + UVW.y, 0.0f);
        SS->N = V3(0.0f, 0.0f, 1.0f);
        SS->UV.x = UVW.x; SS->UV.y = UVW.y;
        SS->P = vmul(SS->P, V3(sh->size[0], sh->size[1], 0.0f));
        break;
    case ER_SHAPE_DISK: {
        const float r = sqrtf(UVW.x);
        const float theta = 2.0f * PI_F * UVW.y;
        float sn, cs; er_sincosf(theta, &sn, &cs);
        SS->P = V3(r * cs, r * sn, 0.0f);
        SS->N = V3(0.0f, 0.0f, 1.0f);
        SS->UV.x = UVW.x; SS->UV.y = UVW.y;
        SS->P = vscale(SS->P, sh->outer_radius);
        break;
    }
    case ER_SHAPE_RING: {
        const float inner = sh->inner_radius / sh->outer_radius;
        const float r = inner + (1.0f - inner) * sqrtf(UVW.x);
        const float theta = 2.0f * PI_F * UVW.y;
        float sn, cs; er_sincosf(theta, &sn, &cs);
        SS->P = V3(r * cs, r * sn, 0.0f);
        SS->N = V3(0.0f, 0.0f, 1.0f);
        SS->P = vscale(SS->P, sh->outer_radius);
        SS->UV.x = SS->P.x; SS->UV.y = SS->P.y;
        break;
    }
    case ER_SHAPE_BOX: {
        const int side = (int)floorf(UVW.x * 6.0f);
        v3 p = V3(0, 0, 0);
        v3 n = SS->N;
        switch (side) {
        case 0: p = V3(0.5f, -0.5f + UVW.z, -0.5f + UVW.y); n = V3(1.0f, 0.0f, 0.0f); break;
        case 1: p = V3(-0.5f, -0.5f + UVW.z, -0.5f + UVW.y); n = V3(-1.0f, 0.0f, 0.0f); break;
        case 2: p = V3(-0.5f + UVW.y, 0.5f, -0.5f + UVW.z); n = V3(0.0f, 1.0f, 0.0f); break;
        case 3: p = V3(-0.5f + UVW.y, -0.5f, -0.5f + UVW.z); n = V3(0.0f, -1.0f, 0.0f); break;
        case 4: p = V3(-0.5f + UVW.y, -0.5f + UVW.z, 0.5f); n = V3(0.0f, 0.0f, 1.0f); break;
        case 5: p = V3(-0.5f + UVW.y, -0.5f + UVW.z, -0.5f); n = V3(0.0f, 0.0f, -1.0f); break;
        default: break;
        }
        SS->P = p; SS->N = n;
        SS->UV.x = UVW.y; SS->UV.y = UVW.z;
        SS->P = vmul(SS->P, V3(sh->size[0], sh->size[1], sh->size[2]));
        break;
    }
    case ER_SHAPE_SPHERE: {
        const float z = 1.0f - 2.0f * UVW.x;
        const float r = sqrtf(smax(0.0f, 1.0f - z * z));
        const float phi = 2.0f * PI_F * UVW.y;
        float sn, cs; er_sincosf(phi, &sn, &cs);
        SS->P = V3(r * cs, r * sn, z);
        SS->N = SS->P;
        SS->UV.x = spherical_theta(SS->P);
        SS->UV.y = spherical_phi(SS->P);
        SS->P = vscale(SS->P, sh->outer_radius);
        break;
    }
    default: break;
    }
    SS->P = xform_point(sh->tm, SS->P);
    SS->N = xform_vector(sh->tm, SS->N);
}

/* ------------------------------------------------------------------ */
/* textures - Source/textures.h:26-111                                  */
/* ------------------------------------------------------------------ */

/* scalar * ColorRGBAuc as the reference evaluates it: the float converts to
   the colour's unsigned char component type (truncation), then multiplies each
   component in unsigned char arithmetic (Source/color.h:282-283,
   Source/vector.h:183-190); sums of colours wrap in unsigned char
   (Source/vector.h OPERATOR_PLUS) */
static inline uint8_t uc_weight(float w) { return (uint8_t)w; }

/* Buffer2D<ColorRGBAuc>::operator()(Vec2f, Normalized = true)
   (Source/buffer2d.h:227-254) followed by ColorXYZf::FromRGBAuc
   (Source/color.h:195-209).  The bilinear weights pass through unsigned char,
   so a lookup is the floor texel when the scaled coordinate is an integer
   and black otherwise; kept as the reference computes it. */
static col3 bitmap_xyz(const uint8_t* px, int w, int h, v2 uv)
{
    const float U = uv.x * (float)w, V = uv.y * (float)h;
    int c0[2] = { (int)floorf(U), (int)ceilf(U) };
    int c1[2] = { (int)floorf(V), (int)ceilf(V) };
    const float du = U - (float)c0[0];
    const float dv = V - (float)c1[0];
    for (int k = 0; k < 2; k++) {
        c0[k] = c0[k] < 0 ? 0 : (c0[k] > w - 1 ? w - 1 : c0[k]);
        c1[k] = c1[k] < 0 ? 0 : (c1[k] > h - 1 ? h - 1 : c1[k]);
    }
    const uint8_t* v00 = px + 4 * ((size_t)c1[0] * w + c0[0]);
    const uint8_t* v10 = px + 4 * ((size_t)c1[0] * w + c0[1]);
    const uint8_t* v01 = px + 4 * ((size_t)c1[1] * w + c0[0]);
    const uint8_t* v11 = px + 4 * ((size_t)c1[1] * w + c0[1]);
    const uint8_t wu0 = uc_weight(1.0f - du), wu1 = uc_weight(du);
    const uint8_t wv0 = uc_weight(1.0f - dv), wv1 = uc_weight(dv);
    uint8_t rgb[3];
    for (int c = 0; c < 3; c++) {
        const uint8_t top = (uint8_t)((uint8_t)(wu0 * v00[c]) + (uint8_t)(wu1 * v10[c]));
        const uint8_t bot = (uint8_t)((uint8_t)(wu0 * v01[c]) + (uint8_t)(wu1 * v11[c]));
        rgb[c] = (uint8_t)((uint8_t)(wv0 * top) + (uint8_t)(wv1 * bot));
    }
    const float k = 1.0f / 255.0f;
    const float r = k * (float)rgb[0], g = k * (float)rgb[1], b = k * (float)rgb[2];
    return C3(0.412453f * r + 0.357580f * g + 0.180423f * b,
              0.212671f * r + 0.715160f * g + 0.072169f * b,
              0.019334f * r + 0.119193f * g + 0.950227f * b);
}

static col3 evaluate_texture(const or_scene* s, int id, v2 UV)
{
    if (id < 0) return C3(0, 0, 0);
    if (id >= s->n_textures) return C3(0, 0, 0);
    const er_texture_desc* T = &s->textures[id];
    col3 L = C3(0, 0, 0);
    v2 tuv = UV;
    tuv.x *= T->repeat[0];
    tuv.y *= T->repeat[1];
    tuv.x += T->offset[0];
    tuv.y += 1.0f - T->offset[1];
    tuv.x = tuv.x - floorf(tuv.x);
    tuv.y = tuv.y - floorf(tuv.y);
    tuv.x = eclamp(tuv.x, 0.0f, 1.0f);
    tuv.y = eclamp(tuv.y, 0.0f, 1.0f);
    if (T->flip[0]) tuv.x = 1.0f - tuv.x;
    if (T->flip[1]) tuv.y = 1.0f - tuv.y;
    if (T->type == ER_TEXTURE_PROCEDURAL) {
        const er_procedural* P = &T->procedural;
        switch (P->type) {
        case ER_PROCEDURAL_UNIFORM: L = C3(P->uniform_color[0], P->uniform_color[1], P->uniform_color[2]); break;
        case ER_PROCEDURAL_CHECKER: {
            const int u = (int)(tuv.x * 2.0f), v = (int)(tuv.y * 2.0f);
            const desc_f32* c1 = P->checker_color1;
            const desc_f32* c2 = P->checker_color2;
            const desc_f32* c = (u % 2 == 0) ? ((v % 2 == 0) ? c1 : c2) : ((v % 2 == 0) ? c2 : c1);
            L = C3(c[0], c[1], c[2]);
            break;
        }
        case ER_PROCEDURAL_GRADIENT: L = ctf_eval(&P->gradient, tuv.y); break;
        default: L = C3(0, 0, 0); break;
        }
    }
    if (T->type == ER_TEXTURE_BITMAP && T->bitmap_id >= 0 && T->bitmap_id < s->n_bitmaps)
        L = bitmap_xyz(s->bitmap_pixels[T->bitmap_id], s->bitmap_res[2 * T->bitmap_id], s->bitmap_res[2 * T->bitmap_id + 1], tuv);
    return cscale(L, T->output_level);
}

/* ------------------------------------------------------------------ */
/* shading - Source/shader.h                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    int type;          /* 0 = BRDF, 1 = isotropic phase (Source/enums.h:95-99) */
    v3 Nn, Nu, Nv;
    col3 Kd, Ks;
    float ior;
    float exponent;
} shader_t;

/* Shader(Type, N, Wo, Kd, Ks, Ior, Exponent) - Source/shader.h:422-427 with BRDF :323-330 */
static void shader_init(shader_t* sh, int type, v3 N, v3 Wo, col3 Kd, col3 Ks, float ior, float exponent)
{
    sh->type = type;
    sh->Nn = vnorm(N);
    sh->Nu = vnorm(vcross(N, Wo));
    sh->Nv = vnorm(vcross(N, sh->Nu));
    sh->Kd = Kd;
    sh->Ks = Ks;
    sh->ior = ior;
    sh->exponent = exponent;
}

/* BRDF::WorldToLocal - Source/shader.h:332-335 */
static inline v3 world_to_local(const shader_t* sh, v3 W) { return V3(vdot(W, sh->Nu), vdot(W, sh->Nv), vdot(W, sh->Nn)); }
/* BRDF::LocalToWorld - :337-342 */
static inline v3 local_to_world(const shader_t* sh, v3 W)
{
    return V3(sh->Nu.x * W.x + sh->Nv.x * W.y + sh->Nn.x * W.z,
              sh->Nu.y * W.x + sh->Nv.y * W.y + sh->Nn.y * W.z,
              sh->Nu.z * W.x + sh->Nv.z * W.y + sh->Nn.z * W.z);
}

/* Fresnel::Evaluate - Source/shader.h:92-117, FrDiel :72-77 (all three
   components of the colour are equal, so one scalar is carried) */
static float fresnel_eval(float ei_, float et_, float cosi)
{
    cosi = eclamp(cosi, -1.0f, 1.0f);
    const int entering = cosi > 0.0f;
    float ei = ei_, et = et_;
    if (!entering) { const float t = ei; ei = et; et = t; }
    const float sint = ei / et * sqrtf(smax(0.f, 1.f - cosi * cosi));
    if (sint >= 1.0f) return 1.0f;
    const float cost = sqrtf(smax(0.f, 1.0f - sint * sint));
    const float ci = fabsf(cosi);
    const float Rparl = ((et * ci) - (ei * cost)) / ((et * ci) + (ei * cost));
    const float Rperp = ((ei * ci) - (et * cost)) / ((ei * ci) + (et * cost));
    return (Rparl * Rparl + Rperp * Rperp) / 2.f;
}

/* Blinn::D - :182-186 */
static inline float blinn_d(float exponent, v3 Wh)
{
    const float c = fabsf(Wh.z);
    return (exponent + 2) * INV_TWO_PI_F * er_powf(c, exponent);
}

/* Blinn::Pdf - :166-180 */
static inline float blinn_pdf(float exponent, v3 Wo, v3 Wi)
{
    const v3 Wh = vnorm(vadd(Wo, Wi));
    const float CosTheta = fabsf(Wh.z);
    float pdf = ((exponent + 1.0f) * er_powf(CosTheta, exponent)) / (2.0f * PI_F * 4.0f * vdot(Wo, Wh));
    if (vdot(Wo, Wh) <= 0.0f) pdf = 0.0f;
    return pdf;
}

/* Microfacet::F - :212-231 with G :251-259 */
static col3 microfacet_f(const shader_t* sh, v3 Wo, v3 Wi)
{
    const float cosThetaO = fabsf(Wo.z);
    const float cosThetaI = fabsf(Wi.z);
    if (cosThetaI == 0.f || cosThetaO == 0.f) return C3(0, 0, 0);
    v3 Wh = vadd(Wi, Wo);
    if (Wh.x == 0. && Wh.y == 0. && Wh.z == 0.) return C3(0, 0, 0);
    Wh = vnorm(Wh);
    const float cosThetaH = vdot(Wi, Wh);
    const float F = fresnel_eval(1.0f, sh->ior, cosThetaH);
    const float NdotWh = fabsf(Wh.z), NdotWo = fabsf(Wo.z), NdotWi = fabsf(Wi.z);
    const float WOdotWh = vabsdot(Wo, Wh);
    const float G = smin(1.0f, smin((2.0f * NdotWh * NdotWo / WOdotWh), (2.0f * NdotWh * NdotWi / WOdotWh)));
    const float D = blinn_d(sh->exponent, Wh);
    const float den = 4.0f * cosThetaI * cosThetaO;
    col3 r = cscale(sh->Ks, D);
    r = cscale(r, G);
    r = cscale(r, F);
    return cdivs(r, den);
}

static inline int same_hemisphere(v3 a, v3 b) { return (a.z * b.z) > 0.0f; }   /* Source/montecarlo.h:57-60 */

/* Shader::F - :429-441 (BRDF::F :344-355, IsotropicPhase::F :288-291) */
static col3 shader_f(const shader_t* sh, v3 Wo, v3 Wi)
{
    if (sh->type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        const v3 Wil = world_to_local(sh, Wi);
        col3 R = C3(0, 0, 0);
        R = cadd(R, cscale(sh->Kd, INV_PI_F));
        R = cadd(R, microfacet_f(sh, Wol, Wil));
        return R;
    }
    return cscale(sh->Kd, INV_PI_F);
}

/* Shader::Pdf - :457-469 (BRDF::Pdf :384-395, Lambertian::Pdf :58-61,
   Microfacet::Pdf :243-249, IsotropicPhase::Pdf :301-304) */
static float shader_pdf(const shader_t* sh, v3 Wo, v3 Wi)
{
    if (sh->type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        const v3 Wil = world_to_local(sh, Wi);
        float pdf = 0.0f;
        pdf += same_hemisphere(Wol, Wil) ? fabsf(Wil.z) * INV_PI_F : 0.0f;
        pdf += same_hemisphere(Wol, Wil) ? blinn_pdf(sh->exponent, Wol, Wil) : 0.0f;
        return pdf;
    }
    return INV_FOUR_PI_EXPANDED;
}

/* GlossinessExponent - Source/utilities.h:28-31 */
static inline float glossiness_exponent(float g) { return 1000000.0f * er_powf(g, 7.0f); }

/* PowerHeuristic(1, f, 1, g) - Source/montecarlo.h:223-227 */
static inline float power_heuristic(float fPdf, float gPdf)
{
    const float f = 1 * fPdf, g = 1 * gPdf;
    return (f * f) / (f * f + g * g);
}

/* ------------------------------------------------------------------ */
/* scatter events and transport                                         */
/* ------------------------------------------------------------------ */

typedef struct {                          /* Source/scatterevent.h:31-151 */
    int type;                             /* 0 volume, 1 light, 2 object */
    int valid;
    float T;
    v3 P, N, Wo;
    col3 Le;
    v2 UV;
    int light_id;
    int object_id;
} scatter_event;

static inline void se_invalid(scatter_event* se, int type)
{
    se->type = type; se->valid = 0; se->T = 0.0f;
    se->P = V3(0, 0, 0); se->N = V3(0, 0, 0); se->Wo = V3(0, 0, 0);
    se->Le = C3(0, 0, 0); se->UV.x = 0.0f; se->UV.y = 0.0f; se->light_id = -1; se->object_id = -1;
}

/* SampleVolume - Source/raymarching.h:30-71 */
static void sample_volume(or_scene* s, ray_t R, rng_t* rng, scatter_event* SE)
{
    isect_t Int; isect_invalid(&Int);
    intersect_box(&R, s->minp, vscale(s->size, 0.5f), &Int);
    if (!Int.valid) return;
    float MinT = smax(Int.near_t, R.MinT);
    const float MaxT = smin(Int.far_t, R.MaxT);
    const float S = -er_logf(rng_get1(rng)) / s->st.density_scale;
    float Sum = 0.0f;
    v3 Ps = V3(0, 0, 0);
    const float StepSize = s->st.step_factor_primary * s->min_step;
    MinT += rng_get1(rng) * StepSize;
    while (Sum < S) {
        Ps = vadd(R.O, vscale(R.D, MinT));
        if (MinT >= MaxT) return;
        const float SigmaT = (s->n_clips && clipped(s, Ps)) ? 0.0f : s->st.density_scale * plf_eval(&s->opacity, get_intensity(s, Ps));
        Sum += SigmaT * StepSize;
        MinT += StepSize;
    }
    SE->valid = 1;
    SE->T = MinT;
    SE->P = Ps;
    SE->N = normalized_gradient(s, Ps);
    SE->Wo = vneg(R.D);
    SE->Le = C3(0, 0, 0);
    SE->UV.x = 0.0f; SE->UV.y = 0.0f;
}

/* ScatterEventInVolume - Source/raymarching.h:73-113 */
static int scatter_event_in_volume(or_scene* s, ray_t R, rng_t* rng)
{
    isect_t Int; isect_invalid(&Int);
    intersect_box(&R, s->minp, vscale(s->size, 0.5f), &Int);
    if (!Int.valid) return 0;
    float MinT = smax(Int.near_t, R.MinT);
    const float MaxT = smin(Int.far_t, R.MaxT);
    const float S = -er_logf(rng_get1(rng)) / s->st.density_scale;
    float Sum = 0.0f;
    const float StepSize = s->st.step_factor_shadow * s->min_step;
    MinT += rng_get1(rng) * StepSize;
    while (Sum < S) {
        const v3 Ps = vadd(R.O, vscale(R.D, MinT));
        if (MinT > MaxT) return 0;
        const float SigmaT = (s->n_clips && clipped(s, Ps)) ? 0.0f : s->st.density_scale * plf_eval(&s->opacity, get_intensity(s, Ps));
        Sum += SigmaT * StepSize;
        MinT += StepSize;
    }
    return 1;
}

/* IntersectLight - Source/lights.h:59-88 */
static void intersect_light(const or_scene* s, const or_light* L, const ray_t* R, scatter_event* SE)
{
    const ray_t Rt = xform_ray(L->d.shape.inv_tm, R);
    isect_t Int; isect_invalid(&Int);
    intersect_shape(&L->d.shape, &Rt, &Int);
    if (Int.valid) {
        SE->valid = 1;
        SE->P = xform_point(L->d.shape.tm, Int.P);
        SE->N = xform_vector(L->d.shape.tm, Int.N);
        SE->T = vlen(vsub(SE->P, R->O));
        SE->Wo = vneg(R->D);
        SE->UV = Int.UV;
        SE->Le = Int.front ? cscale(evaluate_texture(s, L->d.texture_id, SE->UV), L->d.multiplier) : C3(0, 0, 0);
        if (L->d.unit == 1) SE->Le = cdivs(SE->Le, L->area);
    }
}

static inline const or_light* tracer_light(const or_scene* s, int i)
{
    const int id = s->light_idx[i];
    if (id < 0 || id >= s->n_lights) return NULL;
    return &s->lights[id];
}

/* IntersectLights - Source/lights.h:90-113 */
static void intersect_lights(const or_scene* s, const ray_t* R, scatter_event* RS, int respect_visibility)
{
    float T = FLT_MAX;
    for (int i = 0; i < s->light_count; i++) {
        const or_light* L = tracer_light(s, i);
        if (!L) continue;
        scatter_event local; se_invalid(&local, 1);
        local.light_id = i;
        if (respect_visibility && !L->d.visible) continue;
        intersect_light(s, L, R, &local);
        if (local.valid && local.T < T) { *RS = local; T = local.T; }
    }
}

/* IntersectsLight - Source/lights.h:115-131 */
static int intersects_light(const or_scene* s, const ray_t* R)
{
    for (int i = 0; i < s->light_count; i++) {
        const or_light* L = tracer_light(s, i);
        if (!L) continue;
        const ray_t Rt = xform_ray(L->d.shape.inv_tm, R);
        isect_t Int; isect_invalid(&Int);
        intersect_shape(&L->d.shape, &Rt, &Int);
        if (Int.valid) return 1;
    }
    return 0;
}

/* IntersectObject / IntersectObjects - Source/objects.h:26-62: the nearest
   of the tracer's first ObjectIDs.Count bound objects (array order) */
static void intersect_objects(const or_scene* s, const ray_t* R, scatter_event* RS)
{
    float T = FLT_MAX;
    for (int i = 0; i < s->object_count && i < s->n_objects; i++) {
        const er_shape* sh = &s->objects[i].shape;
        scatter_event local; se_invalid(&local, 2);
        local.object_id = i;
        const ray_t Rt = xform_ray(sh->inv_tm, R);
        isect_t Int; isect_invalid(&Int);
        intersect_shape(sh, &Rt, &Int);
        if (Int.valid) {
            local.valid = 1;
            local.N = xform_vector(sh->tm, Int.N);
            local.P = xform_point(sh->tm, Int.P);
            local.T = vlen(vsub(local.P, R->O));
            local.Wo = vneg(R->D);
            local.Le = C3(0, 0, 0);
            local.UV = Int.UV;
        }
        if (local.valid && local.T < T) { *RS = local; T = local.T; }
    }
}

/* IntersectsObject - Source/objects.h:64-80 */
static int intersects_object(const or_scene* s, const ray_t* R)
{
    for (int i = 0; i < s->object_count && i < s->n_objects; i++) {
        const er_shape* sh = &s->objects[i].shape;
        const ray_t Rt = xform_ray(sh->inv_tm, R);
        isect_t Int; isect_invalid(&Int);
        intersect_shape(sh, &Rt, &Int);
        if (Int.valid) return 1;
    }
    return 0;
}

void ER_OR(scene_set_bitmaps)(or_scene* s, const er_bitmap_desc* bitmaps, int32_t n)
{
    for (int i = 0; i < s->n_bitmaps; i++) free(s->bitmap_pixels[i]);
    free(s->bitmap_pixels);
    free(s->bitmap_res);
    s->n_bitmaps = n > 0 ? n : 0;
    s->bitmap_pixels = NULL;
    s->bitmap_res = NULL;
    if (!s->n_bitmaps) return;
    s->bitmap_pixels = (uint8_t**)calloc((size_t)n, sizeof(uint8_t*));
    s->bitmap_res = (int*)calloc(2 * (size_t)n, sizeof(int));
    for (int i = 0; i < n; i++) {
        const size_t bytes = 4 * (size_t)bitmaps[i].resolution[0] * (size_t)bitmaps[i].resolution[1];
        s->bitmap_res[2 * i] = bitmaps[i].resolution[0];
        s->bitmap_res[2 * i + 1] = bitmaps[i].resolution[1];
        s->bitmap_pixels[i] = (uint8_t*)malloc(bytes ? bytes : 1);
        if (bytes) memcpy(s->bitmap_pixels[i], bitmaps[i].pixels, bytes);
    }
}

void ER_OR(scene_set_objects)(or_scene* s, const er_object_desc* objects, int32_t n)
{
    free(s->objects);
    s->objects = NULL;
    s->n_objects = n > 0 ? n : 0;
    if (s->n_objects) {
        s->objects = (er_object_desc*)malloc(sizeof(er_object_desc) * (size_t)n);
        memcpy(s->objects, objects, sizeof(er_object_desc) * (size_t)n);
    }
}

/* BindClippingObject for the scene: clipping object i of `clips` has ID i;
   the tracer's ClippingObjectIDs (Source/ertracer.h:100-116) name the ones
   applied, IDs without a clipping object are skipped */
void ER_OR(scene_set_clipping_objects)(or_scene* s, const er_clipping_object_desc* clips, int32_t n)
{
    free(s->clips);
    s->clips = NULL;
    s->n_clips = 0;
    if (n <= 0) return;
    s->clips = (er_clipping_object_desc*)malloc(sizeof(er_clipping_object_desc) * (size_t)ER_MAX_INDICES);
    for (int i = 0; i < s->clip_ids_count; i++) {
        const int id = s->clip_ids[i];
        if (id < 0 || id >= n) continue;
        s->clips[s->n_clips++] = clips[id];
    }
}

/* Clipping objects: ErClippingObject is a Shape and Invert
   (Source/erclippingobject.h:27-58), bound (Source/core.cu:96-104) but read
   by no transport code of the reference.  Here a point of the volume is
   clipped - its extinction counts as zero in free flight and shadow rays,
   and no lookup is made - when it lies inside a clipping object's shape
   (outside it when Invert is set); any one object clips.  Inside is tested
   in the shape's local frame (InvTM) with the reference's predicates:
   InsidePlane (Source/plane.h:90-93, also for disks and rings), InsideBox
   (Source/box.h:116-120), InsideSphere (Source/sphere.h:147-150) and
   InsideCylinder (Source/cylinder.h:96-99) with radius OuterRadius and
   height Size[2] (the height Shape::Update uses, Source/shape.h:100). */
static int clipped(const or_scene* s, v3 p)
{
    for (int i = 0; i < s->n_clips; i++) {
        const er_clipping_object_desc* c = &s->clips[i];
        const v3 q = xform_point(c->shape.inv_tm, p);
        int in;
        switch (c->shape.type) {
        case ER_SHAPE_PLANE: case ER_SHAPE_DISK: case ER_SHAPE_RING: in = q.z > 0.0f; break;
        case ER_SHAPE_BOX: {
            const float h0 = 0.5f * c->shape.size[0], h1 = 0.5f * c->shape.size[1], h2 = 0.5f * c->shape.size[2];
            in = q.x > -h0 && q.x < h0 && q.y > -h1 && q.y < h1 && q.z > -h2 && q.z < h2;
            break;
        }
        case ER_SHAPE_SPHERE: in = vlen(q) < c->shape.outer_radius; break;
        case ER_SHAPE_CYLINDER:
            in = sqrtf((q.x * q.x) + (q.z * q.z)) < c->shape.outer_radius && fabsf(q.y) < (0.5f * c->shape.size[2]);
            break;
        default: in = 0; break;
        }
        if (in != (c->invert != 0)) return 1;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* extension estimators (settings fields apply_shading_type, mis,        */
/* free_flight of er_capi.h).  The reference has no live code for these; */
/* the designs are Source/scatterevent.h:155-212 (shader selection),     */
/* Source/transport.h:86-112 (BSDF-sampling half) and                    */
/* Source/raymarching.h:115-273 (macrocell delta tracking).              */
/* ------------------------------------------------------------------ */

static inline float sigma_lookup(const or_scene* s, float I)
{
    int i = (int)I;
    i = i < 0 ? 0 : (i > (int)s->vmax ? (int)s->vmax : i);
    return s->sigma[i];
}

/* 3D DDA over the majorant bricks, in local voxel units (the mapping of
   Volume::operator(), Source/volume.h:131-138) */
typedef struct {
    float t, tmax;
    int b[3], step[3];
    float tnext[3], tdelta[3];
    int done;
} dda_t;

static void dda_init(const or_scene* s, const ray_t* R, float t0, float t1, dda_t* d)
{
    const float B = (float)s->brick;
    d->t = t0;
    d->tmax = t1;
    d->done = 0;
    for (int i = 0; i < 3; i++) {
        const float sc = vget(s->inv_size, i) * (float)s->res[i];
        const float lo = (vget(R->O, i) - vget(s->minp, i)) * sc;
        const float ld = vget(R->D, i) * sc;
        const float L = lo + t0 * ld;
        int b = (int)floorf(L / B);
        b = b < 0 ? 0 : (b >= s->nb[i] ? s->nb[i] - 1 : b);
        d->b[i] = b;
        if (ld > 0.0f) { d->step[i] = 1; d->tnext[i] = ((float)(b + 1) * B - lo) / ld; d->tdelta[i] = B / ld; }
        else if (ld < 0.0f) { d->step[i] = -1; d->tnext[i] = ((float)b * B - lo) / ld; d->tdelta[i] = -B / ld; }
        else { d->step[i] = 0; d->tnext[i] = FLT_MAX; d->tdelta[i] = FLT_MAX; }
    }
}

static inline float dda_exit(const dda_t* d)
{
    float e = d->tnext[0];
    if (d->tnext[1] < e) e = d->tnext[1];
    if (d->tnext[2] < e) e = d->tnext[2];
    if (d->tmax < e) e = d->tmax;
    return e < d->t ? d->t : e;
}

static inline void dda_advance(const or_scene* s, dda_t* d, float e)
{
    if (e >= d->tmax) { d->done = 1; d->t = e; return; }
    int a = 0;
    if (d->tnext[1] < d->tnext[a]) a = 1;
    if (d->tnext[2] < d->tnext[a]) a = 2;
    d->b[a] += d->step[a];
    if (d->b[a] < 0 || d->b[a] >= s->nb[a]) d->done = 1;
    d->tnext[a] += d->tdelta[a];
    d->t = e;
}

static inline float dda_majorant(or_scene* s, const dda_t* d)
{
    s->stat[OR_STAT_MAJORANT]++;
    return s->majorant[((size_t)d->b[2] * (size_t)s->nb[1] + (size_t)d->b[1]) * (size_t)s->nb[0] + (size_t)d->b[0]];
}

/* Empty-space jump (exposure-render_gb300/csrc/er_path.cuh dda_jump): an
   empty brick holding -k (k >= 2, its Chebyshev distance in bricks to the
   nearest non-empty brick, see empty_skip_distances) lies in a cube of
   empty bricks of half-width k-1; the DDA moves to that cube's exit in one
   step.  Exit face per axis at next + (k-1) * delta; the earliest (ties to
   x, then y) moves its axis k bricks, each other axis moves past the
   floor((te - next) / delta) + 1 faces (at most k) it crosses before te.
   The same float operations as the GPU, in the same order. */
static inline void dda_jump(const or_scene* s, dda_t* d, int k)
{
    const float r = (float)(k - 1);
    float f[3];
    for (int i = 0; i < 3; i++) f[i] = d->step[i] != 0 ? d->tnext[i] + r * d->tdelta[i] : FLT_MAX;
    int a = 0;
    if (f[1] < f[a]) a = 1;
    if (f[2] < f[a]) a = 2;
    const float te = f[a];
    if (te >= d->tmax) { d->done = 1; d->t = te; return; }
    for (int i = 0; i < 3; i++) {
        if (i == a) {
            d->b[i] += d->step[i] * k;
            d->tnext[i] = f[i] + d->tdelta[i];
        } else if (d->tnext[i] < te) {
            int m = (int)((te - d->tnext[i]) / d->tdelta[i]) + 1;
            m = m > k ? k : m;
            d->b[i] += d->step[i] * m;
            d->tnext[i] = d->tnext[i] + (float)m * d->tdelta[i];
        }
    }
    for (int i = 0; i < 3; i++)
        if (d->b[i] < 0 || d->b[i] >= s->nb[i]) d->done = 1;
    d->t = te;
}

/* extinction at a tentative collision of a tracker in DDA brick b
   (exposure-render_gb300/csrc/er_path.cuh sigma_point_in_brick): the local
   coordinates are clamped to [b B, (b + 1) B] per axis before the lookup, so
   that it blends only voxels of the brick's footprint, which the majorant
   bounds; zero where a clipping object removes the volume */
static inline float sigma_in_brick(or_scene* s, v3 P, const dda_t* d)
{
    if (s->n_clips && clipped(s, P)) return 0.0f;
    v3 L = local_coords(s, P);
    const float B = (float)s->brick;
    const float x0 = (float)d->b[0] * B, y0 = (float)d->b[1] * B, z0 = (float)d->b[2] * B;
    const float x1 = x0 + B, y1 = y0 + B, z1 = z0 + B;
    L.x = L.x < x0 ? x0 : (x1 < L.x ? x1 : L.x);
    L.y = L.y < y0 ? y0 : (y1 < L.y ? y1 : L.y);
    L.z = L.z < z0 ? z0 : (z1 < L.z ? z1 : L.z);
    return s->st.density_scale * sigma_lookup(s, get_intensity_local(s, L));
}

#define ER_DELTA_MAX_COLLISIONS 1048576

/* Delta tracking of the primary ray.  sigma_t(x) = DensityScale *
   DensityScale * Opacity(I(x)) is the extinction the reference's march
   integrates: Sum += DS*Op*Step against S = -ln(U)/DS
   (Source/raymarching.h:45,64-66).  The event is the accepted collision
   itself (the march reports one step past it, :66-70). */
static void sample_volume_delta(or_scene* s, ray_t R, rng_t* rng, scatter_event* SE)
{
    isect_t Int; isect_invalid(&Int);
    intersect_box(&R, s->minp, vscale(s->size, 0.5f), &Int);
    if (!Int.valid) return;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return;
    dda_t d;
    dda_init(s, &R, t0, t1, &d);
    const float u0 = rng_get1(rng);
    float tau = -er_logf(s->tau_u >= 0.0f ? (float)s->tau_u : u0);
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(&d);
        const float mu = dda_majorant(s, &d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 P = vadd(R.O, vscale(R.D, t));
                const float sig = sigma_in_brick(s, P, &d);
                if (rng_get1(rng) * mu < sig) {
                    SE->valid = 1;
                    SE->T = t;
                    SE->P = P;
                    SE->N = normalized_gradient(s, P);
                    SE->Wo = vneg(R.D);
                    SE->Le = C3(0, 0, 0);
                    SE->UV.x = 0.0f; SE->UV.y = 0.0f;
                    return;
                }
                if (++guard > ER_DELTA_MAX_COLLISIONS) return;
                tau = -er_logf(rng_get1(rng));
            }
        } else if (mu <= -2.0f) {
            dda_jump(s, &d, (int)(-mu));
            continue;
        }
        dda_advance(s, &d, e);
    }
}

/* Ratio tracking of a shadow segment with Russian roulette below 0.1 */
static float transmittance_ratio(or_scene* s, ray_t R, rng_t* rng)
{
    isect_t Int; isect_invalid(&Int);
    intersect_box(&R, s->minp, vscale(s->size, 0.5f), &Int);
    if (!Int.valid) return 1.0f;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return 1.0f;
    dda_t d;
    dda_init(s, &R, t0, t1, &d);
    float Tr = 1.0f;
    float tau = -er_logf(rng_get1(rng));
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(&d);
        const float mu = dda_majorant(s, &d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 P = vadd(R.O, vscale(R.D, t));
                const float sig = sigma_in_brick(s, P, &d);
                Tr = Tr * (1.0f - sig / mu);
                if (Tr <= 0.0f) return 0.0f;
                if (Tr < 0.1f) {
                    if (rng_get1(rng) >= 0.5f) return 0.0f;
                    Tr = Tr * 2.0f;
                }
                if (++guard > ER_DELTA_MAX_COLLISIONS) return Tr;
                tau = -er_logf(rng_get1(rng));
            }
        } else if (mu <= -2.0f) {
            dda_jump(s, &d, (int)(-mu));
            continue;
        }
        dda_advance(s, &d, e);
    }
    return Tr;
}

/* Intersect / Visible - Source/transport.h:30-56 (no surface objects):
   1/0 for the reference march, the ratio-tracked transmittance otherwise */
static float visibility_segment(or_scene* s, v3 P1, v3 P2, rng_t* rng);
static float visibility(or_scene* s, v3 P1, v3 P2, rng_t* rng)
{
    const uint64_t lk = s->lookups, mj = s->stat[OR_STAT_MAJORANT];
    s->stat[OR_STAT_SHADOW_RAYS]++;
    const float v = visibility_segment(s, P1, P2, rng);
    s->stat[OR_STAT_SHADOW_LOOKUPS] += s->lookups - lk;
    s->stat[OR_STAT_SHADOW_MAJORANT] += s->stat[OR_STAT_MAJORANT] - mj;
    return v;
}
static float visibility_segment(or_scene* s, v3 P1, v3 P2, rng_t* rng)
{
    if (!s->st.shadows) return 1.0f;
    const v3 W = vnorm(vsub(P2, P1));
    ray_t R;
    R.O = vadd(P1, vscale(W, RAY_EPS));
    R.D = W;
    R.MinT = 0.0f;
    R.MaxT = smin(vlen(vsub(P2, P1)) - 2.0f * RAY_EPS, s->st.max_shadow_distance);
    if (intersects_light(s, &R)) return 0.0f;
    if (intersects_object(s, &R)) return 0.0f;
    if (s->st.free_flight == ER_FREE_FLIGHT_DELTA) return transmittance_ratio(s, R, rng);
    return scatter_event_in_volume(s, R, rng) ? 0.0f : 1.0f;
}

/* shader selection of the commented design Source/scatterevent.h:155-212:
   0 = BRDF, 1 = isotropic phase; GradientMagnitudeRange.Inv is 1 / the
   maximum voxel-centre gradient magnitude of the pre-pass */
static int select_shader_type(or_scene* s, const scatter_event* SE, float I, rng_t* rng)
{
    switch (s->st.shading_type) {
    case ER_SHADING_BRDF_ONLY: return 0;
    case ER_SHADING_PHASE_ONLY: return 1;
    case ER_SHADING_HYBRID: {
        const float NGM = gradient_magnitude(s, SE->P) * s->gm_inv_max;
        const float Exponent = 25.0f * er_powf(s->st.gradient_factor, 3.0f) * NGM;
        const float PdfBrdf = s->st.opacity_modulated ? plf_eval(&s->opacity, I) * (1.0f - er_expf(-Exponent))
                                                      : 1.0f - er_expf(-Exponent);
        return rng_get1(rng) <= PdfBrdf ? 0 : 1;
    }
    case ER_SHADING_MODULATION: {
        const float NGM = gradient_magnitude(s, SE->P) * s->gm_inv_max;
        const float PdfBrdf = 1.0f - er_powf(1.0f - NGM, 2.0f);
        return rng_get1(rng) < PdfBrdf ? 0 : 1;
    }
    case ER_SHADING_THRESHOLD: {
        const float NGM = gradient_magnitude(s, SE->P) * s->gm_inv_max;
        return NGM > s->st.gradient_threshold ? 0 : 1;
    }
    default: return 1;
    }
}

#define INV_FOUR_PI_TRUE 0.0795774715f

/* pdf of the BSDF sampler of the full-MIS estimator: the equal-weight
   mixture of Lambertian and Blinn lobes for the BRDF (BRDF::SampleF picks
   each with probability 1/2, Source/shader.h:364-371), 1/(4 pi) for the
   uniform sphere sampler of IsotropicPhase::SampleF (:293-299) */
static float mis_bsdf_pdf(const shader_t* sh, v3 Wo, v3 Wi)
{
    if (sh->type == 0) {
        const v3 Wol = world_to_local(sh, Wo), Wil = world_to_local(sh, Wi);
        const float pl = same_hemisphere(Wol, Wil) ? fabsf(Wil.z) * INV_PI_F : 0.0f;
        const float pm = same_hemisphere(Wol, Wil) ? blinn_pdf(sh->exponent, Wol, Wil) : 0.0f;
        return 0.5f * (pl + pm);
    }
    return INV_FOUR_PI_TRUE;
}

/* Lambertian::SampleF (Source/shader.h:46-56), Blinn::SampleF (:142-164)
   with the component choice of BRDF::SampleF (:364-371); the sphere sampler
   of IsotropicPhase::SampleF (:293-299, Source/montecarlo.h:191-199) */
static v3 sample_bsdf_dir(const shader_t* sh, v3 Wo, const metro_sample* ms)
{
    if (sh->type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        v3 Wil;
        if (ms->brdf_component <= 0.5f) {
            const v2 d = concentric_sample_disk(ms->brdf_dir);
            Wil = V3(d.x, d.y, sqrtf(smax(0.f, 1.f - d.x * d.x - d.y * d.y)));
            if (Wol.z < 0.0f) Wil.z *= -1.0f;
        } else {
            const float e = sh->exponent;
            const float costheta = er_powf(ms->brdf_dir.x, 1.f / (e + 1));
            const float sintheta = sqrtf(smax(0.f, 1.f - costheta * costheta));
            const float phi = ms->brdf_dir.y * 2.f * PI_F;
            float sn, cs;
            er_sincosf(phi, &sn, &cs);
            v3 wh = V3(sintheta * cs, sintheta * sn, costheta);
            if (!same_hemisphere(Wol, wh)) wh = vneg(wh);
            Wil = vadd(vneg(Wol), vscale(wh, 2.f * vdot(Wol, wh)));
        }
        return local_to_world(sh, Wil);
    }
    const float z = 1.f - 2.f * ms->brdf_dir.x;
    const float r = sqrtf(smax(0.f, 1.f - z * z));
    const float phi = 2.f * PI_F * ms->brdf_dir.y;
    float sn, cs;
    er_sincosf(phi, &sn, &cs);
    return V3(r * cs, r * sn, z);
}

/* SampleLight - Source/lights.h:44-57 */
static void sample_light(const or_scene* s, const or_light* L, v3 uvw, surf_sample* SS, const scatter_event* SE,
                         v3* Wi, col3* Le)
{
    sample_light_surface(L, uvw, SS);
    *Wi = vnorm(vsub(SS->P, SE->P));
    *Le = cscale(evaluate_texture(s, L->d.texture_id, SS->UV), L->d.multiplier);
    if (L->d.shape.one_sided && vdot(vsub(SE->P, SS->P), SS->N) < 0.0f) *Le = C3(0, 0, 0);
    if (L->d.unit == 1) *Le = cdivs(*Le, L->area);
}

/* EstimateDirectLight - Source/transport.h:58-113.  With mis = 0 and the
   fixed-step march this is the live code (the function returns at :84).
   With mis = 1 the BSDF-sampling half of :86-112 runs as well, both halves
   weighted by the power heuristic over (light pdf, mixture BSDF pdf), and
   the light pdf of the BSDF half uses the light's surface normal at the hit
   (the design divides by |N . -Wi| with the scatter point's normal, :102).
   With delta tracking the shadow term is the ratio-tracked transmittance. */
static col3 estimate_direct_light(or_scene* s, const or_light* L, int slot, const metro_sample* ms, scatter_event* SE,
                                  rng_t* rng, const shader_t* sh)
{
    v3 Wi;
    col3 Li, Ld = C3(0, 0, 0);
    surf_sample SS;
    sample_light(s, L, ms->light_uvw, &SS, SE, &Wi, &Li);
    const col3 F = shader_f(sh, SE->Wo, Wi);
    const int full = s->st.mis == ER_MIS_FULL;
    const int delta = s->st.free_flight == ER_FREE_FLIGHT_DELTA;
    const float BsdfPdf = full ? mis_bsdf_pdf(sh, SE->Wo, Wi) : shader_pdf(sh, SE->Wo, Wi);
    if (!full && !delta) {
        if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f && visibility(s, SE->P, SS.P, rng) > 0.0f) {
            const float LightPdf = vlen2(vsub(SE->P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L->area);
            const float Weight = power_heuristic(LightPdf, BsdfPdf);
            if (sh->type == 0) Ld = cadd(Ld, cscale(cmul(F, Li), vabsdot(Wi, SE->N) * Weight / LightPdf));
            else Ld = cadd(Ld, cdivs(cmul(F, Li), LightPdf));
        }
        return Ld;
    }
    if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f) {
        const float Tr = visibility(s, SE->P, SS.P, rng);
        if (Tr > 0.0f) {
            const float LightPdf = vlen2(vsub(SE->P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L->area);
            col3 c;
            if (full) {
                const float w = power_heuristic(LightPdf, BsdfPdf);
                c = cscale(cmul(F, Li), sh->type == 0 ? vabsdot(Wi, SE->N) * w / LightPdf : w / LightPdf);
            } else if (sh->type == 0) {
                c = cscale(cmul(F, Li), vabsdot(Wi, SE->N) * power_heuristic(LightPdf, BsdfPdf) / LightPdf);
            } else {
                c = cdivs(cmul(F, Li), LightPdf);
            }
            Ld = cadd(Ld, cscale(c, Tr));
        }
    }
    if (!full) return Ld;
    const v3 Wb = sample_bsdf_dir(sh, SE->Wo, ms);
    const col3 Fb = shader_f(sh, SE->Wo, Wb);
    const float pb = mis_bsdf_pdf(sh, SE->Wo, Wb);
    if (cblack(Fb) || !(pb > 0.0f)) return Ld;
    ray_t R2;
    R2.O = SE->P;
    R2.D = Wb;
    R2.MinT = 0.0f;
    R2.MaxT = 1000000.0f;                 /* Ray(SE.P, Wi) defaults, Source/ray.h:29 */
    scatter_event SE2;
    se_invalid(&SE2, 1);
    intersect_lights(s, &R2, &SE2, 0);
    if (!SE2.valid || s->light_idx[SE2.light_id] != s->light_idx[slot]) return Ld;
    if (cblack(SE2.Le)) return Ld;
    const float Tr = visibility(s, SE->P, SE2.P, rng);
    if (Tr > 0.0f) {
        const float LightPdf = vlen2(vsub(SE->P, SE2.P)) / (vabsdot(SE2.N, vneg(Wb)) * L->area);
        const float w = power_heuristic(pb, LightPdf);
        const col3 c = cscale(cmul(Fb, SE2.Le), sh->type == 0 ? vabsdot(Wb, SE->N) * w / pb : w / pb);
        Ld = cadd(Ld, cscale(c, Tr));
    }
    return Ld;
}

/* UniformSampleOneLight - Source/transport.h:115-156 (volume events) */
static col3 uniform_sample_one_light(or_scene* s, scatter_event* SE, rng_t* rng, const metro_sample* ms)
{
    col3 Ld = C3(0, 0, 0);
    const float I = get_intensity(s, SE->P);
    Ld = cadd(Ld, ctf_eval(&s->emission, I));
    if (s->light_count <= 0) return Ld;
    const int idx = (int)floorf(ms->light_num * (float)s->light_count);
    const int light_id = s->light_idx[idx];
    if (light_id < 0) return Ld;
    if (light_id >= s->n_lights) return Ld;
    const or_light* L = &s->lights[light_id];
    shader_t sh;
    if (SE->type == 2) {
        /* Source/transport.h:141-149: the object's textures at the hit, IOR 15,
           exponent from the glossiness texture's luminance */
        const er_object_desc* o = &s->objects[SE->object_id];
        const col3 Kd = evaluate_texture(s, o->diffuse_texture_id, SE->UV);
        const col3 Ks = evaluate_texture(s, o->specular_texture_id, SE->UV);
        const col3 G = evaluate_texture(s, o->glossiness_texture_id, SE->UV);
        float Y = 0.0f;
        Y += 0.212671f * G.c[0];
        Y += 0.715160f * G.c[1];
        Y += 0.072169f * G.c[2];
        shader_init(&sh, 0, SE->N, SE->Wo, Kd, Ks, 15.0f, glossiness_exponent(Y));
    } else {
        const float vol_ior = s->st.volume_ior > 0.0f ? s->st.volume_ior : 15.0f;
        const int type = s->st.apply_shading_type ? select_shader_type(s, SE, I, rng) : 0;
        shader_init(&sh, type, SE->N, SE->Wo, ctf_eval(&s->diffuse, I), ctf_eval(&s->specular, I), vol_ior,
                    glossiness_exponent(plf_eval(&s->glossiness, I)));
    }
    Ld = cadd(Ld, estimate_direct_light(s, L, idx, ms, SE, rng, &sh));
    return cscale(Ld, (float)s->light_count);
}

/* ---- per-scene tables of the extension estimators ---- */

typedef struct { or_scene* s; int z0, z1; float mx; } gm_job;

static void* gm_run(void* arg)
{
    gm_job* j = (gm_job*)arg;
    or_scene local = *j->s;
    float mx = 0.0f;
    for (int Z = j->z0; Z < j->z1; Z++)
        for (int Y = 0; Y < local.res[1]; Y++)
            for (int X = 0; X < local.res[0]; X++) {
                const float sx = 2.0f * (local.size.x * 0.5f), sy = 2.0f * (local.size.y * 0.5f), sz = 2.0f * (local.size.z * 0.5f);
                const v3 p = V3(local.minp.x + sx * (((float)X + 0.5f) * (1.0f / (float)local.res[0])),
                                local.minp.y + sy * (((float)Y + 0.5f) * (1.0f / (float)local.res[1])),
                                local.minp.z + sz * (((float)Z + 0.5f) * (1.0f / (float)local.res[2])));
                const float g = gradient_magnitude(&local, p);
                mx = g > mx ? g : mx;
            }
    j->mx = mx;
    return NULL;
}

static float gradient_magnitude_max_threaded(or_scene* s, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > s->res[2]) nthreads = s->res[2];
    gm_job* jobs = (gm_job*)calloc((size_t)nthreads, sizeof(gm_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t].s = s;
        jobs[t].z0 = (int)((long long)s->res[2] * t / nthreads);
        jobs[t].z1 = (int)((long long)s->res[2] * (t + 1) / nthreads);
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, gm_run, &jobs[t]);
    gm_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    float mx = 0.0f;
    for (int t = 0; t < nthreads; t++) mx = jobs[t].mx > mx ? jobs[t].mx : mx;
    free(jobs);
    free(th);
    return mx;
}

/* Empty-space distances (exposure-render_gb300/csrc/er_volume.cu
   k_skip_pass): for each empty brick (majorant 0) the Chebyshev distance
   in bricks to the nearest non-empty brick, capped at 32, by three 1D
   passes -- x: distance to the nearest non-empty brick of the row (0 for a
   non-empty brick, 32 when none is within 31); y, then z: the minimum over
   offsets o of max(|o|, previous pass at o).  Empty bricks then hold minus
   that distance. */
#define ER_SKIP_CAP 32
static void empty_skip_distances(float* majorant, const int nb[3])
{
    const size_t total = (size_t)nb[0] * nb[1] * nb[2];
    uint8_t* a = (uint8_t*)malloc(total);
    uint8_t* b = (uint8_t*)malloc(total);
    for (int axis = 0; axis < 3; axis++) {
        const uint8_t* in = axis == 1 ? a : b;
        uint8_t* out = axis == 1 ? b : a;
        const size_t step = axis == 0 ? 1 : (axis == 1 ? (size_t)nb[0] : (size_t)nb[0] * nb[1]);
        for (size_t i = 0; i < total; i++) {
            const int c0[3] = { (int)(i % nb[0]), (int)((i / nb[0]) % nb[1]), (int)(i / ((size_t)nb[0] * nb[1])) };
            int best = ER_SKIP_CAP;
            for (int o = -(ER_SKIP_CAP - 1); o <= ER_SKIP_CAP - 1; o++) {
                const int c = c0[axis] + o;
                if (c < 0 || c >= nb[axis]) continue;
                const int ao = o < 0 ? -o : o;
                if (ao >= best) continue;
                const size_t j = (size_t)((long long)i + (long long)o * (long long)step);
                const int v = axis == 0 ? (majorant[j] > 0.0f ? 0 : ER_SKIP_CAP) : (int)in[j];
                const int dd = v > ao ? v : ao;
                best = dd < best ? dd : best;
            }
            out[i] = (uint8_t)best;
        }
    }
    for (size_t i = 0; i < total; i++)
        if (!(majorant[i] > 0.0f)) majorant[i] = -(float)a[i];
    free(a);
    free(b);
}

static void prepare_extensions(or_scene* s)
{
    const size_t n = (size_t)s->res[0] * (size_t)s->res[1] * (size_t)s->res[2];
    uint16_t vmax = 0;
    for (size_t i = 0; i < n; i++) vmax = s->vox[i] > vmax ? s->vox[i] : vmax;
    s->vmax = vmax;
    s->sigma = (float*)malloc(sizeof(float) * ((size_t)vmax + 1));
    for (int i = 0; i <= (int)vmax; i++) s->sigma[i] = s->st.density_scale * plf_eval(&s->opacity, (float)i);
    if (s->st.free_flight == ER_FREE_FLIGHT_DELTA) {
        const int B = s->st.majorant_brick > 0 ? s->st.majorant_brick : 8;
        s->brick = B;
        for (int i = 0; i < 3; i++) s->nb[i] = (s->res[i] + B - 1) / B;
        const size_t nbt = (size_t)s->nb[0] * s->nb[1] * s->nb[2];
        s->majorant = (float*)malloc(sizeof(float) * nbt);
        for (int bz = 0; bz < s->nb[2]; bz++)
            for (int by = 0; by < s->nb[1]; by++)
                for (int bx = 0; bx < s->nb[0]; bx++) {
                    /* voxel footprint of the brick: b B .. (b + 1) B per axis
                       (the trackers clamp their lookups to [b B, (b + 1) B]) */
                    int lo[3], hi[3];
                    const int b[3] = { bx, by, bz };
                    for (int i = 0; i < 3; i++) {
                        lo[i] = b[i] * B;
                        hi[i] = (b[i] + 1) * B;
                        hi[i] = hi[i] > s->res[i] - 1 ? s->res[i] - 1 : hi[i];
                    }
                    uint16_t vlo = 65535, vhi = 0;
                    for (int z = lo[2]; z <= hi[2]; z++)
                        for (int y = lo[1]; y <= hi[1]; y++)
                            for (int x = lo[0]; x <= hi[0]; x++) {
                                const uint16_t v = s->vox[(size_t)z * s->res[0] * s->res[1] + (size_t)y * s->res[0] + x];
                                vlo = v < vlo ? v : vlo;
                                vhi = v > vhi ? v : vhi;
                            }
                    /* a truncated blend can land one intensity below the
                       smallest corner (float rounding of (1 - t) a + t b) */
                    float m = 0.0f;
                    for (int i = vlo > 0 ? (int)vlo - 1 : 0; i <= (int)vhi; i++) m = s->sigma[i] > m ? s->sigma[i] : m;
                    s->majorant[((size_t)bz * s->nb[1] + by) * s->nb[0] + bx] = s->st.density_scale * m;
                }
        empty_skip_distances(s->majorant, s->nb);
    }
    s->gm_inv_max = 0.0f;
    s->gm_ready = 0;
    if (s->st.apply_shading_type && s->st.shading_type >= ER_SHADING_HYBRID && s->st.shading_type <= ER_SHADING_THRESHOLD) {
        const long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
        const float mx = gradient_magnitude_max_threaded(s, ncpu > 0 ? (int)ncpu : 8);
        s->gm_inv_max = mx > 0.0f ? 1.0f / mx : 0.0f;
        s->gm_ready = 1;
    }
}

/* SampleCamera - Source/singlescattering.h:29-50 */
static ray_t sample_camera(const or_scene* s, int u, int v, v2 film_uv, v2 lens_uv)
{
    ray_t R;
    const float sp0 = s->screen[0][0] + (s->inv_screen[0] * ((float)u + film_uv.x * 1.0f / (float)s->film[0]));
    const float sp1 = s->screen[1][0] + (s->inv_screen[1] * ((float)v + film_uv.y * 1.0f / (float)s->film[1]));
    R.O = s->pos;
    R.D = vnorm(vsub(vadd(s->N, vscale(s->U, sp0)), vscale(s->V, sp1)));
    R.MinT = s->clip_near;
    R.MaxT = s->clip_far;
    if (s->aperture != 0.0f) {
        const v2 d = concentric_sample_disk(lens_uv);
        const v2 lens = { d.x * s->aperture, d.y * s->aperture };
        const v3 LI = vadd(vscale(s->U, lens.x), vscale(s->V, lens.y));
        R.O = vadd(R.O, LI);
        R.D = vnorm(vsub(vscale(R.D, s->focal_distance), LI));
    }
    return R;
}

/* SampleRay - Source/singlescattering.h:52-74: volume, light and object events, nearest wins */
static void sample_ray(or_scene* s, ray_t R, rng_t* rng, scatter_event* nearest)
{
    scatter_event se[3];
    se_invalid(&se[0], 0);
    se_invalid(&se[1], 1);
    se_invalid(&se[2], 2);
    if (s->st.free_flight == ER_FREE_FLIGHT_DELTA) sample_volume_delta(s, R, rng, &se[0]);
    else sample_volume(s, R, rng, &se[0]);
    intersect_lights(s, &R, &se[1], 1);
    intersect_objects(s, &R, &se[2]);
    float T = FLT_MAX;
    se_invalid(nearest, 0);
    for (int i = 0; i < 3; i++) {
        if (se[i].valid && se[i].T < T) { *nearest = se[i]; T = se[i].T; }
    }
}

/* SingleScattering - Source/singlescattering.h:76-102 */
/* `sample` (view, pixel, sample index) identifies a sample of a
   multi-sample render, NULL for a frame; with settings.stratify the light
   sample's (u, v), the light choice, the BSDF sample and the first
   free-flight draw of delta tracking come from er_stratified_sample (the
   random stream still draws them first, so every later draw is unchanged) */
typedef struct { uint32_t view, pixel, index; } sample_id;

static void single_scattering(or_scene* s, int x, int y, rng_t* rng, float out[4], const sample_id* sample)
{
    col3 Lv = C3(0, 0, 0);
    metro_sample ms;
    metro_large_step(&ms, rng);
    s->tau_u = -1.0f;
    if (sample && s->st.stratify) {
        desc_f32 u[7];
        er_stratified_sample(s->st.seed, sample->view, sample->pixel, sample->index, u);
        ms.light_uvw.x = u[0];
        ms.light_uvw.y = u[1];
        ms.light_num = u[2];
        ms.brdf_dir.x = u[3];
        ms.brdf_dir.y = u[4];
        ms.brdf_component = u[5];
        s->tau_u = u[6];
    }
    const ray_t R = sample_camera(s, x, y, ms.film_uv, ms.lens_uv);
    scatter_event SE;
    const uint64_t lk = s->lookups;
    sample_ray(s, R, rng, &SE);
    s->stat[OR_STAT_FREE_FLIGHT_LOOKUPS] += s->lookups - lk;
    if (SE.valid && SE.type == 0) s->stat[OR_STAT_EVENTS]++;
    if (SE.valid && SE.type == 0) Lv = cadd(Lv, uniform_sample_one_light(s, &SE, rng, &ms));
    if (SE.valid && SE.type == 1) Lv = cadd(Lv, SE.Le);
    if (SE.valid && SE.type == 2) Lv = cadd(Lv, uniform_sample_one_light(s, &SE, rng, &ms));
    out[0] = Lv.c[0];
    out[1] = Lv.c[1];
    out[2] = Lv.c[2];
    out[3] = SE.valid ? 1.0f : 0.0f;
}

/* KrnlComputeAutoFocusDistance - Source/autofocus.cuh:26-62: 100 rays
   through the screen point of film pixel (u, v) (no film jitter), each
   moved by 0.01 x ConcentricSampleDisk(Get2()), pinhole, traced by the
   fixed-step march; the mean distance from the camera to the scatter
   event.  The event is not reset between rays, so after the first hit a
   ray that misses adds the previous hit's distance again; with no hit at
   all the result is the distance from the camera to the origin (the
   invalid event's P). */
float ER_OR(autofocus)(or_scene* s, int32_t u, int32_t v, uint32_t lane0, uint32_t lane1)
{
    rng_t rng;
    rng.s0 = lane0;
    rng.s1 = lane1;
    scatter_event SE;
    se_invalid(&SE, 0);
    ray_t Rc;
    Rc.O = s->pos; Rc.D = s->N; Rc.MinT = s->clip_near; Rc.MaxT = s->clip_far;
    float Sum = 0.0f, SumWeight = 0.0f;
    for (int i = 0; i < 100; i++) {
        float sp0 = s->screen[0][0] + (s->inv_screen[0] * (float)u);
        float sp1 = s->screen[1][0] + (s->inv_screen[1] * (float)v);
        const v2 d = concentric_sample_disk(rng_get2(&rng));
        sp0 += 0.01f * d.x;
        sp1 += 0.01f * d.y;
        Rc.O = s->pos;
        Rc.D = vnorm(vsub(vadd(s->N, vscale(s->U, sp0)), vscale(s->V, sp1)));
        Rc.MinT = s->clip_near;
        Rc.MaxT = s->clip_far;
        sample_volume(s, Rc, &rng, &SE);
        if (SE.valid) {
            Sum += vlen(vsub(SE.P, Rc.O));
            SumWeight += 1.0f;
        }
    }
    if (Sum <= 0.0f) return vlen(vsub(SE.P, Rc.O));
    return Sum / SumWeight;
}

/* ------------------------------------------------------------------ */
/* threaded drivers                                                     */
/* ------------------------------------------------------------------ */

typedef struct {
    or_scene* scene;
    or_scene local;
    int mode;               /* 0 frame, 1 sum */
    uint32_t* lanes;
    float* out;
    float* out2;            /* sums of squares (render_moments) or NULL */
    int spp;
    uint32_t view, first;
    int x0, y0, w, h;
    int row0, row1;
} job_t;

static void* job_run(void* arg)
{
    job_t* j = (job_t*)arg;
    or_scene* s = &j->local;
    const int W = s->film[0], H = s->film[1];
    for (int r = j->row0; r < j->row1; r++) {
        if (j->mode == 0) {
            for (int x = 0; x < W; x++) {
                const size_t p = (size_t)r * (size_t)W + (size_t)x;
                rng_t rng;
                rng.s0 = j->lanes[p];
                rng.s1 = j->lanes[(size_t)W * (size_t)H + p];
                single_scattering(s, x, r, &rng, &j->out[4 * p], NULL);
                j->lanes[p] = rng.s0;
                j->lanes[(size_t)W * (size_t)H + p] = rng.s1;
                s->samples++;
            }
        } else {
            const int y = j->y0 + r;
            for (int xi = 0; xi < j->w; xi++) {
                const int x = j->x0 + xi;
                const uint32_t pix = (uint32_t)y * (uint32_t)W + (uint32_t)x;
                float acc[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
                float acc2[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
                for (int k = 0; k < j->spp; k++) {
                    rng_t rng;
                    er_seed_lanes(s->st.seed, j->view, pix, j->first + (uint32_t)k, &rng.s0, &rng.s1);
                    float o[4];
                    const sample_id sid = { j->view, pix, j->first + (uint32_t)k };
                    single_scattering(s, x, y, &rng, o, &sid);
                    acc[0] += o[0]; acc[1] += o[1]; acc[2] += o[2]; acc[3] += o[3];
                    if (j->out2) {
                        acc2[0] += o[0] * o[0]; acc2[1] += o[1] * o[1]; acc2[2] += o[2] * o[2]; acc2[3] += o[3] * o[3];
                    }
                    s->samples++;
                }
                const size_t q = 4 * ((size_t)r * (size_t)j->w + (size_t)xi);
                float* d = &j->out[q];
                d[0] = acc[0]; d[1] = acc[1]; d[2] = acc[2]; d[3] = acc[3];
                if (j->out2) {
                    float* d2 = &j->out2[q];
                    d2[0] = acc2[0]; d2[1] = acc2[1]; d2[2] = acc2[2]; d2[3] = acc2[3];
                }
            }
        }
    }
    return NULL;
}

static void run_jobs(or_scene* s, job_t* proto, int rows, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > rows) nthreads = rows > 0 ? rows : 1;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = *proto;
        jobs[t].local = *s;
        jobs[t].local.lookups = 0;
        jobs[t].local.samples = 0;
        memset(jobs[t].local.stat, 0, sizeof(jobs[t].local.stat));
        jobs[t].row0 = (int)((long long)rows * t / nthreads);
        jobs[t].row1 = (int)((long long)rows * (t + 1) / nthreads);
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, job_run, &jobs[t]);
    job_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    uint64_t lk = 0, sm = 0;
    uint64_t st[OR_NSTATS] = {0};
    for (int t = 0; t < nthreads; t++) {
        lk += jobs[t].local.lookups;
        sm += jobs[t].local.samples;
        for (int k = 0; k < OR_NSTATS; k++) st[k] += jobs[t].local.stat[k];
    }
    g_lookups_per_sample = sm ? (double)lk / (double)sm : 0.0;
    for (int k = 0; k < OR_NSTATS; k++) g_stats[k] = sm ? (double)st[k] / (double)sm : 0.0;
    free(jobs);
    free(th);
}

void ER_OR(render_frame)(or_scene* s, uint32_t* lanes, float* frame, int32_t nthreads)
{
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.scene = s; proto.mode = 0; proto.lanes = lanes; proto.out = frame;
    run_jobs(s, &proto, s->film[1], nthreads);
}

void ER_OR(render_sum)(or_scene* s, int32_t spp, uint32_t view, uint32_t first_sample,
                       int32_t x0, int32_t y0, int32_t w, int32_t h, float* sum, int32_t nthreads)
{
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.scene = s; proto.mode = 1; proto.out = sum; proto.spp = spp; proto.view = view; proto.first = first_sample;
    proto.x0 = x0; proto.y0 = y0; proto.w = w; proto.h = h;
    run_jobs(s, &proto, h, nthreads);
}

void ER_OR(render_moments)(or_scene* s, int32_t spp, uint32_t view, uint32_t first_sample,
                           int32_t x0, int32_t y0, int32_t w, int32_t h, float* sum, float* sum2, int32_t nthreads)
{
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.scene = s; proto.mode = 1; proto.out = sum; proto.out2 = sum2; proto.spp = spp; proto.view = view;
    proto.first = first_sample;
    proto.x0 = x0; proto.y0 = y0; proto.w = w; proto.h = h;
    run_jobs(s, &proto, h, nthreads);
}

double ER_OR(lookups_per_sample)(void) { return g_lookups_per_sample; }

void ER_OR(render_stats)(double* out)
{
    for (int k = 0; k < OR_NSTATS; k++) out[k] = g_stats[k];
}

/* ------------------------------------------------------------------ */
/* post-processing                                                      */
/* ------------------------------------------------------------------ */

/* Gauss2D - Source/filterframeestimate.cuh:28-31 */
static inline float gauss2d(float sigma, int X, int Y)
{
    return er_expf(-((float)(X * X + Y * Y) / (2 * sigma * sigma)));
}

/* ToneMap - Source/tonemap.cuh:30-47, alpha :58; FromXYZAf Source/color.h:155-164 */
static inline void tonemap_px(const float* R, float exposure, uint8_t* o)
{
    float rgb[3];
    rgb[0] = 3.240479f * R[0] - 1.537150f * R[1] - 0.498535f * R[2];
    rgb[1] = -0.969256f * R[0] + 1.875991f * R[1] + 0.041556f * R[2];
    rgb[2] = 0.055648f * R[0] - 0.204043f * R[1] + 1.057311f * R[2];
    for (int i = 0; i < 3; i++) {
        rgb[i] = 1.0f - er_expf(-(rgb[i] / exposure));
        rgb[i] = smax(0.0f, smin(rgb[i], 1.0f));          /* ColorRGBf::Clamp, Source/vector.h:345-350 */
        o[i] = (uint8_t)(255.0f * rgb[i]);
    }
    o[3] = (uint8_t)(R[3] * 255.0f);
}

void ER_OR(post_frame)(float* frame, float* running, uint8_t* rgba, int32_t W, int32_t H,
                       int32_t no_iterations, float exposure)
{
    float* tmp = (float*)malloc(sizeof(float) * 4 * (size_t)W * (size_t)H);
    /* KrnlFilterFrameEstimate(1, 1.0f) - Source/filterframeestimate.cuh:33-64 */
    for (int IDy = 0; IDy < H; IDy++) {
        for (int IDx = 0; IDx < W; IDx++) {
            const int KernelRadius = 1;
            const float Sigma = 1.0f;
            const int x0 = (IDx - KernelRadius) > 0 ? (IDx - KernelRadius) : 0;
            const int x1 = (IDx + KernelRadius) < (W - 1) ? (IDx + KernelRadius) : (W - 1);
            const int y0 = (IDy - KernelRadius) > 0 ? (IDy - KernelRadius) : 0;
            const int y1 = (IDy + KernelRadius) < (H - 1) ? (IDy + KernelRadius) : (H - 1);
            float sum[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
            float total = 0.0f;
            for (int y = y0; y <= y1; y++) {
                for (int x = x0; x <= x1; x++) {
                    const float w = gauss2d(Sigma, x - IDx, y - IDy);
                    const float* f = &frame[4 * ((size_t)y * W + x)];
                    for (int k = 0; k < 4; k++) sum[k] += f[k] * w;
                    total += w;
                }
            }
            sum[3] = frame[4 * ((size_t)IDy * W + IDx) + 3];
            float* d = &tmp[4 * ((size_t)IDy * W + IDx)];
            for (int k = 0; k < 4; k++) d[k] = (total > 0.0f) ? sum[k] / total : 0.0f;
        }
    }
    memcpy(frame, tmp, sizeof(float) * 4 * (size_t)W * (size_t)H);
    free(tmp);
    /* KrnlComputeEstimate - Source/estimate.cuh:27-32, CumulativeMovingAverage Source/utilities.h:59-62 */
    const float div = smax((float)no_iterations, 1.0f);
    for (size_t p = 0; p < (size_t)W * (size_t)H; p++) {
        for (int k = 0; k < 4; k++) {
            const float A = running[4 * p + k];
            running[4 * p + k] = A + (frame[4 * p + k] - A) / div;
        }
    }
    /* KrnlToneMap - Source/tonemap.cuh:49-59 */
    for (size_t p = 0; p < (size_t)W * (size_t)H; p++) tonemap_px(&running[4 * p], exposure, &rgba[4 * p]);
}

/* ------------------------------------------------------------------ */
/* known-answer helpers                                                 */
/* ------------------------------------------------------------------ */

void ER_OR(rng_draws)(uint32_t lane0, uint32_t lane1, int32_t n, float* out)
{
    rng_t r; r.s0 = lane0; r.s1 = lane1;
    for (int i = 0; i < n; i++) out[i] = rng_get1(&r);
}

void ER_OR(rng_get2_get3)(uint32_t lane0, uint32_t lane1, float* out5)
{
    rng_t r; r.s0 = lane0; r.s1 = lane1;
    const v2 a = rng_get2(&r);
    const v3 b = rng_get3(&r);
    out5[0] = a.x; out5[1] = a.y; out5[2] = b.x; out5[3] = b.y; out5[4] = b.z;
}

void ER_OR(plf_evaluate)(const er_plf* plf, int32_t n, const float* x, float* y)
{
    for (int i = 0; i < n; i++) y[i] = plf_eval(plf, x[i]);
}

void ER_OR(get_intensity)(or_scene* s, int32_t n, const float* p, float* out)
{
    for (int i = 0; i < n; i++) out[i] = get_intensity(s, V3(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
}

void ER_OR(normalized_gradient)(or_scene* s, int32_t n, const float* p, float* out)
{
    for (int i = 0; i < n; i++) {
        const v3 g = normalized_gradient(s, V3(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
        out[3 * i] = g.x; out[3 * i + 1] = g.y; out[3 * i + 2] = g.z;
    }
}

void ER_OR(gradient_magnitude)(or_scene* s, int32_t n, const float* p, float* out)
{
    for (int i = 0; i < n; i++) out[i] = gradient_magnitude(s, V3(p[3 * i], p[3 * i + 1], p[3 * i + 2]));
}

void ER_OR(intersect_volume_box)(or_scene* s, int32_t n, const float* r8, float* out3)
{
    for (int i = 0; i < n; i++) {
        ray_t R;
        R.O = V3(r8[8 * i], r8[8 * i + 1], r8[8 * i + 2]);
        R.D = V3(r8[8 * i + 3], r8[8 * i + 4], r8[8 * i + 5]);
        R.MinT = r8[8 * i + 6]; R.MaxT = r8[8 * i + 7];
        isect_t I; isect_invalid(&I);
        intersect_box(&R, s->minp, vscale(s->size, 0.5f), &I);
        out3[3 * i] = (float)I.valid; out3[3 * i + 1] = I.near_t; out3[3 * i + 2] = I.far_t;
    }
}

/* The majorant-brick walk of the trackers along rays (r8: origin,
   direction, MinT, MaxT), with the empty-space jump or brick by brick
   (jump = 0): per ray, up to `cap` records (t in, t out, bx, by, bz) of the
   non-empty bricks it crosses, in order; counts[2 i] = records,
   counts[2 i + 1] = DDA iterations.  Test infrastructure for the jump. */
void ER_OR(dda_walk)(or_scene* s, int32_t n, const float* r8, int32_t jump, int32_t cap, float* out, int32_t* counts)
{
    for (int i = 0; i < n; i++) {
        ray_t R;
        R.O = V3(r8[8 * i], r8[8 * i + 1], r8[8 * i + 2]);
        R.D = V3(r8[8 * i + 3], r8[8 * i + 4], r8[8 * i + 5]);
        R.MinT = r8[8 * i + 6]; R.MaxT = r8[8 * i + 7];
        int nrec = 0, iters = 0;
        isect_t Int; isect_invalid(&Int);
        intersect_box(&R, s->minp, vscale(s->size, 0.5f), &Int);
        const float t0 = smax(Int.near_t, R.MinT);
        const float t1 = smin(Int.far_t, R.MaxT);
        if (Int.valid && t0 < t1 && s->majorant) {
            dda_t d;
            dda_init(s, &R, t0, t1, &d);
            while (!d.done && iters < (1 << 20)) {
                iters++;
                const float e = dda_exit(&d);
                const float mu = s->majorant[((size_t)d.b[2] * (size_t)s->nb[1] + (size_t)d.b[1]) * (size_t)s->nb[0] + (size_t)d.b[0]];
                if (mu > 0.0f && nrec < cap) {
                    float* o = out + ((size_t)i * cap + nrec) * 5;
                    o[0] = d.t; o[1] = e; o[2] = (float)d.b[0]; o[3] = (float)d.b[1]; o[4] = (float)d.b[2];
                    nrec++;
                }
                if (jump && mu <= -2.0f) dda_jump(s, &d, (int)(-mu));
                else dda_advance(s, &d, e);
            }
        }
        counts[2 * i] = nrec;
        counts[2 * i + 1] = iters;
    }
}

/* For points p (3 floats each) given with a brick index b3 (3 ints each):
   out2 = (the extinction a tracker in that brick looks up at p, the brick's
   majorant).  Test infrastructure for the majorant bound. */
void ER_OR(brick_bound)(or_scene* s, int32_t n, const float* p, const int32_t* b3, float* out2)
{
    for (int i = 0; i < n; i++) {
        dda_t d;
        memset(&d, 0, sizeof(d));
        d.b[0] = b3[3 * i]; d.b[1] = b3[3 * i + 1]; d.b[2] = b3[3 * i + 2];
        out2[2 * i] = sigma_in_brick(s, V3(p[3 * i], p[3 * i + 1], p[3 * i + 2]), &d);
        out2[2 * i + 1] = s->majorant[((size_t)d.b[2] * (size_t)s->nb[1] + (size_t)d.b[1]) * (size_t)s->nb[0] + (size_t)d.b[0]];
    }
}

void ER_OR(concentric_sample_disk)(int32_t n, const float* u2, float* out2)
{
    for (int i = 0; i < n; i++) {
        v2 u; u.x = u2[2 * i]; u.y = u2[2 * i + 1];
        const v2 d = concentric_sample_disk(u);
        out2[2 * i] = d.x; out2[2 * i + 1] = d.y;
    }
}

void ER_OR(tonemap)(int32_t n, const float* xyza, float exposure, uint8_t* rgba)
{
    for (int i = 0; i < n; i++) tonemap_px(&xyza[4 * i], exposure, &rgba[4 * i]);
}

void ER_OR(camera_ray)(or_scene* s, int32_t x, int32_t y, const float* uv4, float* out6)
{
    v2 f, l; f.x = uv4[0]; f.y = uv4[1]; l.x = uv4[2]; l.y = uv4[3];
    const ray_t R = sample_camera(s, x, y, f, l);
    out6[0] = R.O.x; out6[1] = R.O.y; out6[2] = R.O.z; out6[3] = R.D.x; out6[4] = R.D.y; out6[5] = R.D.z;
}

void ER_OR(camera_frame)(or_scene* s, float* o)
{
    o[0] = s->N.x; o[1] = s->N.y; o[2] = s->N.z;
    o[3] = s->U.x; o[4] = s->U.y; o[5] = s->U.z;
    o[6] = s->V.x; o[7] = s->V.y; o[8] = s->V.z;
    o[9] = s->screen[0][0]; o[10] = s->screen[0][1]; o[11] = s->screen[1][0]; o[12] = s->screen[1][1];
    o[13] = s->inv_screen[0]; o[14] = s->inv_screen[1];
}

void ER_OR(volume_frame)(or_scene* s, float* o)
{
    o[0] = s->minp.x; o[1] = s->minp.y; o[2] = s->minp.z;
    o[3] = s->inv_size.x; o[4] = s->inv_size.y; o[5] = s->inv_size.z;
    o[6] = s->min_step;
    o[7] = s->spacing.x; o[8] = s->spacing.y; o[9] = s->spacing.z;
    o[10] = s->size.x; o[11] = s->size.y; o[12] = s->size.z;
}

/* ------------------------------------------------------------------ */
/* bilateral filter - design of Source/filterrunningestimate.cuh:35-200 */
/* ------------------------------------------------------------------ */

/* LUMINANCE weights (Source/color.h:37-51) applied to 0..255 channels;
   LuminanceFromRGB is called but not defined by the reference. */
static inline float lum255(const uint8_t* c)
{
    float L = 0.0f;
    L += 0.212671f * (float)c[0];
    L += 0.715160f * (float)c[1];
    L += 0.072169f * (float)c[2];
    return L;
}

static void bilateral_pass(const uint8_t* in, uint8_t* out, int W, int H, int r, const float* spatial, const float* range,
                           int horizontal)
{
    for (int y = 0; y < H; y++) {
        for (int x = 0; x < W; x++) {
            const int i = horizontal ? x : y;
            const int lim = horizontal ? W : H;
            const int r0 = (i - r) > 0 ? (i - r) : 0;
            const int r1 = (i + r) < (lim - 1) ? (i + r) : (lim - 1);
            const uint8_t* ctr = &in[4 * ((size_t)y * W + x)];
            const float lc = lum255(ctr);
            float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, tot = 0.0f;
            for (int k = r0; k < r1; k++) {   /* window end exclusive (:88, :157) */
                const uint8_t* c = horizontal ? &in[4 * ((size_t)y * W + k)] : &in[4 * ((size_t)k * W + x)];
                int d = (int)fabsf(lum255(c) - lc);
                d = d > 255 ? 255 : d;
                const float w = spatial[r + k - i] * range[d];
                tot += w;
                s0 += (float)c[0] * w; s1 += (float)c[1] * w; s2 += (float)c[2] * w;
            }
            uint8_t* o = &out[4 * ((size_t)y * W + x)];
            if (tot > 0.0f) {
                o[0] = (uint8_t)eclamp(s0 / tot, 0.0f, 255.0f);
                o[1] = (uint8_t)eclamp(s1 / tot, 0.0f, 255.0f);
                o[2] = (uint8_t)eclamp(s2 / tot, 0.0f, 255.0f);
            } else {
                o[0] = 0; o[1] = 0; o[2] = 0;
            }
            o[3] = 255;
        }
    }
}

/* KernelD[r + k] = exp(-k^2 / (2 sd^2)), GaussSimilarity[d] = exp(-d^2 / (2 sr^2)):
   the tables of BilateralFilter (Source/filter.h:34-40), which the reference
   declares but never fills */
void ER_OR(bilateral)(const uint8_t* in, uint8_t* tmp, uint8_t* out, int32_t W, int32_t H, int32_t radius, float sigma_d,
                      float sigma_r)
{
    float spatial[256], range[256];
    const int r = radius < 0 ? 0 : (radius > 127 ? 127 : radius);
    const float sd = sigma_d > 0.0f ? sigma_d : 1.0f;
    const float sr = sigma_r > 0.0f ? sigma_r : 1.0f;
    for (int k = -r; k <= r; k++) spatial[r + k] = er_expf(-((float)(k * k)) / (2.0f * sd * sd));
    for (int d = 0; d < 256; d++) range[d] = er_expf(-((float)(d * d)) / (2.0f * sr * sr));
    bilateral_pass(in, tmp, W, H, r, spatial, range, 1);
    bilateral_pass(tmp, out, W, H, r, spatial, range, 0);
}

/* gradient magnitude at every voxel centre (Source/gradientmagnitude.cuh:38
   with the current Volume fields) and its maximum */
float ER_OR(gradient_magnitude_volume)(or_scene* s, uint16_t* gm)
{
    float mx = 0.0f;
    for (int Z = 0; Z < s->res[2]; Z++)
        for (int Y = 0; Y < s->res[1]; Y++)
            for (int X = 0; X < s->res[0]; X++) {
                const float sx = 2.0f * (s->size.x * 0.5f), sy = 2.0f * (s->size.y * 0.5f), sz = 2.0f * (s->size.z * 0.5f);
                const v3 p = V3(s->minp.x + sx * (((float)X + 0.5f) * (1.0f / (float)s->res[0])),
                                s->minp.y + sy * (((float)Y + 0.5f) * (1.0f / (float)s->res[1])),
                                s->minp.z + sz * (((float)Z + 0.5f) * (1.0f / (float)s->res[2])));
                const float g = gradient_magnitude(s, p);
                if (gm) gm[(size_t)Z * s->res[0] * s->res[1] + (size_t)Y * s->res[0] + X] = (uint16_t)(g < 65535.0f ? g : 65535.0f);
                mx = g > mx ? g : mx;
            }
    return mx;
}

/* er_math functions on the host: fn 0 log, 1 exp, 2 sin, 3 cos, 4 tan,
   5 pow(x, y), 6 acos, 7 atan2(x, y) */
/* IntersectsLight for one light shape and n segments (origin, unit
   direction, MinT, MaxT: 8 floats each): 1 where the exact test of
   Visible (Source/transport.h:46-56) finds the shape on the segment.  Test
   infrastructure for the occlusion early-outs of the GPU shadow stage. */
void ER_OR(segments_hit_shape)(const er_shape* shape, int32_t n, const float* seg, int32_t* hit)
{
    for (int i = 0; i < n; i++) {
        const float* q = seg + 8 * (size_t)i;
        ray_t R;
        R.O = V3(q[0], q[1], q[2]);
        R.D = V3(q[3], q[4], q[5]);
        R.MinT = q[6];
        R.MaxT = q[7];
        const ray_t Rt = xform_ray(shape->inv_tm, &R);
        isect_t Int; isect_invalid(&Int);
        intersect_shape(shape, &Rt, &Int);
        hit[i] = Int.valid ? 1 : 0;
    }
}

void ER_OR(math_eval)(int32_t fn, int32_t n, const float* x, const float* y, float* out)
{
    for (int i = 0; i < n; i++) {
        switch (fn) {
        case 0: out[i] = er_logf(x[i]); break;
        case 1: out[i] = er_expf(x[i]); break;
        case 2: out[i] = er_sinf(x[i]); break;
        case 3: out[i] = er_cosf(x[i]); break;
        case 4: out[i] = er_tanf(x[i]); break;
        case 5: out[i] = er_powf(x[i], y[i]); break;
        case 6: out[i] = er_acosf(x[i]); break;
        case 7: out[i] = er_atan2f(x[i], y[i]); break;
        default: out[i] = 0.0f; break;
        }
    }
}

/* majorant grid by brute force over each brick's footprint (the grid the
   delta tracker of this file uses, exported for the device pre-pass tests) */
void ER_OR(majorant_grid)(const uint16_t* vox, const int32_t* res, int32_t B, const float* sigma, int32_t n, float ds, float* out)
{
    int nb[3];
    for (int i = 0; i < 3; i++) nb[i] = (res[i] + B - 1) / B;
    for (int bz = 0; bz < nb[2]; bz++)
        for (int by = 0; by < nb[1]; by++)
            for (int bx = 0; bx < nb[0]; bx++) {
                int lo[3], hi[3];
                const int b[3] = { bx, by, bz };
                for (int i = 0; i < 3; i++) {
                    lo[i] = b[i] * B;
                    hi[i] = (b[i] + 1) * B;
                    hi[i] = hi[i] > res[i] - 1 ? res[i] - 1 : hi[i];
                }
                int vlo = 65535, vhi = 0;
                for (int z = lo[2]; z <= hi[2]; z++)
                    for (int y = lo[1]; y <= hi[1]; y++)
                        for (int x = lo[0]; x <= hi[0]; x++) {
                            const int v = vox[(size_t)z * res[0] * res[1] + (size_t)y * res[0] + x];
                            vlo = v < vlo ? v : vlo;
                            vhi = v > vhi ? v : vhi;
                        }
                vlo = vlo - 1;
                vlo = vlo < 0 ? 0 : (vlo > n - 1 ? n - 1 : vlo);
                vhi = vhi > n - 1 ? n - 1 : vhi;
                float m = 0.0f;
                for (int i = vlo; i <= vhi; i++) m = sigma[i] > m ? sigma[i] : m;
                out[((size_t)bz * nb[1] + by) * nb[0] + bx] = ds * m;
            }
}

/* ------------------------------------------------------------------ */
/* differentiable medium (extension, no reference counterpart)           */
/*                                                                      */
/* sigma(x) = scale * alpha(rho(x)): rho is the trilinear interpolation  */
/* of a float density grid with the addressing of the intensity volume  */
/* (Source/buffer3d.h:222-242, without the unsigned-short truncation);  */
/* alpha is a uniform cubic B-spline of the n opacity values over       */
/* u = 2 + rho * (n - 5), so that alpha is C2 in rho on                  */
/* [-1/(n-5), 1 + 1/(n-5)] and linear in the values.                     */
/*                                                                      */
/* Estimator (per sample): the camera ray's tentative collisions are    */
/* drawn from the fixed majorant grid (DDA as the delta tracker); at    */
/* each, with probability q (a random number independent of the        */
/* medium), next-event estimation to one uniformly picked light with a  */
/* ratio-tracked shadow segment (its own random stream, by the index of  */
/* the next-event estimate along the ray); the contribution is weighted by the */
/* collision weight sigma/mu and the ratio-tracked throughput          */
/* T = prod (1 - sigma_j/mu_j) of the earlier collisions.  Nothing the  */
/* RNG draws depends on the medium, so for fixed seeds the estimate is  */
/* a smooth function of the density and opacity values; the adjoint     */
/* replays the same draws (path replay).                                */
/* ------------------------------------------------------------------ */

#define DM_INV_4PI 0.0795774715459476678f

void ER_OR(dm_attach)(or_scene* s, const float* rho, const float* tf_val, int32_t tf_n, float scale, const float* albedo,
                      float q, const float* majorant, int32_t brick)
{
    s->rho = rho;
    s->tf_val = tf_val;
    s->tf_n = tf_n;
    s->dm_scale = scale;
    s->dm_albedo = C3(albedo[0], albedo[1], albedo[2]);
    s->dm_q = q;
    s->brick = brick;
    for (int i = 0; i < 3; i++) s->nb[i] = (s->res[i] + brick - 1) / brick;
    const size_t nbt = (size_t)s->nb[0] * (size_t)s->nb[1] * (size_t)s->nb[2];
    free(s->majorant);
    s->majorant = (float*)malloc(sizeof(float) * nbt);
    for (size_t i = 0; i < nbt; i++) s->majorant[i] = majorant[i];
}

/* corners and weights of the trilinear density lookup */
typedef struct { size_t idx[8]; float w[8]; float rho; } dm_lookup;

static inline size_t dm_index(const or_scene* s, int x, int y, int z)
{
    const int cx = iclamp(x, 0, s->res[0] - 1);
    const int cy = iclamp(y, 0, s->res[1] - 1);
    const int cz = iclamp(z, 0, s->res[2] - 1);
    return (size_t)cz * (size_t)s->res[0] * (size_t)s->res[1] + (size_t)cy * (size_t)s->res[0] + (size_t)cx;
}

static void dm_density(or_scene* s, v3 P, dm_lookup* k)
{
    s->lookups++;
    const v3 off = vsub(P, s->minp);
    const v3 L = V3(off.x * s->inv_size.x * (float)s->res[0], off.y * s->inv_size.y * (float)s->res[1],
                    off.z * s->inv_size.z * (float)s->res[2]);
    const int vx = (int)floorf(L.x), vy = (int)floorf(L.y), vz = (int)floorf(L.z);
    const float dx = L.x - (float)vx, dy = L.y - (float)vy, dz = L.z - (float)vz;
    const float ex = 1.0f - dx, ey = 1.0f - dy, ez = 1.0f - dz;
    float r = 0.0f;
    for (int c = 0; c < 8; c++) {
        const int ox = c & 1, oy = (c >> 1) & 1, oz = (c >> 2) & 1;
        k->idx[c] = dm_index(s, vx + ox, vy + oy, vz + oz);
        k->w[c] = (ox ? dx : ex) * (oy ? dy : ey) * (oz ? dz : ez);
        r = r + k->w[c] * s->rho[k->idx[c]];
    }
    k->rho = r;
}

/* opacity: value, d alpha / d rho, the nb parameters it depends on (first
   index i0) and their weights */
typedef struct { float alpha, dalpha; int i0, nb; float b[4]; } dm_tf;

/* PiecewiseLinearFunction::Evaluate (Source/plf.h:68-91) with the node
   values `vals` at the positions of `p`: the value, the slope d/dx of the
   segment (0 where it clamps) and the two values it blends (i0 and i0 + 1
   with weights b[0], b[1]; one value where it clamps; none for the x equal
   to the last node, where Evaluate returns 0) */
static float dm_plf(const er_plf* p, const float* vals, float x, int* i0, int* nb, float* b, float* slope)
{
    const int n = p->count;
    *slope = 0.0f;
    *nb = 0;
    *i0 = 0;
    if (n <= 0) return 0.0f;
    if (x < p->node_range[0]) { *nb = 1; b[0] = 1.0f; return vals[0]; }
    if (x > p->node_range[1]) { *nb = 1; *i0 = n - 1; b[0] = 1.0f; return vals[n - 1]; }
    for (int i = 1; i < n; i++) {
        const float P1 = p->position[i - 1];
        const float P2 = p->position[i];
        const float DeltaP = P2 - P1;
        const float LerpT = (x - P1) / DeltaP;
        if (x >= P1 && x < P2) {
            *i0 = i - 1;
            *nb = 2;
            b[0] = 1.0f - LerpT;
            b[1] = LerpT;
            *slope = (vals[i] - vals[i - 1]) / DeltaP;
            return vals[i - 1] + LerpT * (vals[i] - vals[i - 1]);
        }
    }
    return 0.0f;
}

/* d/dx of a transfer function of the tracer (its own node values) */
static float plf_slope(const er_plf* p, float x)
{
    if (p->count <= 0 || x < p->node_range[0] || x > p->node_range[1]) return 0.0f;
    for (int i = 1; i < p->count; i++) {
        const float P1 = p->position[i - 1];
        const float P2 = p->position[i];
        if (x >= P1 && x < P2) return (p->value[i] - p->value[i - 1]) / (P2 - P1);
    }
    return 0.0f;
}

static void dm_opacity(const or_scene* s, float rho, dm_tf* o)
{
    if (s->dm_model == 1) {
        o->alpha = dm_plf(&s->opacity, s->tf_val, rho, &o->i0, &o->nb, o->b, &o->dalpha);
        return;
    }
    o->nb = 4;
    const int n = s->tf_n;
    const float du = (float)(n - 5);
    float u = 2.0f + rho * du;
    int slope = 1;
    if (u < 1.0f) { u = 1.0f; slope = 0; }
    if (u > (float)(n - 2)) { u = (float)(n - 2); slope = 0; }
    int i = (int)floorf(u);
    if (i > n - 3) i = n - 3;
    const float f = u - (float)i;
    const float g = 1.0f - f;
    const float f2 = f * f, f3 = f2 * f;
    o->b[0] = g * g * g / 6.0f;
    o->b[1] = (3.0f * f3 - 6.0f * f2 + 4.0f) / 6.0f;
    o->b[2] = (-3.0f * f3 + 3.0f * f2 + 3.0f * f + 1.0f) / 6.0f;
    o->b[3] = f3 / 6.0f;
    const float d0 = -0.5f * g * g, d1 = 1.5f * f2 - 2.0f * f, d2 = -1.5f * f2 + f + 0.5f, d3 = 0.5f * f2;
    o->i0 = i - 1;
    const float* v = &s->tf_val[i - 1];
    o->alpha = o->b[0] * v[0] + o->b[1] * v[1] + o->b[2] * v[2] + o->b[3] * v[3];
    o->dalpha = slope ? du * (d0 * v[0] + d1 * v[1] + d2 * v[2] + d3 * v[3]) : 0.0f;
}

/* adjoint of sigma at a lookup: a = dLoss/dsigma, scattered into the
   density and opacity gradients */
static void dm_scatter(const or_scene* s, const dm_lookup* k, const dm_tf* o, float a, float* g_rho, float* g_tf)
{
    const float as = a * s->dm_scale;
    if (g_tf)
        for (int j = 0; j < o->nb; j++) g_tf[o->i0 + j] += as * o->b[j];
    if (g_rho && o->dalpha != 0.0f) {
        const float ar = as * o->dalpha;
        for (int c = 0; c < 8; c++) g_rho[k->idx[c]] += ar * k->w[c];
    }
}

static void dm_scatter_rho(const dm_lookup* k, float a, float* g_rho)
{
    if (!g_rho || a == 0.0f) return;
    for (int c = 0; c < 8; c++) g_rho[k->idx[c]] += a * k->w[c];
}

/* ---- model 1: the tracer's shading at a tentative collision ----------
   At intensity I (the float grid's trilinear value): Kd = Diffuse1D(I),
   Ks = Specular1D(I), exponent = 1e6 Glossiness1D(I)^7, IOR of the volume
   BRDF (Source/transport.h:136-139, Source/utilities.h:28-31); the normal
   from central differences of the grid at +-MinStep (Source/volumes.h:31-
   91); the shader chosen by the settings: BRDF (also without
   apply_shading_type, as the live reference), isotropic phase, or hybrid
   (Source/scatterevent.h:155-212), whose random choice between the two is
   replaced by its expected value, P_brdf * BRDF + (1 - P_brdf) * phase, so
   that a sample stays smooth in the parameters.  The next-event estimate is
   S(Wo, Wi) Li LightCount / (LightPdf q): S = F |Wi . N| for the BRDF, F
   for the phase function (Source/transport.h:58-84 without the MIS
   weight, which a light-sampling-only estimator does not need). */
typedef struct {
    col3 Kd, Ks;
    float gl, e;        /* Glossiness1D(I) and the exponent */
    int type;           /* 0 BRDF, 1 isotropic phase, 2 hybrid (expected value) */
    dm_lookup g[6];     /* I(P - d), I(P + d) per axis, d = MinStep */
    v3 N;
    float gm, pb;       /* gradient magnitude, probability of the BRDF */
} dm_shade_t;

static void dm_shade_prepare(or_scene* s, v3 P, const dm_lookup* k, const dm_tf* o, dm_shade_t* h)
{
    const float I = k->rho;
    h->Kd = ctf_eval(&s->diffuse, I);
    h->Ks = ctf_eval(&s->specular, I);
    h->gl = plf_eval(&s->glossiness, I);
    h->e = glossiness_exponent(h->gl);
    h->type = !s->st.apply_shading_type ? 0 : (s->st.shading_type == ER_SHADING_PHASE_ONLY ? 1 : (s->st.shading_type == ER_SHADING_HYBRID ? 2 : 0));
    h->pb = h->type == 0 ? 1.0f : 0.0f;
    h->gm = 0.0f;
    h->N = V3(0.0f, 0.0f, 0.0f);
    if (h->type == 1) return;
    const v3 d[3] = { s->gdx, s->gdy, s->gdz };
    for (int i = 0; i < 3; i++) {
        dm_density(s, vsub(P, d[i]), &h->g[2 * i]);
        dm_density(s, vadd(P, d[i]), &h->g[2 * i + 1]);
    }
    /* Normalize(V) = V / Length(V) (Source/vector.h:469-475); where the
       grid is flat the normal is undefined and the BRDF term is taken as 0
       (the hybrid's P_brdf is 0 there anyway) */
    const v3 gv = V3(h->g[0].rho - h->g[1].rho, h->g[2].rho - h->g[3].rho, h->g[4].rho - h->g[5].rho);
    const float L = vlen(gv);
    if (L > 0.0f) h->N = V3(gv.x / L, gv.y / L, gv.z / L);
    if (h->type != 2) return;
    float sum = 0.0f;
    for (int i = 0; i < 3; i++) {
        float D = h->g[2 * i].rho - h->g[2 * i + 1].rho;
        D *= 0.5f / vget(s->spacing, i);
        sum += D * D;
    }
    h->gm = sqrtf(sum);
    const float NGM = h->gm * s->dm_gm_inv;
    const float Exponent = 25.0f * er_powf(s->st.gradient_factor, 3.0f) * NGM;
    h->pb = s->st.opacity_modulated ? o->alpha * (1.0f - er_expf(-Exponent)) : 1.0f - er_expf(-Exponent);
}

static inline float dm_ior(const or_scene* s) { return s->st.volume_ior > 0.0f ? s->st.volume_ior : 15.0f; }

/* S(Wo, Wi), and the BRDF and phase parts */
static col3 dm_shade_eval(const or_scene* s, const dm_shade_t* h, v3 Wo, v3 Wi, col3* Sb_out, col3* Sp_out)
{
    const col3 Sp = cscale(h->Kd, INV_PI_F);
    col3 Sb = C3(0.0f, 0.0f, 0.0f);
    if (h->type != 1 && !(h->N.x == 0.0f && h->N.y == 0.0f && h->N.z == 0.0f)) {
        shader_t sh;
        shader_init(&sh, 0, h->N, Wo, h->Kd, h->Ks, dm_ior(s), h->e);
        Sb = cscale(shader_f(&sh, Wo, Wi), vabsdot(Wi, h->N));
    }
    if (Sb_out) *Sb_out = Sb;
    if (Sp_out) *Sp_out = Sp;
    if (h->type == 1) return Sp;
    if (h->type == 0) return Sb;
    return cadd(cscale(Sb, h->pb), cscale(Sp, 1.0f - h->pb));
}

static inline float sgnf(float x) { return x < 0.0f ? -1.0f : 1.0f; }

/* adjoint of S: aS = dLoss/dS; adds dLoss/dI to *aI, dLoss/d(opacity at
   I) through the hybrid's modulation to *aop, and dLoss/d(each of the six
   gradient lookups) to ag[6].  The microfacet term depends on the normal
   only through a = Wh.N, b = Wo.N, c = Wi.N (the Fresnel term and |Wo.Wh|
   do not). */
static void dm_shade_adjoint(const or_scene* s, const dm_shade_t* h, const dm_tf* o, float I, v3 Wo, v3 Wi, col3 aS, float* aI, float* aop,
                             float ag[6])
{
    for (int i = 0; i < 6; i++) ag[i] = 0.0f;
    col3 Sb, Sp;
    dm_shade_eval(s, h, Wo, Wi, &Sb, &Sp);
    col3 aSb = aS, aSp = aS;
    float angm = 0.0f;
    if (h->type == 2) {
        const float apb = aS.c[0] * (Sb.c[0] - Sp.c[0]) + aS.c[1] * (Sb.c[1] - Sp.c[1]) + aS.c[2] * (Sb.c[2] - Sp.c[2]);
        const float GF3 = er_powf(s->st.gradient_factor, 3.0f);
        const float ex = er_expf(-25.0f * GF3 * h->gm * s->dm_gm_inv);
        const float mod = s->st.opacity_modulated ? o->alpha : 1.0f;
        if (s->st.opacity_modulated) *aop += apb * (1.0f - ex);
        angm = apb * mod * ex * 25.0f * GF3;
        aSb = cscale(aS, h->pb);
        aSp = cscale(aS, 1.0f - h->pb);
    }
    if (h->type != 0) {
        for (int c = 0; c < 3; c++) *aI += aSp.c[c] * plf_slope(&s->diffuse.plf[c], I) * INV_PI_F;
    }
    if (h->type == 1) return;
    /* BRDF: Sb = (Kd / pi + Ks m(a, b, c, e)) |c| */
    const v3 N = h->N;
    const v3 Wsum = vadd(Wi, Wo);
    const float b = vdot(Wo, N), c = vdot(Wi, N);
    const float ab = fabsf(b), ac = fabsf(c);
    float m = 0.0f, dmda = 0.0f, dmdb = 0.0f, dmdc = 0.0f, dmde = 0.0f;
    v3 Wh = V3(0.0f, 0.0f, 0.0f);
    if (ab > 0.0f && ac > 0.0f && !(Wsum.x == 0.0f && Wsum.y == 0.0f && Wsum.z == 0.0f)) {
        Wh = vnorm(Wsum);
        const float a = vdot(Wh, N), aa = fabsf(a);
        const float k = vabsdot(Wo, Wh);
        const float F = fresnel_eval(1.0f, dm_ior(s), vdot(Wi, Wh));
        const float D = (h->e + 2.0f) * INV_TWO_PI_F * er_powf(aa, h->e);
        const float g1 = 2.0f * aa * ab / k, g2 = 2.0f * aa * ac / k;
        const float gmin = (g2 < g1) ? g2 : g1;
        float G = 1.0f, dGda = 0.0f, dGdb = 0.0f, dGdc = 0.0f;
        if (gmin < 1.0f) {
            G = gmin;
            if (g2 < g1) { dGda = 2.0f * ac / k * sgnf(a); dGdc = 2.0f * aa / k * sgnf(c); }
            else { dGda = 2.0f * ab / k * sgnf(a); dGdb = 2.0f * aa / k * sgnf(b); }
        }
        const float den = 4.0f * ac * ab;
        m = D * G * F / den;
        const float dDda = aa > 0.0f ? D * h->e / aa * sgnf(a) : 0.0f;
        dmda = (dDda * G + D * dGda) * F / den;
        dmdb = D * F / (4.0f * ac) * (dGdb / ab - G * sgnf(b) / (ab * ab));
        dmdc = D * F / (4.0f * ab) * (dGdc / ac - G * sgnf(c) / (ac * ac));
        dmde = aa > 0.0f ? m * (1.0f / (h->e + 2.0f) + er_logf(aa)) : 0.0f;
    }
    /* through I: Kd', Ks' and the exponent's 7e6 gl^6 gl' */
    const float gls = plf_slope(&s->glossiness, I);
    const float dedI = 7000000.0f * er_powf(h->gl, 6.0f) * gls;
    float ks_dot = 0.0f, f_dot = 0.0f;
    for (int ch = 0; ch < 3; ch++) {
        const float kd_s = plf_slope(&s->diffuse.plf[ch], I), ks_s = plf_slope(&s->specular.plf[ch], I);
        *aI += aSb.c[ch] * (kd_s * INV_PI_F + ks_s * m + h->Ks.c[ch] * dmde * dedI) * ac;
        ks_dot += aSb.c[ch] * h->Ks.c[ch];
        f_dot += aSb.c[ch] * (h->Kd.c[ch] * INV_PI_F + h->Ks.c[ch] * m);
    }
    /* through the normal */
    v3 aN = vscale(vadd(vadd(vscale(Wh, dmda), vscale(Wo, dmdb)), vscale(Wi, dmdc)), ks_dot * ac);
    aN = vadd(aN, vscale(Wi, f_dot * sgnf(c)));
    const v3 gv = V3(h->g[0].rho - h->g[1].rho, h->g[2].rho - h->g[3].rho, h->g[4].rho - h->g[5].rho);
    const float glen = vlen(gv);
    float aG[3] = { 0.0f, 0.0f, 0.0f };
    if (glen > 0.0f) {
        const float an = vdot(aN, N);
        aG[0] = (aN.x - an * N.x) / glen;
        aG[1] = (aN.y - an * N.y) / glen;
        aG[2] = (aN.z - an * N.z) / glen;
    }
    if (h->type == 2 && h->gm > 0.0f) {
        for (int i = 0; i < 3; i++) {
            const float hi = 0.5f / vget(s->spacing, i);
            aG[i] += angm * s->dm_gm_inv * vget(gv, i) * hi * hi / h->gm;
        }
    }
    for (int i = 0; i < 3; i++) {
        ag[2 * i] = aG[i];
        ag[2 * i + 1] = -aG[i];
    }
}

/* model 1: the emission TF of the tracer at I and its slope per channel */
static col3 dm_emission(const or_scene* s, float I)
{
    return s->dm_emissive ? ctf_eval(&s->emission, I) : C3(0.0f, 0.0f, 0.0f);
}

/* the model of the differentiable medium (the dm_model field); gm_inv is
   the hybrid shader's 1 / gradient-magnitude range, a constant of the
   estimator */
void ER_OR(dm_set_model)(or_scene* s, int32_t model, float gm_inv)
{
    s->dm_model = model;
    s->dm_gm_inv = gm_inv;
    s->dm_emissive = 0;
    for (int c = 0; c < 3; c++)
        for (int i = 0; i < s->emission.plf[c].count; i++)
            if (s->emission.plf[c].value[i] != 0.0f) s->dm_emissive = 1;
}

/* the ray's box segment, as the delta tracker clips it */
static int dm_segment(or_scene* s, const ray_t* R, float* t0, float* t1)
{
    isect_t Int; isect_invalid(&Int);
    intersect_box(R, s->minp, vscale(s->size, 0.5f), &Int);
    if (!Int.valid) return 0;
    *t0 = smax(Int.near_t, R->MinT);
    *t1 = smin(Int.far_t, R->MaxT);
    return *t0 < *t1;
}

/* random stream of the k-th next-event shadow segment of a sample: its own
   lanes, so that the camera ray's draws do not depend on how many the
   shadow segments take */
static void dm_shadow_stream(uint32_t seed, uint32_t view, uint32_t pix, uint32_t sample, uint32_t k, rng_t* r)
{
    er_seed_lanes(seed ^ er_hash32(0x51ED2705u + k), view ^ 0x6A09E667u, pix, sample, &r->s0, &r->s1);
}

/* ratio-tracked transmittance of a shadow segment; with a_scale != 0 the
   adjoint pass scatters -a_scale / (mu - sigma) at every collision */
static float dm_shadow(or_scene* s, v3 P1, v3 P2, rng_t* rng, float a_scale, float* g_rho, float* g_tf)
{
    if (!s->st.shadows) return 1.0f;
    const v3 W = vnorm(vsub(P2, P1));
    ray_t R;
    R.O = vadd(P1, vscale(W, RAY_EPS));
    R.D = W;
    R.MinT = 0.0f;
    R.MaxT = smin(vlen(vsub(P2, P1)) - 2.0f * RAY_EPS, s->st.max_shadow_distance);
    float t0, t1;
    if (!dm_segment(s, &R, &t0, &t1)) return 1.0f;
    dda_t d;
    dda_init(s, &R, t0, t1, &d);
    float Tr = 1.0f;
    float tau = -er_logf(rng_get1(rng));
    while (!d.done) {
        const float e = dda_exit(&d);
        const float mu = dda_majorant(s, &d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 P = vadd(R.O, vscale(R.D, t));
                dm_lookup k;
                dm_density(s, P, &k);
                dm_tf o;
                dm_opacity(s, k.rho, &o);
                const float sig = s->dm_scale * o.alpha;
                if (a_scale != 0.0f) dm_scatter(s, &k, &o, -a_scale / (mu - sig), g_rho, g_tf);
                Tr = Tr * (1.0f - sig / mu);
                tau = -er_logf(rng_get1(rng));
            }
        }
        dda_advance(s, &d, e);
    }
    return Tr;
}

/* next-event estimate at P (without the collision weight): one uniformly
   picked light, isotropic phase, albedo, ratio-tracked shadow; the light
   sample is written to *S for the adjoint's shadow replay */
static col3 dm_nee(or_scene* s, v3 P, rng_t* rng, v3* S, float* unshadowed_scale, const dm_shade_t* h, v3 Wo, v3* Wi_out,
                   col3* LiK)
{
    *unshadowed_scale = 0.0f;
    const float pick = rng_get1(rng);
    const v3 uvw = rng_get3(rng);
    if (s->light_count <= 0) return C3(0, 0, 0);
    int idx = (int)floorf(pick * (float)s->light_count);
    if (idx >= s->light_count) idx = s->light_count - 1;
    const int light_id = s->light_idx[idx];
    if (light_id < 0 || light_id >= s->n_lights) return C3(0, 0, 0);
    const or_light* L = &s->lights[light_id];
    scatter_event SE;
    se_invalid(&SE, 0);
    SE.P = P;
    v3 Wi;
    col3 Li;
    surf_sample SS;
    sample_light(s, L, uvw, &SS, &SE, &Wi, &Li);
    *S = SS.P;
    if (cblack(Li)) return C3(0, 0, 0);
    const float LightPdf = vlen2(vsub(P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L->area);
    if (!(LightPdf > 0.0f)) return C3(0, 0, 0);
    *unshadowed_scale = 1.0f;
    if (s->dm_model == 1) {
        /* the tracer's shading (model 1) */
        *Wi_out = Wi;
        *LiK = cscale(Li, (float)s->light_count / (LightPdf * s->dm_q));
        return cmul(dm_shade_eval(s, h, Wo, Wi, NULL, NULL), *LiK);
    }
    const col3 c = cscale(cmul(s->dm_albedo, Li), DM_INV_4PI * (float)s->light_count / (LightPdf * s->dm_q));
    return c;
}

/* one sample (pixel pix, stream index sample); with g != NULL the adjoint
   pass (Ltot = the sample's forward value, g = dLoss/dL) */
static col3 dm_sample(or_scene* s, int x, int y, uint32_t view, uint32_t pix, uint32_t sample, rng_t* rng, const col3* g, col3 Ltot,
                      float* g_rho, float* g_tf)
{
    uint32_t nee = 0;
    col3 L = C3(0, 0, 0);
    col3 E = C3(0, 0, 0);     /* model 1: emission, summed apart from the next-event estimates */
    const v2 film_uv = rng_get2(rng);
    const v2 lens_uv = rng_get2(rng);
    const ray_t R = sample_camera(s, x, y, film_uv, lens_uv);
    float t0, t1;
    if (!dm_segment(s, &R, &t0, &t1)) return L;
    dda_t d;
    dda_init(s, &R, t0, t1, &d);
    float T = 1.0f;
    float tau = -er_logf(rng_get1(rng));
    while (!d.done) {
        const float e = dda_exit(&d);
        const float mu = dda_majorant(s, &d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 P = vadd(R.O, vscale(R.D, t));
                dm_lookup k;
                dm_density(s, P, &k);
                dm_tf o;
                dm_opacity(s, k.rho, &o);
                const float sig = s->dm_scale * o.alpha;
                const float w = sig / mu;
                col3 A = C3(0, 0, 0);
                /* model 1: the tracer's emission at every collision and its
                   shading at the next-event estimates */
                const col3 Le = s->dm_model == 1 ? dm_emission(s, k.rho) : C3(0, 0, 0);
                dm_shade_t sd;
                v3 Wi = V3(0, 0, 0);
                col3 LiK = C3(0, 0, 0);
                float Tr = 0.0f;
                int shaded = 0;
                if (rng_get1(rng) < s->dm_q) {
                    v3 S;
                    float has;
                    if (s->dm_model == 1) dm_shade_prepare(s, P, &k, &o, &sd);
                    const col3 A0 = dm_nee(s, P, rng, &S, &has, &sd, vneg(R.D), &Wi, &LiK);
                    const uint32_t k_nee = nee++;
                    if (has != 0.0f) {
                        rng_t sh;
                        dm_shadow_stream(s->st.seed, view, pix, sample, k_nee, &sh);
                        Tr = dm_shadow(s, P, S, &sh, 0.0f, NULL, NULL);
                        A = cscale(A0, Tr);
                        shaded = s->dm_model == 1;
                        if (g) {
                            /* the adjoint replay of the same segment */
                            const col3 c = cscale(A, T * w);
                            const float gc = g->c[0] * c.c[0] + g->c[1] * c.c[1] + g->c[2] * c.c[2];
                            if (gc != 0.0f) {
                                dm_shadow_stream(s->st.seed, view, pix, sample, k_nee, &sh);
                                dm_shadow(s, P, S, &sh, gc, g_rho, g_tf);
                            }
                        }
                    }
                }
                const col3 c = cscale(A, T * w);
                L = cadd(L, c);
                if (s->dm_model == 1) E = cadd(E, cscale(Le, T * w));
                if (g) {
                    /* dL/dsigma = T A / mu - (Ltot - L_<=k) / (mu - sigma), A the
                       collision's whole contribution before T w */
                    const col3 Ak = s->dm_model == 1 ? cadd(Le, A) : A;
                    const col3 rest = csub(Ltot, s->dm_model == 1 ? cadd(L, E) : L);
                    const col3 dLds = csub(cscale(Ak, T / mu), cdivs(rest, mu - sig));
                    const float a = g->c[0] * dLds.c[0] + g->c[1] * dLds.c[1] + g->c[2] * dLds.c[2];
                    if (s->dm_model == 1) {
                        /* through the shading and emission at I, and the hybrid's
                           opacity modulation */
                        const col3 gA = cscale(*g, T * w);
                        float aI = 0.0f, aop = 0.0f;
                        if (s->dm_emissive)
                            for (int ch = 0; ch < 3; ch++) aI += gA.c[ch] * plf_slope(&s->emission.plf[ch], k.rho);
                        if (shaded) {
                            float ag[6];
                            const col3 aS = cmul(cscale(gA, Tr), LiK);
                            dm_shade_adjoint(s, &sd, &o, k.rho, vneg(R.D), Wi, aS, &aI, &aop, ag);
                            if (sd.type != 1)
                                for (int i = 0; i < 6; i++) dm_scatter_rho(&sd.g[i], ag[i], g_rho);
                        }
                        dm_scatter_rho(&k, aI, g_rho);
                        const float at = a + aop / s->dm_scale;
                        if (at != 0.0f) dm_scatter(s, &k, &o, at, g_rho, g_tf);
                    } else if (a != 0.0f) {
                        dm_scatter(s, &k, &o, a, g_rho, g_tf);
                    }
                }
                T = T * (1.0f - w);
                tau = -er_logf(rng_get1(rng));
            }
        }
        dda_advance(s, &d, e);
    }
    return s->dm_model == 1 ? cadd(L, E) : L;
}

typedef struct {
    or_scene local;
    int spp;
    uint32_t view, first;
    int row0, row1;
    float* sum;            /* W*H*3 */
    float* samples;        /* W*H*spp*3 or NULL (sample-major: (s*H*W + p)*3) */
    const float* dimg;     /* adjoint: dLoss/dImage-sum per pixel, W*H*3 */
    const float* fwd;      /* adjoint: the forward samples */
    float* g_rho;          /* per-thread gradient buffers */
    float* g_tf;
} dm_job_t;

static void* dm_job_run(void* arg)
{
    dm_job_t* j = (dm_job_t*)arg;
    or_scene* s = &j->local;
    const int W = s->film[0], H = s->film[1];
    for (int y = j->row0; y < j->row1; y++)
        for (int x = 0; x < W; x++) {
            const uint32_t pix = (uint32_t)y * (uint32_t)W + (uint32_t)x;
            float acc[3] = { 0.0f, 0.0f, 0.0f };
            for (int k = 0; k < j->spp; k++) {
                rng_t rng;
                er_seed_lanes(s->st.seed, j->view, pix, j->first + (uint32_t)k, &rng.s0, &rng.s1);
                const size_t q = ((size_t)k * (size_t)W * (size_t)H + pix) * 3;
                if (j->dimg) {
                    const col3 g = C3(j->dimg[3 * pix], j->dimg[3 * pix + 1], j->dimg[3 * pix + 2]);
                    const col3 Lt = C3(j->fwd[q], j->fwd[q + 1], j->fwd[q + 2]);
                    dm_sample(s, x, y, j->view, pix, j->first + (uint32_t)k, &rng, &g, Lt, j->g_rho, j->g_tf);
                } else {
                    const col3 L = dm_sample(s, x, y, j->view, pix, j->first + (uint32_t)k, &rng, NULL, C3(0, 0, 0), NULL, NULL);
                    acc[0] += L.c[0]; acc[1] += L.c[1]; acc[2] += L.c[2];
                    if (j->samples) { j->samples[q] = L.c[0]; j->samples[q + 1] = L.c[1]; j->samples[q + 2] = L.c[2]; }
                }
                s->samples++;
            }
            if (!j->dimg) { j->sum[3 * pix] = acc[0]; j->sum[3 * pix + 1] = acc[1]; j->sum[3 * pix + 2] = acc[2]; }
        }
    return NULL;
}

static void dm_run(or_scene* s, dm_job_t* proto, int nthreads, float* g_rho, float* g_tf)
{
    const int H = s->film[1];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > H) nthreads = H;
    const size_t nvox = (size_t)s->res[0] * (size_t)s->res[1] * (size_t)s->res[2];
    dm_job_t* jobs = (dm_job_t*)calloc((size_t)nthreads, sizeof(dm_job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = *proto;
        jobs[t].local = *s;
        jobs[t].row0 = (int)((long long)H * t / nthreads);
        jobs[t].row1 = (int)((long long)H * (t + 1) / nthreads);
        if (proto->dimg) {
            jobs[t].g_rho = g_rho ? (float*)calloc(nvox, sizeof(float)) : NULL;
            jobs[t].g_tf = g_tf ? (float*)calloc((size_t)s->tf_n, sizeof(float)) : NULL;
        }
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, dm_job_run, &jobs[t]);
    dm_job_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    /* per-thread gradients summed in thread order */
    for (int t = 0; t < nthreads; t++) {
        if (jobs[t].g_rho) { for (size_t i = 0; i < nvox; i++) g_rho[i] += jobs[t].g_rho[i]; free(jobs[t].g_rho); }
        if (jobs[t].g_tf) { for (int i = 0; i < s->tf_n; i++) g_tf[i] += jobs[t].g_tf[i]; free(jobs[t].g_tf); }
    }
    free(jobs);
    free(th);
}

/* forward: per-pixel sums (W*H*3) and, if samples != NULL, every sample */
void ER_OR(dm_render)(or_scene* s, int32_t spp, uint32_t view, uint32_t first, float* sum, float* samples, int32_t nthreads)
{
    dm_job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.spp = spp; proto.view = view; proto.first = first; proto.sum = sum; proto.samples = samples;
    dm_run(s, &proto, nthreads, NULL, NULL);
}

/* adjoint: dimg = dLoss/d(pixel sum) (W*H*3), fwd = the forward samples;
   gradients are added to g_rho (density grid) and g_tf (opacity values) */
void ER_OR(dm_adjoint)(or_scene* s, int32_t spp, uint32_t view, uint32_t first, const float* dimg, const float* fwd,
                       float* g_rho, float* g_tf, int32_t nthreads)
{
    dm_job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.spp = spp; proto.view = view; proto.first = first; proto.dimg = dimg; proto.fwd = fwd;
    dm_run(s, &proto, nthreads, g_rho, g_tf);
}
