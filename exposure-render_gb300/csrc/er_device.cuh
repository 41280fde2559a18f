/*
 * er_device.cuh - device-side scene layout and the reference-order vector
 * algebra used by the transport kernels.
 *
 * Layout in HBM (one set per bound tracer, uploaded by er_runtime.cpp):
 *   - voxels: uint16, x-fastest (z*Rx*Ry + y*Rx + x), as Buffer3D stores them
 *     (Source/buffer3d.h:210-214);
 *   - sigma table: float[max_voxel+1], DensityScale * Opacity1D(I) for every
 *     integer intensity I.  GetIntensity returns an unsigned short
 *     (Source/volume.h:131-138), so the opacity transfer function is only ever
 *     evaluated at integers and the table holds exactly the values the
 *     reference computes per step (Source/raymarching.h:64,106);
 *   - transfer functions, lights and textures as POD blocks read with uniform
 *     (broadcast) loads.
 *
 * Everything in this file is `__device__ __forceinline__` and keeps the
 * reference's evaluation order; translation units that must reproduce the
 * reference bit-for-bit are compiled with --fmad=false.
 */
#ifndef ER_DEVICE_CUH
#define ER_DEVICE_CUH

#include <stdint.h>
#include <cuda_runtime.h>

#include "er_math.h"

#define ER_D __device__ __forceinline__

namespace erd {

/* ------------------------------------------------------------------ */
/* POD scene blocks                                                     */
/* ------------------------------------------------------------------ */

struct Plf {                 /* PiecewiseLinearFunction<128> (Source/plf.h:26-92) */
    int count;
    float range0, range1;
    float pos[128];
    float val[128];
};

struct Tfs {                 /* the four colour/scalar TFs read at scatter events */
    Plf diffuse[3];
    Plf specular[3];
    Plf glossiness;
    Plf emission[3];
    Plf opacity;             /* kept for the hybrid switch's opacity modulation */
};

struct Light {               /* ErLight + Shape (Source/erlight.h, Source/shape.h) */
    float tm[3][4];
    float inv_tm[3][4];
    int one_sided;
    int type;
    float size[3];
    float area;
    float inner_radius;
    float outer_radius;
    int visible;
    int texture_id;
    float multiplier;
    int unit;
    int tex_const;           /* 1 when the light's texture does not vary over the surface (a uniform
                                procedural texture, or none): tex_rgb is its value */
    float tex_rgb[3];
    float inner_c[3];        /* sphere lights with a rigid transform: the centre in world space and */
    float inner_r2;          /* (0.9 radius)^2 (< 0 otherwise): a segment with both ends inside cannot hit */
};

struct Object {              /* ErObject (Source/erobject.h:27-67) */
    Light shape;             /* the shape fields of a light record (tm, inv_tm, type, one_sided, size, radii);
                                the emitter fields are unused */
    int diffuse_texture_id;
    int specular_texture_id;
    int glossiness_texture_id;
    int pad;
};

struct Texture {             /* ErTexture + Procedural (Source/ertexture.h, Source/procedural.h) */
    int type;
    float output_level;
    int bitmap_id;
    int proc_type;
    float uniform[3];
    float checker1[3];
    float checker2[3];
    float offset[2];
    float repeat[2];
    int flip[2];
    Plf gradient[3];
};

struct Bitmap {              /* Bitmap (Source/bitmap.h): RGBA8, row-major */
    const uchar4* pixels;
    int res[2];
};

struct Clip {                /* ErClippingObject (Source/erclippingobject.h:27-58): Shape + Invert */
    float inv_tm[3][4];
    int type;
    float size[3];
    float outer_radius;
    int invert;
};

struct Params {
    /* volume (Source/volume.h:140-149) */
    const uint16_t* vox;
    const uint2* quad;       /* per voxel (x, y, z): the x/y 2x2 corner quad at z, packed uint16 pairs, or NULL */
    int qb_nbx;              /* quads in 8^3 bricks (brick-major, x fastest inside a brick): bricks along x;
                                0: quads x fastest over the whole volume */
    unsigned long long qb_slab;  /* bricked quads: entries per z-slab of bricks (nbx * nby * 512) */
    int tile_order;          /* wavefront: the samples of a sample row go to lanes in tiles of 32
                                pixels (1: 8x4, 2: 4x8, the default, 3: 16x2; films whose sides are
                                multiples of the tile's), else (0) row by row */
    int res[3];
    float minp[3];
    float inv_size[3];
    float half_size[3];      /* BoundingBox.MaxP = 0.5 * Size */
    float spacing[3];
    float min_step;
    const float* sigma;      /* DensityScale * Opacity(I), I in [0, sigma_n) */
    int sigma_n;
    const float4* shade_tab; /* per integer intensity I in [0, sigma_n), 3 records: (Diffuse1D(I), glossiness
                                exponent 1e6 * Glossiness1D(I)^7), (Specular1D(I), Opacity1D(I)),
                                (Emission1D(I), 0) */
    /* delta tracking: majorant per brick of `brick`^3 voxels */
    int free_flight;
    int brick;
    int nb[3];
    const float* majorant;
    float gm_inv_max;        /* 1 / max gradient magnitude (hybrid switch) */
    /* camera (Source/camera.h:98-116) */
    int film[2];
    float pos[3], N[3], U[3], V[3];
    float screen00, screen10, inv_screen0, inv_screen1;
    float clip_near, clip_far, aperture, focal_distance;
    /* settings (Source/rendersettings.h) */
    float step_primary, step_shadow, density_scale, max_shadow_distance;
    int shadows;
    int gradient_mode;
    int shading_type;
    int apply_shading_type;
    int opacity_modulated;
    float gradient_factor, gradient_threshold;
    int mis;
    float volume_ior;
    uint32_t seed;
    int stratify;            /* multi-sample renders: stratified dimensions from er_stratified_sample */
    /* lights (tracer's LightIDs resolved to light records) */
    int light_count;
    const Light* lights;     /* light_count entries, in LightIDs order; NULL entries are skipped */
    const int* light_valid;  /* 1 where LightIDs[i] named a bound light */
    const int* light_ids;    /* the tracer's LightIDs (slot -> light ID) */
    /* surface objects: the first ObjectIDs.Count bound objects in bind-list
       order, as IntersectObjects indexes gpObjects[i] (Source/objects.h:45-62) */
    int object_count;
    const Object* objects;
    const Texture* textures;
    int n_textures;
    const Bitmap* bitmaps;   /* indexed by ErTexture::BitmapID */
    int n_bitmaps;
    const Tfs* tfs;
    int* err;                /* device error word (bit 0: a march exceeded its step budget) */
    /* clipping objects: the tracer's ClippingObjectIDs resolved to their shapes */
    int clip_count;
    const Clip* clips;
    /* 1 for a volume bound without NormalizeSize: Volume's copy scales the
       spacing by 0 (Source/volume.h:106-117), so its box has no extent and
       no ray meets the volume */
    int box_empty;
};

/* index of voxel (x, y, z)'s corner quad: x fastest over the volume, or in
   8^3 bricks (brick-major, x fastest inside a brick) when nbx > 0, which
   keeps a trilinear lookup's two z-slices 512 bytes apart instead of a whole
   slice */
__host__ __device__ __forceinline__ size_t quad_index(int x, int y, int z, int rx, int ry, int nbx, unsigned long long slab)
{
    if (nbx > 0)
        return (size_t)(z >> 3) * (size_t)slab + ((size_t)(y >> 3) * (size_t)nbx + (size_t)(x >> 3)) * 512u +
               (size_t)(((z & 7) << 6) | ((y & 7) << 3) | (x & 7));
    return (size_t)z * (size_t)rx * (size_t)ry + (size_t)y * (size_t)rx + (size_t)x;
}

/* ------------------------------------------------------------------ */
/* vector algebra in the order of Source/vector.h                       */
/* ------------------------------------------------------------------ */

struct v3 { float x, y, z; };
struct v2 { float x, y; };
struct c3 { float r, g, b; };

ER_D v3 V3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
ER_D v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
ER_D v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
ER_D v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
ER_D v3 vscale(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
ER_D v3 vneg(v3 a) { return V3(-a.x, -a.y, -a.z); }
ER_D float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ER_D float vlen2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
ER_D float vlen(v3 a) { return sqrtf(vlen2(a)); }
ER_D v3 vnorm(v3 a) { const float L = vlen(a); return V3(a.x / L, a.y / L, a.z / L); }
ER_D v3 vcross(v3 a, v3 b) { return V3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)); }
ER_D float vabsdot(v3 a, v3 b) { return fabsf(vdot(a, b)); }
ER_D float vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
ER_D v3 vload(const float* p) { return V3(p[0], p[1], p[2]); }

/* std::min / std::max and ExposureRender::Min / Max / Clamp semantics */
ER_D float smin(float a, float b) { return (b < a) ? b : a; }
ER_D float smax(float a, float b) { return (a < b) ? b : a; }
ER_D float emin(float a, float b) { return a < b ? a : b; }
ER_D float emax(float a, float b) { return a > b ? a : b; }
ER_D float eclamp(float v, float lo, float hi) { return emax(lo, emin(v, hi)); }
ER_D int iclamp(int v, int lo, int hi) { const int m = v < hi ? v : hi; return lo > m ? lo : m; }

ER_D c3 C3(float r, float g, float b) { c3 c; c.r = r; c.g = g; c.b = b; return c; }
ER_D c3 cadd(c3 a, c3 b) { return C3(a.r + b.r, a.g + b.g, a.b + b.b); }
ER_D c3 csub(c3 a, c3 b) { return C3(a.r - b.r, a.g - b.g, a.b - b.b); }
ER_D c3 cmul(c3 a, c3 b) { return C3(a.r * b.r, a.g * b.g, a.b * b.b); }
ER_D c3 cscale(c3 a, float s) { return C3(a.r * s, a.g * s, a.b * s); }
ER_D c3 cdivs(c3 a, float s) { return C3(a.r / s, a.g / s, a.b / s); }
ER_D bool cblack(c3 a) { return a.r == 0.0f && a.g == 0.0f && a.b == 0.0f; }

/* ------------------------------------------------------------------ */
/* RNG - Source/rng.h:26-66                                             */
/* ------------------------------------------------------------------ */

struct Rng {
    uint32_t s0, s1;
    ER_D float get1()
    {
        s0 = 36969u * (s0 & 65535u) + (s0 >> 16);
        s1 = 18000u * (s1 & 65535u) + (s1 >> 16);
        const uint32_t ires = (s0 << 16) + s1;
        return (__uint_as_float((ires & 0x007fffffu) | 0x40000000u) - 2.0f) / 2.0f;
    }
    /* Vec2f(Get1(), Get1()) evaluated right to left by the host compiler */
    ER_D v2 get2() { v2 v; v.y = get1(); v.x = get1(); return v; }
    ER_D v3 get3() { v3 v; v.z = get1(); v.y = get1(); v.x = get1(); return v; }
};

/* ------------------------------------------------------------------ */
/* transfer functions - Source/plf.h:68-91                              */
/* ------------------------------------------------------------------ */

ER_D float plf_eval(const Plf& p, float x)
{
    const int n = p.count;
    if (n <= 0) return 0.0f;
    if (x < p.range0) return p.val[0];
    if (x > p.range1) return p.val[n - 1];
    for (int i = 1; i < n; i++) {
        const float P1 = p.pos[i - 1];
        const float P2 = p.pos[i];
        const float DeltaP = P2 - P1;
        const float LerpT = (x - P1) / DeltaP;
        if (x >= P1 && x < P2) return p.val[i - 1] + LerpT * (p.val[i] - p.val[i - 1]);
    }
    return 0.0f;
}

ER_D c3 ctf_eval(const Plf* t, float x) { return C3(plf_eval(t[0], x), plf_eval(t[1], x), plf_eval(t[2], x)); }

}  // namespace erd

#endif
