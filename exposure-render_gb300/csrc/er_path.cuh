/*
 * er_path.cuh - one camera path of Exposure Render's single-scattering
 * estimator on the GPU, in the reference's evaluation order.
 *
 * Function-by-function counterpart of the reference transport code
 * (Source/singlescattering.h, Source/transport.h, Source/raymarching.h,
 * Source/lights.h, Source/shader.h, Source/volumes.h, Source/buffer3d.h).
 * Include only from translation units compiled with --fmad=false.
 */
#ifndef ER_PATH_CUH
#define ER_PATH_CUH

#include <float.h>

#include "er_device.cuh"

namespace erd {

#define ER_PI_F 3.141592654f
#define ER_INV_PI_F 0.31830988618379067154f
#define ER_INV_TWO_PI_F 0.15915494309189533577f
#define ER_RAY_EPS 0.0001f
#define ER_INV_FOUR_PI_EXPANDED (1.0f / 4.0f * ER_PI_F)   /* INV_FOUR_PI_F as the macro expands */

/* ---- volume access: Source/buffer3d.h:210-242, Source/volume.h:131-138 ---- */

ER_D float voxel(const Params& P, int x, int y, int z)
{
    const int cx = iclamp(x, 0, P.res[0] - 1);
    const int cy = iclamp(y, 0, P.res[1] - 1);
    const int cz = iclamp(z, 0, P.res[2] - 1);
    const size_t idx = (size_t)cz * (size_t)P.res[0] * (size_t)P.res[1] + (size_t)cy * (size_t)P.res[0] + (size_t)cx;
    return (float)__ldg(P.vox + idx);
}

/* Lerp (Source/geometry.h:87-90) stored into unsigned short: truncation of a
   non-negative value below 65536 */
ER_D float lerp_u16(float t, float a, float b)
{
    const float r = (1.0f - t) * a + t * b;
    return truncf(r);
}

/* the eight corners read voxel by voxel, clamped to the volume: lookups
   without corner quads or at the x/y faces (out of line: it is rare, and
   inlined it would sit in the trackers' hot loops) */
static __device__ __noinline__ float get_intensity_voxels(const Params& P, int vx, int vy, int vz, float dx, float dy, float dz)
{
    const float d00 = lerp_u16(dx, voxel(P, vx, vy, vz), voxel(P, vx + 1, vy, vz));
    const float d10 = lerp_u16(dx, voxel(P, vx, vy + 1, vz), voxel(P, vx + 1, vy + 1, vz));
    const float d01 = lerp_u16(dx, voxel(P, vx, vy, vz + 1), voxel(P, vx + 1, vy, vz + 1));
    const float d11 = lerp_u16(dx, voxel(P, vx, vy + 1, vz + 1), voxel(P, vx + 1, vy + 1, vz + 1));
    const float d0 = lerp_u16(dy, d00, d10);
    const float d1 = lerp_u16(dy, d01, d11);
    return lerp_u16(dz, d0, d1);
}

/* the trilinear lookup at local voxel coordinates (Lx, Ly, Lz) */
ER_D float get_intensity_local(const Params& P, float Lx, float Ly, float Lz)
{
    const int vx = (int)floorf(Lx);
    const int vy = (int)floorf(Ly);
    const int vz = (int)floorf(Lz);
    const float dx = Lx - (float)vx;
    const float dy = Ly - (float)vy;
    const float dz = Lz - (float)vz;
    if (P.quad && vx >= 0 && vx < P.res[0] - 1 && vy >= 0 && vy < P.res[1] - 1) {
        /* the same eight corners from two 8-byte quad loads (no x/y clamping
           needed inside the volume; z clamps per corner) */
        const int z0 = iclamp(vz, 0, P.res[2] - 1), z1 = iclamp(vz + 1, 0, P.res[2] - 1);
        size_t i0, i1;
        if (P.qb_nbx > 0) {
            const size_t xy = ((size_t)(vy >> 3) * (size_t)P.qb_nbx + (size_t)(vx >> 3)) * 512u + (size_t)(((vy & 7) << 3) | (vx & 7));
            i0 = (size_t)(z0 >> 3) * (size_t)P.qb_slab + xy + (size_t)((z0 & 7) << 6);
            i1 = (size_t)(z1 >> 3) * (size_t)P.qb_slab + xy + (size_t)((z1 & 7) << 6);
        } else {
            const size_t slice = (size_t)P.res[0] * (size_t)P.res[1];
            const size_t xy = (size_t)vy * (size_t)P.res[0] + (size_t)vx;
            i0 = (size_t)z0 * slice + xy;
            i1 = (size_t)z1 * slice + xy;
        }
        const uint2 a = __ldg(P.quad + i0);
        const uint2 b = __ldg(P.quad + i1);
        const float q00 = lerp_u16(dx, (float)(a.x & 0xffffu), (float)(a.x >> 16));
        const float q10 = lerp_u16(dx, (float)(a.y & 0xffffu), (float)(a.y >> 16));
        const float q01 = lerp_u16(dx, (float)(b.x & 0xffffu), (float)(b.x >> 16));
        const float q11 = lerp_u16(dx, (float)(b.y & 0xffffu), (float)(b.y >> 16));
        return lerp_u16(dz, lerp_u16(dy, q00, q10), lerp_u16(dy, q01, q11));
    }
    return get_intensity_voxels(P, vx, vy, vz, dx, dy, dz);
}

ER_D void local_coords(const Params& P, v3 p, float& Lx, float& Ly, float& Lz)
{
    const v3 off = V3(p.x - P.minp[0], p.y - P.minp[1], p.z - P.minp[2]);
    Lx = off.x * P.inv_size[0] * (float)P.res[0];
    Ly = off.y * P.inv_size[1] * (float)P.res[1];
    Lz = off.z * P.inv_size[2] * (float)P.res[2];
}

ER_D float get_intensity(const Params& P, v3 p)
{
    float Lx, Ly, Lz;
    local_coords(P, p, Lx, Ly, Lz);
    return get_intensity_local(P, Lx, Ly, Lz);
}

/* DensityScale * Opacity1D.Evaluate(I) from the integer-intensity table */
ER_D float sigma_at(const Params& P, float I)
{
    int i = (int)I;
    i = i < 0 ? 0 : (i >= P.sigma_n ? P.sigma_n - 1 : i);
    return __ldg(P.sigma + i);
}

/* The transfer functions the shading reads at a scatter event, at its
   intensity I.  I is an integer (GetIntensity returns an unsigned short,
   Source/volume.h:131-138), so a per-tracer table built with the same
   evaluations (k_shade_table) holds exactly the floats ctf_eval / plf_eval
   give at I, without the node scans. */
ER_D float opacity_at(const Params& P, float I)
{
    int i = (int)I;
    i = i < 0 ? 0 : (i >= P.sigma_n ? P.sigma_n - 1 : i);
    return __ldg(&P.shade_tab[3 * i + 1].w);
}

struct ShadeTF {
    c3 Kd, Ks, Le;
    float exponent, opacity;
};

ER_D void shade_tf(const Params& P, float I, ShadeTF& s)
{
    int i = (int)I;
    i = i < 0 ? 0 : (i >= P.sigma_n ? P.sigma_n - 1 : i);
    const float4 a = __ldg(P.shade_tab + 3 * i), b = __ldg(P.shade_tab + 3 * i + 1), c = __ldg(P.shade_tab + 3 * i + 2);
    s.Kd = C3(a.x, a.y, a.z);
    s.exponent = a.w;
    s.Ks = C3(b.x, b.y, b.z);
    s.opacity = b.w;
    s.Le = C3(c.x, c.y, c.z);
}

/* ---- gradients: Source/volumes.h:31-114 ---- */

ER_D v3 gdelta(const Params& P, int axis) { return V3(axis == 0 ? P.min_step : 0.0f, axis == 1 ? P.min_step : 0.0f, axis == 2 ? P.min_step : 0.0f); }

ER_D v3 gradient_cd(const Params& P, v3 p)
{
    const v3 dx = gdelta(P, 0), dy = gdelta(P, 1), dz = gdelta(P, 2);
    const float i00 = get_intensity(P, vadd(p, dx)), i01 = get_intensity(P, vsub(p, dx));
    const float i10 = get_intensity(P, vadd(p, dy)), i11 = get_intensity(P, vsub(p, dy));
    const float i20 = get_intensity(P, vadd(p, dz)), i21 = get_intensity(P, vsub(p, dz));
    return V3(i01 - i00, i11 - i10, i21 - i20);
}

ER_D v3 gradient_fd(const Params& P, v3 p)
{
    const float i0 = get_intensity(P, p);
    const float i1 = get_intensity(P, vadd(p, gdelta(P, 0)));
    const float i2 = get_intensity(P, vadd(p, gdelta(P, 1)));
    const float i3 = get_intensity(P, vadd(p, gdelta(P, 2)));
    return V3(i0 - i1, i0 - i2, i0 - i3);
}

ER_D v3 vlerp(v3 a, v3 b, float c) { return vadd(a, vscale(vsub(b, a), c)); }

static __device__ __noinline__ v3 gradient_filtered(const Params& P, v3 p)
{
    const float o = P.min_step;
    const v3 G0 = gradient_cd(P, p);
    const v3 G1 = gradient_cd(P, vadd(p, V3(-o, -o, -o)));
    const v3 G2 = gradient_cd(P, vadd(p, V3(o, o, o)));
    const v3 G3 = gradient_cd(P, vadd(p, V3(-o, o, -o)));
    const v3 G4 = gradient_cd(P, vadd(p, V3(o, -o, o)));
    const v3 G5 = gradient_cd(P, vadd(p, V3(-o, -o, o)));
    const v3 G6 = gradient_cd(P, vadd(p, V3(o, o, -o)));
    const v3 G7 = gradient_cd(P, vadd(p, V3(-o, o, o)));
    const v3 G8 = gradient_cd(P, vadd(p, V3(o, -o, -o)));
    const v3 L0 = vlerp(vlerp(G1, G2, 0.5f), vlerp(G3, G4, 0.5f), 0.5f);
    const v3 L1 = vlerp(vlerp(G5, G6, 0.5f), vlerp(G7, G8, 0.5f), 0.5f);
    return vlerp(G0, vlerp(L0, L1, 0.5f), 0.75f);
}

/* functions called once per path or per light are kept out of line, so the
   free-flight loops do not carry their registers and code */
#define ER_COLD static __device__ __noinline__

ER_D v3 normalized_gradient(const Params& P, v3 p)
{
    v3 g;
    if (P.gradient_mode == 1) g = gradient_cd(P, p);
    else if (P.gradient_mode == 2) g = gradient_filtered(P, p);
    else g = gradient_fd(P, p);
    return vnorm(g);
}

/* GradientCD and GradientMagnitude read the same six intensities
   (p -/+ the gradient delta of each axis): read once, both follow */
struct Grad6 {
    float m[3], p[3];    /* I(p - d_i), I(p + d_i) */
};

ER_D void gradient_samples(const Params& P, v3 p, Grad6& g)
{
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const v3 d = gdelta(P, i);
        g.m[i] = get_intensity(P, vsub(p, d));
        g.p[i] = get_intensity(P, vadd(p, d));
    }
}

/* gradient_cd from the six samples */
ER_D v3 gradient_cd6(const Grad6& g) { return V3(g.m[0] - g.p[0], g.m[1] - g.p[1], g.m[2] - g.p[2]); }

/* gradient_magnitude from the six samples */
ER_D float gradient_magnitude6(const Params& P, const Grad6& g)
{
    float sum = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float D = g.m[i] - g.p[i];
        D *= 0.5f / P.spacing[i];
        sum += D * D;
    }
    return sqrtf(sum);
}

ER_D float gradient_magnitude(const Params& P, v3 p)
{
    float sum = 0.0f;
    for (int i = 0; i < 3; i++) {
        const v3 d = gdelta(P, i);
        float D = get_intensity(P, vsub(p, d)) - get_intensity(P, vadd(p, d));
        D *= 0.5f / P.spacing[i];
        sum += D * D;
    }
    return sqrtf(sum);
}

/* Out-of-line copies of the elementary functions for code that runs once per
   event or per light sample (shading, light and BSDF sampling, shape UVs):
   one copy each instead of one inlined copy per call site keeps the shade
   stage within the instruction cache.  Same functions, same results; the
   tracking loops keep the inlined er_logf. */
ER_COLD float pow_c(float x, float y) { return er_powf(x, y); }
ER_COLD float exp_c(float x) { return er_expf(x); }
ER_COLD float acos_c(float x) { return er_acosf(x); }
ER_COLD float atan2_c(float y, float x) { return er_atan2f(y, x); }
ER_COLD v2 sincos_c(float x)
{
    v2 r;
    er_sincosf(x, &r.x, &r.y);
    return r;
}

/* ---- geometry ---- */

struct Ray { v3 O, D; float MinT, MaxT; };

ER_D v3 ray_at(const Ray& r, float t) { return vadd(r.O, vscale(vnorm(r.D), t)); }

struct Isect {
    bool valid, front;
    float near_t, far_t;
    v3 P, N;
    v2 UV;
    ER_D void invalid()
    {
        valid = false; front = true; near_t = 0.0f; far_t = FLT_MAX;
        P = V3(0, 0, 0); N = V3(0, 0, 0); UV.x = 0.0f; UV.y = 0.0f;
    }
};

ER_D v3 xform_point(const float m[3][4], v3 p)
{
    return V3(m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3],
              m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3],
              m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3]);
}
ER_D v3 xform_vector(const float m[3][4], v3 v)
{
    return V3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z,
              m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}
ER_D Ray xform_ray(const float m[3][4], const Ray& r)
{
    Ray t;
    const v3 Pp = xform_point(m, r.O);
    const v3 MinP = xform_point(m, ray_at(r, r.MinT));
    const v3 MaxP = xform_point(m, ray_at(r, r.MaxT));
    t.O = Pp;
    t.D = vnorm(vsub(MaxP, t.O));
    t.MinT = vlen(vsub(MinP, t.O));
    t.MaxT = vlen(vsub(MaxP, t.O));
    return t;
}

ER_D float spherical_theta(v3 w) { return acos_c(eclamp(w.y, -1.0f, 1.0f)); }
ER_D float spherical_phi(v3 w)
{
    const float p = atan2_c(w.z, w.x);
    return (p < 0.0f) ? p + 2.0f * ER_PI_F : p;
}

/* IntersectBox (Source/box.h:51-83); `full` also fills P and N */
ER_D void intersect_box(const Ray& R, v3 mn, v3 mx, Isect& I, bool full)
{
    const v3 InvR = V3(1.0f / R.D.x, 1.0f / R.D.y, 1.0f / R.D.z);
    const v3 B = vmul(InvR, vsub(mn, R.O));
    const v3 T = vmul(InvR, vsub(mx, R.O));
    const v3 MinT = V3(smin(T.x, B.x), smin(T.y, B.y), smin(T.z, B.z));
    const v3 MaxT = V3(smax(T.x, B.x), smax(T.y, B.y), smax(T.z, B.z));
    const float LargestMinT = fmaxf(fmaxf(MinT.x, MinT.y), fmaxf(MinT.x, MinT.z));
    const float LargestMaxT = fminf(fminf(MaxT.x, MaxT.y), fminf(MaxT.x, MaxT.z));
    if (LargestMaxT < LargestMinT) return;
    I.near_t = LargestMinT > 0.0f ? LargestMinT : 0.0f;
    I.far_t = LargestMaxT;
    if (I.near_t < R.MinT || I.near_t > R.MaxT) return;
    I.valid = true;
    if (full) {
        I.P = ray_at(R, I.near_t);
        float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
        if (I.P.x <= mn.x + 0.0001f) n0 = -1.0f;
        if (I.P.x >= mx.x - 0.0001f) n0 = 1.0f;
        if (I.P.y <= mn.y + 0.0001f) n1 = -1.0f;
        if (I.P.y >= mx.y - 0.0001f) n1 = 1.0f;
        if (I.P.z <= mn.z + 0.0001f) n2 = -1.0f;
        if (I.P.z >= mx.z - 0.0001f) n2 = 1.0f;
        I.N = V3(n0, n1, n2);
        I.UV.x = 0.0f; I.UV.y = 0.0f;
    }
}

/* The volume's bounding box (Source/raymarching.h:32-36 and :75-79 intersect
   it first).  A volume bound without NormalizeSize has no extent
   (Source/volume.h:106-117 scales its spacing by 0): no ray meets it. */
ER_D void intersect_volume(const Params& P, const Ray& R, Isect& I)
{
    if (P.box_empty) return;
    intersect_box(R, vload(P.minp), vload(P.half_size), I, false);
}

/* Clipping objects (ErClippingObject, Source/erclippingobject.h:27-58: a
   Shape and Invert; bound by BindClippingObject, Source/core.cu:96-104, and
   listed in the tracer's ClippingObjectIDs, Source/ertracer.h:100-116).  The
   reference binds them but no transport code reads them; here a point of the
   volume is clipped - its extinction counts as zero in free flight and in
   shadow rays - when it lies inside a clipping object's shape, or outside it
   when Invert is set; with several objects, any one of them clips.  Inside
   is tested in the shape's local frame (InvTM) with the reference's
   predicates: InsidePlane z > 0 (Source/plane.h:90-93; also for disks and
   rings, which have no predicate of their own), InsideBox open slabs of
   Size (Source/box.h:116-120), InsideSphere Length < OuterRadius
   (Source/sphere.h:147-150), InsideCylinder radial distance in x/z below
   OuterRadius and |y| below half of Size[2] (Source/cylinder.h:96-99, with
   the height Shape::Update uses, Source/shape.h:100). */
/* out of line: only views with clipping objects call it */
ER_COLD bool clipped(const Params& P, v3 p)
{
    for (int i = 0; i < P.clip_count; i++) {
        const Clip& c = P.clips[i];
        const v3 q = xform_point(c.inv_tm, p);
        bool in;
        switch (c.type) {
        case 0: case 1: case 2: in = q.z > 0.0f; break;
        case 3: {
            const float h0 = 0.5f * c.size[0], h1 = 0.5f * c.size[1], h2 = 0.5f * c.size[2];
            in = q.x > -h0 && q.x < h0 && q.y > -h1 && q.y < h1 && q.z > -h2 && q.z < h2;
            break;
        }
        case 4: in = vlen(q) < c.outer_radius; break;
        case 5: in = sqrtf((q.x * q.x) + (q.z * q.z)) < c.outer_radius && fabsf(q.y) < (0.5f * c.size[2]); break;
        default: in = false; break;
        }
        if (in != (c.invert != 0)) return true;
    }
    return false;
}

/* DensityScale * Opacity1D(I(p)) at a point of a free-flight or shadow
   march, zero where a clipping object removes the volume (no lookup) */
ER_D float sigma_point(const Params& P, v3 p)
{
    if (P.clip_count > 0 && clipped(P, p)) return 0.0f;
    return sigma_at(P, get_intensity(P, p));
}

/* sigma_point at a tentative collision of a tracker in majorant brick
   (bx, by, bz): the local coordinates are clamped to the brick's extent
   [b B, (b + 1) B] per axis before the lookup, so that it blends only
   voxels of the brick's footprint (b B .. (b + 1) B), whose maximum the
   brick's majorant bounds.  The clamp moves a point only when float
   rounding put it outside its DDA brick (a distance of a few ulps). */
ER_D float sigma_point_in_brick(const Params& P, v3 p, int bx, int by, int bz)
{
    if (P.clip_count > 0 && clipped(P, p)) return 0.0f;
    float Lx, Ly, Lz;
    local_coords(P, p, Lx, Ly, Lz);
    const float B = (float)P.brick;
    const float x0 = (float)bx * B, y0 = (float)by * B, z0 = (float)bz * B;
    const float x1 = x0 + B, y1 = y0 + B, z1 = z0 + B;
    Lx = Lx < x0 ? x0 : (x1 < Lx ? x1 : Lx);
    Ly = Ly < y0 ? y0 : (y1 < Ly ? y1 : Ly);
    Lz = Lz < z0 ? z0 : (z1 < Lz ? z1 : Lz);
    return sigma_at(P, get_intensity_local(P, Lx, Ly, Lz));
}

/* IntersectPlane(R, OneSided, Int) - Source/plane.h:41-62 */
ER_D void intersect_plane_inf(const Ray& R, int one_sided, Isect& I)
{
    if (fabsf(R.O.z - R.D.z) < ER_RAY_EPS) return;
    I.near_t = (0.0f - R.O.z) / R.D.z;
    if (I.near_t < R.MinT || I.near_t > R.MaxT) return;
    I.P = ray_at(R, I.near_t);
    I.UV.x = I.P.x; I.UV.y = I.P.y;
    I.N = V3(0.0f, 0.0f, 1.0f);
    if (one_sided && R.D.z >= 0.0f) {
        I.front = false;
        I.N = V3(0.0f, 0.0f, -1.0f);
    }
    I.valid = true;
}

ER_D float v2len(v2 a) { return sqrtf(a.x * a.x + a.y * a.y); }

ER_COLD void intersect_shape(const Light& L, const Ray& R, Isect& I)
{
    switch (L.type) {
    case 0: {   /* Source/plane.h:76-88 */
        intersect_plane_inf(R, L.one_sided, I);
        const float sx = L.size[0], sy = L.size[1];
        if (I.valid && (I.UV.x < -0.5f * sx || I.UV.x > 0.5f * sx || I.UV.y < -0.5f * sy || I.UV.y > 0.5f * sy)) I.valid = false;
        I.UV.x /= sx; I.UV.y /= sy;
        I.UV.x = I.UV.x + 0.5f; I.UV.y = I.UV.y + 0.5f;
        I.UV.x = 1.0f - I.UV.x;
        break;
    }
    case 1: {   /* Source/disk.h:37-49 */
        intersect_plane_inf(R, L.one_sided, I);
        if (I.valid && v2len(I.UV) > L.outer_radius) I.valid = false;
        const float dia = 2.0f * L.outer_radius;
        I.UV.x /= dia; I.UV.y /= dia;
        I.UV.x = I.UV.x + 0.5f; I.UV.y = I.UV.y + 0.5f;
        I.UV.x = 1.0f - I.UV.x;
        break;
    }
    case 2: {   /* Source/ring.h:45-57 */
        intersect_plane_inf(R, L.one_sided, I);
        if (I.valid && (v2len(I.UV) < L.inner_radius || v2len(I.UV) > L.outer_radius)) I.valid = false;
        const float dia = 2.0f * L.outer_radius;
        I.UV.x /= dia; I.UV.y /= dia;
        I.UV.x = I.UV.x + 0.5f; I.UV.y = I.UV.y + 0.5f;
        I.UV.x = 1.0f - I.UV.x;
        break;
    }
    case 3: {   /* Source/box.h:85-88 */
        const v3 s = V3(L.size[0], L.size[1], L.size[2]);
        intersect_box(R, vscale(s, -0.5f), vscale(s, 0.5f), I, true);
        break;
    }
    case 4: {   /* Source/sphere.h:84-140 */
        const float r = L.outer_radius;
        const float a = vdot(R.D, R.D);
        const float b = 2 * vdot(R.D, R.O);
        const float c = vdot(R.O, R.O) - (r * r);
        const float disc = b * b - 4 * a * c;
        if (disc < 0) return;
        const float ds = sqrtf(disc);
        float q;
        if (b < 0) q = (-b - ds) / 2.0f;
        else q = (-b + ds) / 2.0f;
        float t0 = q / a;
        float t1 = c / q;
        if (t0 > t1) { const float tmp = t0; t0 = t1; t1 = tmp; }
        if (t0 >= R.MinT && t0 < R.MaxT) I.near_t = t0;
        else {
            if (t1 >= R.MinT && t1 < R.MaxT) I.near_t = t1;
            else return;
        }
        if (I.near_t < R.MinT || I.near_t > R.MaxT) return;
        I.valid = true;
        I.P = ray_at(R, I.near_t);
        I.N = vnorm(I.P);
        const v3 Vn = vnorm(I.P);
        I.UV.x = ER_INV_TWO_PI_F * spherical_phi(Vn);
        I.UV.y = 1.0f - (ER_INV_PI_F * spherical_theta(Vn));
        break;
    }
    default: break;
    }
}

/* ---- sampling ---- */

ER_D v2 concentric_sample_disk(v2 U)   /* Source/montecarlo.h:86-137 */
{
    float r, theta;
    const float sx = 2 * U.x - 1;
    const float sy = 2 * U.y - 1;
    v2 out;
    if (sx == 0.0f && sy == 0.0f) { out.x = 0.0f; out.y = 0.0f; return out; }
    if (sx >= -sy) {
        if (sx > sy) { r = sx; theta = (sy > 0.0f) ? sy / r : 8.0f + sy / r; }
        else { r = sy; theta = 2.0f - sx / r; }
    } else {
        if (sx <= sy) { r = -sx; theta = 4.0f - sy / r; }
        else { r = -sy; theta = 6.0f + sx / r; }
    }
    theta *= ER_PI_F / 4.f;
    const v2 scv = sincos_c(theta);
    const float sn = scv.x, cs = scv.y;
    out.x = r * cs;
    out.y = r * sn;
    return out;
}

struct Surf { v3 P, N; v2 UV; };

/* SampleLightSurface - Source/lights.h:28-42 and the shape samplers */
ER_COLD void sample_light_surface(const Light& L, v3 UVW, Surf& SS)
{
    SS.P = V3(0, 0, 0); SS.N = V3(0.0f, 0.0f, 1.0f); SS.UV.x = 0.0f; SS.UV.y = 0.0f;
    switch (L.type) {
    case 0:
        SS.P = V3(-0.5f + UVW.x, -0.5f + UVW.y, 0.0f);
        SS.UV.x = UVW.x; SS.UV.y = UVW.y;
        SS.P = vmul(SS.P, V3(L.size[0], L.size[1], 0.0f));
        break;
    case 1: {
        const float r = sqrtf(UVW.x);
        const float theta = 2.0f * ER_PI_F * UVW.y;
        const v2 scv = sincos_c(theta); const float sn = scv.x, cs = scv.y;
        SS.P = V3(r * cs, r * sn, 0.0f);
        SS.UV.x = UVW.x; SS.UV.y = UVW.y;
        SS.P = vscale(SS.P, L.outer_radius);
        break;
    }
    case 2: {
        const float inner = L.inner_radius / L.outer_radius;
        const float r = inner + (1.0f - inner) * sqrtf(UVW.x);
        const float theta = 2.0f * ER_PI_F * UVW.y;
        const v2 scv = sincos_c(theta); const float sn = scv.x, cs = scv.y;
        SS.P = V3(r * cs, r * sn, 0.0f);
        SS.P = vscale(SS.P, L.outer_radius);
        SS.UV.x = SS.P.x; SS.UV.y = SS.P.y;
        break;
    }
    case 3: {
        const int side = (int)floorf(UVW.x * 6.0f);
        v3 p = V3(0, 0, 0), n = SS.N;
        switch (side) {
        case 0: p = V3(0.5f, -0.5f + UVW.z, -0.5f + UVW.y); n = V3(1.0f, 0.0f, 0.0f); break;
        case 1: p = V3(-0.5f, -0.5f + UVW.z, -0.5f + UVW.y); n = V3(-1.0f, 0.0f, 0.0f); break;
        case 2: p = V3(-0.5f + UVW.y, 0.5f, -0.5f + UVW.z); n = V3(0.0f, 1.0f, 0.0f); break;
        case 3: p = V3(-0.5f + UVW.y, -0.5f, -0.5f + UVW.z); n = V3(0.0f, -1.0f, 0.0f); break;
        case 4: p = V3(-0.5f + UVW.y, -0.5f + UVW.z, 0.5f); n = V3(0.0f, 0.0f, 1.0f); break;
        case 5: p = V3(-0.5f + UVW.y, -0.5f + UVW.z, -0.5f); n = V3(0.0f, 0.0f, -1.0f); break;
        default: break;
        }
        SS.P = p; SS.N = n;
        SS.UV.x = UVW.y; SS.UV.y = UVW.z;
        SS.P = vmul(SS.P, V3(L.size[0], L.size[1], L.size[2]));
        break;
    }
    case 4: {
        const float z = 1.0f - 2.0f * UVW.x;
        const float r = sqrtf(smax(0.0f, 1.0f - z * z));
        const float phi = 2.0f * ER_PI_F * UVW.y;
        const v2 scv = sincos_c(phi); const float sn = scv.x, cs = scv.y;
        SS.P = V3(r * cs, r * sn, z);
        SS.N = SS.P;
        SS.UV.x = spherical_theta(SS.P);
        SS.UV.y = spherical_phi(SS.P);
        SS.P = vscale(SS.P, L.outer_radius);
        break;
    }
    default: break;
    }
    SS.P = xform_point(L.tm, SS.P);
    SS.N = xform_vector(L.tm, SS.N);
}

/* Buffer2D<ColorRGBAuc>::operator()(Vec2f, Normalized = true)
   (Source/buffer2d.h:227-254) and ColorXYZf::FromRGBAuc (Source/color.h:195-209).
   `float * ColorRGBAuc` converts the weight to the unsigned char component
   type and multiplies per component in unsigned char arithmetic
   (Source/color.h:282-283, Source/vector.h:183-190), colour sums wrap in
   unsigned char: the lookup returns the floor texel where the scaled
   coordinate is an integer and black elsewhere, as the reference does. */
ER_D uint8_t uc_weight(float w) { return (uint8_t)w; }

ER_D c3 bitmap_xyz(const Bitmap& B, v2 uv)
{
    const int w = B.res[0], h = B.res[1];
    const float U = uv.x * (float)w, V = uv.y * (float)h;
    int x0 = (int)floorf(U), x1 = (int)ceilf(U), y0 = (int)floorf(V), y1 = (int)ceilf(V);
    const float du = U - (float)x0;
    const float dv = V - (float)y0;
    x0 = min(max(x0, 0), w - 1);
    x1 = min(max(x1, 0), w - 1);
    y0 = min(max(y0, 0), h - 1);
    y1 = min(max(y1, 0), h - 1);
    const uchar4 v00 = B.pixels[(size_t)y0 * w + x0], v10 = B.pixels[(size_t)y0 * w + x1];
    const uchar4 v01 = B.pixels[(size_t)y1 * w + x0], v11 = B.pixels[(size_t)y1 * w + x1];
    const uint8_t wu0 = uc_weight(1.0f - du), wu1 = uc_weight(du);
    const uint8_t wv0 = uc_weight(1.0f - dv), wv1 = uc_weight(dv);
    const uint8_t a00[3] = { v00.x, v00.y, v00.z }, a10[3] = { v10.x, v10.y, v10.z };
    const uint8_t a01[3] = { v01.x, v01.y, v01.z }, a11[3] = { v11.x, v11.y, v11.z };
    uint8_t rgb[3];
    for (int c = 0; c < 3; c++) {
        const uint8_t top = (uint8_t)((uint8_t)(wu0 * a00[c]) + (uint8_t)(wu1 * a10[c]));
        const uint8_t bot = (uint8_t)((uint8_t)(wu0 * a01[c]) + (uint8_t)(wu1 * a11[c]));
        rgb[c] = (uint8_t)((uint8_t)(wv0 * top) + (uint8_t)(wv1 * bot));
    }
    const float k = 1.0f / 255.0f;
    const float r = k * (float)rgb[0], g = k * (float)rgb[1], b = k * (float)rgb[2];
    return C3(0.412453f * r + 0.357580f * g + 0.180423f * b,
              0.212671f * r + 0.715160f * g + 0.072169f * b,
              0.019334f * r + 0.119193f * g + 0.950227f * b);
}

/* EvaluateTexture - Source/textures.h:26-111 (procedural and bitmap textures) */
ER_COLD c3 evaluate_texture(const Params& P, int id, v2 UV)
{
    if (id < 0 || id >= P.n_textures) return C3(0, 0, 0);
    const Texture& T = P.textures[id];
    c3 L = C3(0, 0, 0);
    v2 t = UV;
    t.x *= T.repeat[0];
    t.y *= T.repeat[1];
    t.x += T.offset[0];
    t.y += 1.0f - T.offset[1];
    t.x = t.x - floorf(t.x);
    t.y = t.y - floorf(t.y);
    t.x = eclamp(t.x, 0.0f, 1.0f);
    t.y = eclamp(t.y, 0.0f, 1.0f);
    if (T.flip[0]) t.x = 1.0f - t.x;
    if (T.flip[1]) t.y = 1.0f - t.y;
    if (T.type == 0) {
        switch (T.proc_type) {
        case 0: L = C3(T.uniform[0], T.uniform[1], T.uniform[2]); break;
        case 1: {
            const int u = (int)(t.x * 2.0f), v = (int)(t.y * 2.0f);
            const bool first = (u % 2 == 0) ? (v % 2 == 0) : (v % 2 != 0);
            L = first ? C3(T.checker1[0], T.checker1[1], T.checker1[2]) : C3(T.checker2[0], T.checker2[1], T.checker2[2]);
            break;
        }
        case 2: L = ctf_eval(T.gradient, t.y); break;
        default: break;
        }
    } else if (T.type == 1 && T.bitmap_id >= 0 && T.bitmap_id < P.n_bitmaps && P.bitmaps[T.bitmap_id].pixels) {
        L = bitmap_xyz(P.bitmaps[T.bitmap_id], t);
    }
    return cscale(L, T.output_level);
}

/* EvaluateTexture(L.TextureID, UV) of a light; uniform textures were
   evaluated on the host (the same float products) */
ER_D c3 light_texture(const Params& P, const Light& L, v2 UV)
{
    if (L.tex_const) return C3(L.tex_rgb[0], L.tex_rgb[1], L.tex_rgb[2]);
    return evaluate_texture(P, L.texture_id, UV);
}

/* ---- shading: Source/shader.h ---- */

struct Shader {
    int type;            /* 0 BRDF, 1 isotropic phase */
    v3 Nn, Nu, Nv;
    c3 Kd, Ks;
    float ior, exponent;
};

ER_D void shader_init(Shader& sh, int type, v3 N, v3 Wo, c3 Kd, c3 Ks, float ior, float exponent)
{
    sh.type = type;
    sh.Nn = vnorm(N);
    sh.Nu = vnorm(vcross(N, Wo));
    sh.Nv = vnorm(vcross(N, sh.Nu));
    sh.Kd = Kd; sh.Ks = Ks; sh.ior = ior; sh.exponent = exponent;
}

ER_D v3 world_to_local(const Shader& sh, v3 W) { return V3(vdot(W, sh.Nu), vdot(W, sh.Nv), vdot(W, sh.Nn)); }
ER_D v3 local_to_world(const Shader& sh, v3 W)
{
    return V3(sh.Nu.x * W.x + sh.Nv.x * W.y + sh.Nn.x * W.z,
              sh.Nu.y * W.x + sh.Nv.y * W.y + sh.Nn.y * W.z,
              sh.Nu.z * W.x + sh.Nv.z * W.y + sh.Nn.z * W.z);
}

ER_D float fresnel_eval(float ei_, float et_, float cosi)
{
    cosi = eclamp(cosi, -1.0f, 1.0f);
    const bool entering = cosi > 0.0f;
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

ER_D float blinn_d(float e, v3 Wh) { return (e + 2) * ER_INV_TWO_PI_F * pow_c(fabsf(Wh.z), e); }

ER_D float blinn_pdf(float e, v3 Wo, v3 Wi)
{
    const v3 Wh = vnorm(vadd(Wo, Wi));
    const float ct = fabsf(Wh.z);
    float pdf = ((e + 1.0f) * pow_c(ct, e)) / (2.0f * ER_PI_F * 4.0f * vdot(Wo, Wh));
    if (vdot(Wo, Wh) <= 0.0f) pdf = 0.0f;
    return pdf;
}

ER_COLD c3 microfacet_f(const Shader& sh, v3 Wo, v3 Wi)
{
    const float co = fabsf(Wo.z), ci = fabsf(Wi.z);
    if (ci == 0.f || co == 0.f) return C3(0, 0, 0);
    v3 Wh = vadd(Wi, Wo);
    if (Wh.x == 0.f && Wh.y == 0.f && Wh.z == 0.f) return C3(0, 0, 0);
    Wh = vnorm(Wh);
    const float F = fresnel_eval(1.0f, sh.ior, vdot(Wi, Wh));
    const float NdotWh = fabsf(Wh.z), NdotWo = fabsf(Wo.z), NdotWi = fabsf(Wi.z);
    const float WOdotWh = vabsdot(Wo, Wh);
    const float G = smin(1.0f, smin((2.0f * NdotWh * NdotWo / WOdotWh), (2.0f * NdotWh * NdotWi / WOdotWh)));
    const float D = blinn_d(sh.exponent, Wh);
    const float den = 4.0f * ci * co;
    c3 r = cscale(sh.Ks, D);
    r = cscale(r, G);
    r = cscale(r, F);
    return cdivs(r, den);
}

ER_D bool same_hemisphere(v3 a, v3 b) { return (a.z * b.z) > 0.0f; }

ER_D c3 shader_f(const Shader& sh, v3 Wo, v3 Wi)
{
    if (sh.type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        const v3 Wil = world_to_local(sh, Wi);
        c3 R = C3(0, 0, 0);
        R = cadd(R, cscale(sh.Kd, ER_INV_PI_F));
        R = cadd(R, microfacet_f(sh, Wol, Wil));
        return R;
    }
    return cscale(sh.Kd, ER_INV_PI_F);
}

ER_D float shader_pdf(const Shader& sh, v3 Wo, v3 Wi)
{
    if (sh.type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        const v3 Wil = world_to_local(sh, Wi);
        float pdf = 0.0f;
        pdf += same_hemisphere(Wol, Wil) ? fabsf(Wil.z) * ER_INV_PI_F : 0.0f;
        pdf += same_hemisphere(Wol, Wil) ? blinn_pdf(sh.exponent, Wol, Wil) : 0.0f;
        return pdf;
    }
    return ER_INV_FOUR_PI_EXPANDED;
}

ER_D float power_heuristic(float fPdf, float gPdf)
{
    const float f = 1 * fPdf, g = 1 * gPdf;
    return (f * f) / (f * f + g * g);
}

/* ---- events ---- */

struct Event {
    int type;            /* 0 volume, 1 light, 2 object */
    bool valid;
    float T;
    v3 P, N, Wo;
    c3 Le;
};

/* the surface of an object event (ScatterEvent::UV and ::ObjectID), kept
   apart from Event so that volume-only code carries none of it */
struct ObjHit {
    v2 UV;
    int id;
};

/* step budget of a fixed-step march: the loop ends after at most
   (MaxT - MinT)/StepSize steps; a budget of twice that plus slack only trips
   when float accumulation stalls (a step below the ulp of t) */
ER_D long long march_budget(float t0, float t1, float step)
{
    const float n = (t1 - t0) / step;
    if (!(n < 1.0e9f)) return 2000000000LL;
    return (long long)(2.0f * n) + 64;
}

/* SampleVolume - Source/raymarching.h:30-71 */
template <bool WITH_NORMAL = true>
ER_D void sample_volume(const Params& P, const Ray& R, Rng& rng, Event& SE)
{
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return;
    float MinT = smax(Int.near_t, R.MinT);
    const float MaxT = smin(Int.far_t, R.MaxT);
    const float S = -er_logf(rng.get1()) / P.density_scale;
    float Sum = 0.0f;
    v3 Ps = V3(0, 0, 0);
    const float StepSize = P.step_primary * P.min_step;
    MinT += rng.get1() * StepSize;
    long long budget = march_budget(MinT, MaxT, StepSize);
    while (Sum < S) {
        Ps = vadd(R.O, vscale(R.D, MinT));
        if (MinT >= MaxT) return;
        if (--budget < 0) { atomicOr(P.err, 1); return; }
        const float SigmaT = sigma_point(P, Ps);
        Sum += SigmaT * StepSize;
        MinT += StepSize;
    }
    SE.valid = true;
    SE.T = MinT;
    SE.P = Ps;
    SE.N = WITH_NORMAL ? normalized_gradient(P, Ps) : V3(0.0f, 0.0f, 0.0f);
    SE.Wo = vneg(R.D);
    SE.Le = C3(0, 0, 0);
}

/* ScatterEventInVolume - Source/raymarching.h:73-113 */
ER_D bool scatter_event_in_volume(const Params& P, const Ray& R, Rng& rng)
{
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return false;
    float MinT = smax(Int.near_t, R.MinT);
    const float MaxT = smin(Int.far_t, R.MaxT);
    const float S = -er_logf(rng.get1()) / P.density_scale;
    float Sum = 0.0f;
    const float StepSize = P.step_shadow * P.min_step;
    MinT += rng.get1() * StepSize;
    long long budget = march_budget(MinT, MaxT, StepSize);
    while (Sum < S) {
        const v3 Ps = vadd(R.O, vscale(R.D, MinT));
        if (MinT > MaxT) return false;
        if (--budget < 0) { atomicOr(P.err, 1); return false; }
        Sum += sigma_point(P, Ps) * StepSize;
        MinT += StepSize;
    }
    return true;
}

/* IntersectLight / IntersectLights - Source/lights.h:59-113, without the
   emission: the nearest hit's (P, N, T, Wo) in RS, its LightIDs index in
   `slot` (ScatterEvent::LightID) and what its emission needs in `lh`;
   light_emission gives the Le IntersectLight computes, for the hits that are
   used (the environment sphere's texture is not evaluated for the rays whose
   volume event or chosen light wins).  Same operations, same nearest hit. */
struct LightHit {
    v2 UV;
    bool front;
};

ER_D void intersect_lights_geom(const Params& P, const Ray& R, Event& RS, bool respect_visibility, int& slot, LightHit& lh)
{
    float T = FLT_MAX;
    for (int i = 0; i < P.light_count; i++) {
        if (!P.light_valid[i]) continue;
        const Light& L = P.lights[i];
        if (respect_visibility && !L.visible) continue;
        const Ray Rt = xform_ray(L.inv_tm, R);
        Isect Int; Int.invalid();
        intersect_shape(L, Rt, Int);
        if (!Int.valid) continue;
        Event local;
        local.type = 1;
        local.valid = true;
        local.P = xform_point(L.tm, Int.P);
        local.N = xform_vector(L.tm, Int.N);
        local.T = vlen(vsub(local.P, R.O));
        local.Wo = vneg(R.D);
        local.Le = C3(0, 0, 0);
        if (local.T < T) { RS = local; T = local.T; slot = i; lh.UV = Int.UV; lh.front = Int.front; }
    }
}

/* the emission of a light hit (Source/lights.h:78-84) */
ER_D c3 light_emission(const Params& P, const Light& L, const LightHit& lh)
{
    c3 Le = lh.front ? cscale(light_texture(P, L, lh.UV), L.multiplier) : C3(0, 0, 0);
    if (L.unit == 1) Le = cdivs(Le, L.area);
    return Le;
}

/* IntersectsLight - Source/lights.h:115-131 */
ER_D bool intersects_light(const Params& P, const Ray& R)
{
    for (int i = 0; i < P.light_count; i++) {
        if (!P.light_valid[i]) continue;
        const Light& L = P.lights[i];
        if (L.inner_r2 > 0.0f) {
            /* a sphere (rigid transform) whose inner ball holds both ends of the
               segment: the segment stays inside, 0.1 radius from the surface,
               so the exact test below cannot find a root in [MinT, MaxT] */
            const v3 c = vload(L.inner_c);
            const v3 a = vsub(vadd(R.O, vscale(R.D, R.MinT)), c);
            const v3 b = vsub(vadd(R.O, vscale(R.D, R.MaxT)), c);
            if (vlen2(a) < L.inner_r2 && vlen2(b) < L.inner_r2) continue;
        }
        const Ray Rt = xform_ray(L.inv_tm, R);
        Isect Int; Int.invalid();
        intersect_shape(L, Rt, Int);
        if (Int.valid) return true;
    }
    return false;
}

/* IntersectObject / IntersectObjects - Source/objects.h:26-62: the nearest of
   the tracer's objects (array order, ObjectID = index) */
ER_D void intersect_objects(const Params& P, const Ray& R, Event& RS, ObjHit& hit)
{
    float T = FLT_MAX;
    for (int i = 0; i < P.object_count; i++) {
        const Object& O = P.objects[i];
        const Ray Rt = xform_ray(O.shape.inv_tm, R);
        Isect Int; Int.invalid();
        intersect_shape(O.shape, Rt, Int);
        if (!Int.valid) continue;
        Event local;
        local.type = 2;
        local.valid = true;
        local.N = xform_vector(O.shape.tm, Int.N);
        local.P = xform_point(O.shape.tm, Int.P);
        local.T = vlen(vsub(local.P, R.O));
        local.Wo = vneg(R.D);
        local.Le = C3(0, 0, 0);
        if (local.T < T) { RS = local; T = local.T; hit.UV = Int.UV; hit.id = i; }
    }
}

/* IntersectsObject - Source/objects.h:64-80 */
ER_D bool intersects_object(const Params& P, const Ray& R)
{
    for (int i = 0; i < P.object_count; i++) {
        const Object& O = P.objects[i];
        const Ray Rt = xform_ray(O.shape.inv_tm, R);
        Isect Int; Int.invalid();
        intersect_shape(O.shape, Rt, Int);
        if (Int.valid) return true;
    }
    return false;
}

/* ---- extension estimators (delta tracking, shader selection, full MIS) ---- */

/* 3D DDA over the majorant bricks in local voxel units.  The state is kept
   in scalars (no arrays indexed by the stepping axis), so it stays in
   registers; the arithmetic is the oracle's, operation for operation. */
struct Dda {
    float t, tmax;
    int bx, by, bz;
    int sx, sy, sz;
    float nx, ny, nz;        /* t of the next brick face per axis */
    float dx, dy, dz;        /* t between faces per axis */
    bool done;
};

ER_D void dda_axis(float o, float dirc, float minp, float inv_size, int res, int nb, float B, float t0, int& b, int& step,
                   float& tnext, float& tdelta)
{
    const float sc = inv_size * (float)res;
    const float lo = (o - minp) * sc;
    const float ld = dirc * sc;
    const float L = lo + t0 * ld;
    b = (int)floorf(L / B);
    b = b < 0 ? 0 : (b >= nb ? nb - 1 : b);
    if (ld > 0.0f) { step = 1; tnext = ((float)(b + 1) * B - lo) / ld; tdelta = B / ld; }
    else if (ld < 0.0f) { step = -1; tnext = ((float)b * B - lo) / ld; tdelta = -B / ld; }
    else { step = 0; tnext = FLT_MAX; tdelta = FLT_MAX; }
}

ER_D void dda_init(const Params& P, const Ray& R, float t0, float t1, Dda& d)
{
    const float B = (float)P.brick;
    d.t = t0;
    d.tmax = t1;
    d.done = false;
    dda_axis(R.O.x, R.D.x, P.minp[0], P.inv_size[0], P.res[0], P.nb[0], B, t0, d.bx, d.sx, d.nx, d.dx);
    dda_axis(R.O.y, R.D.y, P.minp[1], P.inv_size[1], P.res[1], P.nb[1], B, t0, d.by, d.sy, d.ny, d.dy);
    dda_axis(R.O.z, R.D.z, P.minp[2], P.inv_size[2], P.res[2], P.nb[2], B, t0, d.bz, d.sz, d.nz, d.dz);
}

ER_D float dda_exit(const Dda& d)
{
    float e = d.nx;
    if (d.ny < e) e = d.ny;
    if (d.nz < e) e = d.nz;
    if (d.tmax < e) e = d.tmax;
    return e < d.t ? d.t : e;
}

ER_D void dda_advance(const Params& P, Dda& d, float e)
{
    if (e >= d.tmax) { d.done = true; d.t = e; return; }
    /* axis with the nearest face; ties go to x, then y */
    const bool ax = !(d.ny < d.nx) && !(d.nz < d.nx);
    const bool ay = !ax && !(d.nz < d.ny);
    if (ax) {
        d.bx += d.sx;
        if (d.bx < 0 || d.bx >= P.nb[0]) d.done = true;
        d.nx += d.dx;
    } else if (ay) {
        d.by += d.sy;
        if (d.by < 0 || d.by >= P.nb[1]) d.done = true;
        d.ny += d.dy;
    } else {
        d.bz += d.sz;
        if (d.bz < 0 || d.bz >= P.nb[2]) d.done = true;
        d.nz += d.dz;
    }
    d.t = e;
}

ER_D float dda_majorant(const Params& P, const Dda& d)
{
    return __ldg(P.majorant + ((size_t)d.bz * (size_t)P.nb[1] + (size_t)d.by) * (size_t)P.nb[0] + (size_t)d.bx);
}

#define ER_DELTA_MAX_COLLISIONS 1048576

/* Empty-space jump.  An empty brick of the tracker's majorant grid holds
   -k, k the Chebyshev distance in bricks to the nearest non-empty brick
   (er_volume.cu k_skip_pass), so the cube of bricks within k-1 of it is
   empty: nothing is drawn and tau is unchanged while the ray crosses it.
   dda_jump moves the DDA to the cube's exit in one step.  The exit face of
   each axis is k-1 bricks past its next face (time next + (k-1) * delta);
   the earliest of the three (ties to x, then y, as dda_advance) is the exit
   time te, that axis moves k bricks, and each other axis moves past the m
   faces it crosses before te, m = floor((te - next) / delta) + 1 (at most
   k).  The oracle makes the same float operations (oracle/er_oracle.c
   dda_jump), so the face times after a jump are those of the oracle, not
   those of k-1 brick-by-brick advances (a sum of deltas rounds
   differently); the segment [t, te] lies in empty bricks either way. */
ER_D void dda_jump(const Params& P, Dda& d, int k)
{
    const float r = (float)(k - 1);
    const float fx = d.sx != 0 ? d.nx + r * d.dx : FLT_MAX;
    const float fy = d.sy != 0 ? d.ny + r * d.dy : FLT_MAX;
    const float fz = d.sz != 0 ? d.nz + r * d.dz : FLT_MAX;
    const bool ax = !(fy < fx) && !(fz < fx);
    const bool ay = !ax && !(fz < fy);
    const float te = ax ? fx : (ay ? fy : fz);
    if (te >= d.tmax) { d.done = true; d.t = te; return; }
    int m;
    if (ax) { d.bx += d.sx * k; d.nx = fx + d.dx; }
    else if (d.nx < te) {
        m = (int)((te - d.nx) / d.dx) + 1;
        m = m > k ? k : m;
        d.bx += d.sx * m;
        d.nx = d.nx + (float)m * d.dx;
    }
    if (ay) { d.by += d.sy * k; d.ny = fy + d.dy; }
    else if (d.ny < te) {
        m = (int)((te - d.ny) / d.dy) + 1;
        m = m > k ? k : m;
        d.by += d.sy * m;
        d.ny = d.ny + (float)m * d.dy;
    }
    if (!ax && !ay) { d.bz += d.sz * k; d.nz = fz + d.dz; }
    else if (d.nz < te) {
        m = (int)((te - d.nz) / d.dz) + 1;
        m = m > k ? k : m;
        d.bz += d.sz * m;
        d.nz = d.nz + (float)m * d.dz;
    }
    if (d.bx < 0 || d.bx >= P.nb[0] || d.by < 0 || d.by >= P.nb[1] || d.bz < 0 || d.bz >= P.nb[2]) d.done = true;
    d.t = te;
}

/* Delta tracking of the primary ray: sigma_t = DensityScale^2 * Opacity(I),
   the extinction the reference's march integrates (Source/raymarching.h:45,64-66) */
/* SKIP: compile the empty-space jump.  Every delta-tracking caller passes
   true (the tracker's grid carries skip distances, and the jump sets the
   face times the tracker continues from); false compiles the stages of the
   fixed-step march, which never run this tracker, with fewer registers. */
template <bool WITH_NORMAL = true, bool SKIP = true>
ER_D void sample_volume_delta(const Params& P, const Ray& R, Rng& rng, Event& SE, float u0 = -1.0f)
{
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return;
    Dda d;
    dda_init(P, R, t0, t1, d);
    const float ud = rng.get1();
    float tau = -er_logf(u0 >= 0.0f ? u0 : ud);
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(d);
        const float mu = dda_majorant(P, d);
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
                const v3 Pt = vadd(R.O, vscale(R.D, t));
                const float sig = P.density_scale * sigma_point_in_brick(P, Pt, d.bx, d.by, d.bz);
                if (rng.get1() * mu < sig) {
                    SE.valid = true;
                    SE.T = t;
                    SE.P = Pt;
                    SE.N = WITH_NORMAL ? normalized_gradient(P, Pt) : V3(0.0f, 0.0f, 0.0f);
                    SE.Wo = vneg(R.D);
                    SE.Le = C3(0, 0, 0);
                    return;
                }
                if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); return; }
                tau = -er_logf(rng.get1());
            }
        } else if (SKIP && mu <= -2.0f) {
            dda_jump(P, d, (int)(-mu));
            continue;
        }
        dda_advance(P, d, e);
    }
}

/* Delta tracking of the primary ray (sample_volume_delta) as a resumable
   state machine for the persistent primary stage: delta_begin sets the ray
   up, each delta_step makes one tentative collision or crosses one majorant
   brick; at the end `hit` says whether a real collision was found, at ray
   parameter t.  Same operations in the same order as sample_volume_delta. */
struct DeltaTracker {
    Dda d;
    float tau, t, e, mu;
    int guard;
    bool in_brick, done, hit;
};

ER_D void delta_begin(const Params& P, const Ray& R, Rng& rng, DeltaTracker& k, float u0 = -1.0f)
{
    k.done = true;
    k.hit = false;
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return;
    dda_init(P, R, t0, t1, k.d);
    const float ud = rng.get1();
    k.tau = -er_logf(u0 >= 0.0f ? u0 : ud);
    k.guard = 0;
    k.in_brick = false;
    k.done = false;
}

template <bool SKIP = true>
ER_D void delta_step(const Params& P, const Ray& R, Rng& rng, DeltaTracker& k)
{
    if (!k.in_brick) {
        k.e = dda_exit(k.d);
        k.mu = dda_majorant(P, k.d);
        k.t = k.d.t;
        k.in_brick = true;
    }
    if (k.mu > 0.0f) {
        const float dt = k.tau / k.mu;
        if (k.t + dt < k.e) {
            k.t = k.t + dt;
            const v3 Pt = vadd(R.O, vscale(R.D, k.t));
            const float sig = P.density_scale * sigma_point_in_brick(P, Pt, k.d.bx, k.d.by, k.d.bz);
            if (rng.get1() * k.mu < sig) { k.hit = true; k.done = true; return; }
            if (++k.guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); k.done = true; return; }
            k.tau = -er_logf(rng.get1());
            return;
        }
        k.tau = k.tau - k.mu * (k.e - k.t);
        if (k.tau < 0.0f) k.tau = 0.0f;
    } else if (SKIP && k.mu <= -2.0f) {
        dda_jump(P, k.d, (int)(-k.mu));
        k.in_brick = false;
        if (k.d.done) k.done = true;
        return;
    }
    dda_advance(P, k.d, k.e);
    k.in_brick = false;
    if (k.d.done) k.done = true;
}

/* Ratio tracking of a shadow segment with Russian roulette below 0.1, as a
   resumable state machine: ratio_begin sets the segment up, each ratio_step
   makes one collision or crosses one majorant brick.  The persistent shadow
   stage interleaves the steps of one lane's successive segments, so a lane
   whose segment ended takes the next one instead of idling until its warp's
   longest segment ends.  transmittance_ratio below is the same tracking as
   one loop: both make the same floating-point operations in the same order
   (the parity tests compare both paths with the oracle). */
struct RatioTracker {
    Dda d;
    float Tr, tau, t, e, mu;
    int guard;
    bool in_brick, done;
};

ER_D void ratio_begin(const Params& P, const Ray& R, Rng& rng, RatioTracker& k)
{
    k.Tr = 1.0f;
    k.done = true;
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return;
    dda_init(P, R, t0, t1, k.d);
    k.tau = -er_logf(rng.get1());
    k.guard = 0;
    k.in_brick = false;
    k.done = false;
}

template <bool SKIP = true>
ER_D void ratio_step(const Params& P, const Ray& R, Rng& rng, RatioTracker& k)
{
    if (!k.in_brick) {
        k.e = dda_exit(k.d);
        k.mu = dda_majorant(P, k.d);
        k.t = k.d.t;
        k.in_brick = true;
    }
    if (k.mu > 0.0f) {
        const float dt = k.tau / k.mu;
        if (k.t + dt < k.e) {
            k.t = k.t + dt;
            const v3 Pt = vadd(R.O, vscale(R.D, k.t));
            const float sig = P.density_scale * sigma_point_in_brick(P, Pt, k.d.bx, k.d.by, k.d.bz);
            k.Tr = k.Tr * (1.0f - sig / k.mu);
            if (k.Tr <= 0.0f) { k.Tr = 0.0f; k.done = true; return; }
            if (k.Tr < 0.1f) {
                if (rng.get1() >= 0.5f) { k.Tr = 0.0f; k.done = true; return; }
                k.Tr = k.Tr * 2.0f;
            }
            if (++k.guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); k.done = true; return; }
            k.tau = -er_logf(rng.get1());
            return;
        }
        k.tau = k.tau - k.mu * (k.e - k.t);
        if (k.tau < 0.0f) k.tau = 0.0f;
    } else if (SKIP && k.mu <= -2.0f) {
        dda_jump(P, k.d, (int)(-k.mu));
        k.in_brick = false;
        if (k.d.done) k.done = true;
        return;
    }
    dda_advance(P, k.d, k.e);
    k.in_brick = false;
    if (k.d.done) k.done = true;
}

/* the same tracking as one loop (the one-kernel paths and the non-persistent
   shadow stage, where it compiles to fewer registers) */
template <bool SKIP = true>
ER_D float transmittance_ratio(const Params& P, const Ray& R, Rng& rng)
{
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return 1.0f;
    const float t0 = smax(Int.near_t, R.MinT);
    const float t1 = smin(Int.far_t, R.MaxT);
    if (!(t0 < t1)) return 1.0f;
    Dda d;
    dda_init(P, R, t0, t1, d);
    float Tr = 1.0f;
    float tau = -er_logf(rng.get1());
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(d);
        const float mu = dda_majorant(P, d);
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
                const v3 Pt = vadd(R.O, vscale(R.D, t));
                const float sig = P.density_scale * sigma_point_in_brick(P, Pt, d.bx, d.by, d.bz);
                Tr = Tr * (1.0f - sig / mu);
                if (Tr <= 0.0f) return 0.0f;
                if (Tr < 0.1f) {
                    if (rng.get1() >= 0.5f) return 0.0f;
                    Tr = Tr * 2.0f;
                }
                if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); return Tr; }
                tau = -er_logf(rng.get1());
            }
        } else if (SKIP && mu <= -2.0f) {
            dda_jump(P, d, (int)(-mu));
            continue;
        }
        dda_advance(P, d, e);
    }
    return Tr;
}

/* Visible / Intersect - Source/transport.h:30-56: 1/0 for the reference
   march, the ratio-tracked transmittance with delta tracking */
/* the shadow ray of Visible (Source/transport.h:46-56) */
ER_D Ray shadow_ray(const Params& P, v3 P1, v3 P2)
{
    const v3 W = vnorm(vsub(P2, P1));
    Ray R;
    R.O = vadd(P1, vscale(W, ER_RAY_EPS));
    R.D = W;
    R.MinT = 0.0f;
    R.MaxT = smin(vlen(vsub(P2, P1)) - 2.0f * ER_RAY_EPS, P.max_shadow_distance);
    return R;
}

template <bool OBJ = true, bool SKIP = true>
ER_D float visibility(const Params& P, v3 P1, v3 P2, Rng& rng)
{
    if (!P.shadows) return 1.0f;
    const Ray R = shadow_ray(P, P1, P2);
    if (intersects_light(P, R)) return 0.0f;
    if (OBJ && P.object_count > 0 && intersects_object(P, R)) return 0.0f;
    if (P.free_flight == 1) return transmittance_ratio<SKIP>(P, R, rng);
    return scatter_event_in_volume(P, R, rng) ? 0.0f : 1.0f;
}

/* shader selection of the design Source/scatterevent.h:155-212 (0 BRDF, 1 phase) */
/* gm: the gradient magnitude at SE.P when the caller has it, else < 0 */
ER_D int select_shader_type(const Params& P, const Event& SE, float I, Rng& rng, float gm = -1.0f)
{
    switch (P.shading_type) {
    case 0: return 0;
    case 1: return 1;
    case 2: {
        const float NGM = (gm >= 0.0f ? gm : gradient_magnitude(P, SE.P)) * P.gm_inv_max;
        const float Exponent = 25.0f * pow_c(P.gradient_factor, 3.0f) * NGM;
        const float PdfBrdf = P.opacity_modulated ? opacity_at(P, I) * (1.0f - exp_c(-Exponent))
                                                  : 1.0f - exp_c(-Exponent);
        return rng.get1() <= PdfBrdf ? 0 : 1;
    }
    case 3: {
        const float NGM = (gm >= 0.0f ? gm : gradient_magnitude(P, SE.P)) * P.gm_inv_max;
        const float PdfBrdf = 1.0f - pow_c(1.0f - NGM, 2.0f);
        return rng.get1() < PdfBrdf ? 0 : 1;
    }
    case 4: {
        const float NGM = (gm >= 0.0f ? gm : gradient_magnitude(P, SE.P)) * P.gm_inv_max;
        return NGM > P.gradient_threshold ? 0 : 1;
    }
    default: return 1;
    }
}

#define ER_INV_FOUR_PI_TRUE 0.0795774715f

/* SampleLight - Source/lights.h:44-57 */
ER_D void sample_light(const Params& P, const Light& L, v3 uvw, Surf& SS, const Event& SE, v3& Wi, c3& Le)
{
    sample_light_surface(L, uvw, SS);
    Wi = vnorm(vsub(SS.P, SE.P));
    Le = cscale(light_texture(P, L, SS.UV), L.multiplier);
    if (L.one_sided && vdot(vsub(SE.P, SS.P), SS.N) < 0.0f) Le = C3(0, 0, 0);
    if (L.unit == 1) Le = cdivs(Le, L.area);
}

struct Metro {               /* MetroSample::LargeStep - Source/sample.h:258-262 */
    float brdf_component;
    v2 brdf_dir;
    v3 light_uvw;
    float light_num;
    v2 film_uv;
    v2 lens_uv;
    ER_D void large_step(Rng& r)
    {
        brdf_component = r.get1();
        brdf_dir = r.get2();
        light_uvw = r.get3();
        light_num = r.get1();
        film_uv = r.get2();
        lens_uv = r.get2();
    }
    float tau_u;             /* the stratified first free-flight draw, or < 0 */
    /* settings.stratify: the light sample, the BSDF sample and the first
       free-flight draw of sample `index` of a pixel from the per-pixel
       shifted lattices of er_stratified_sample (after large_step, whose
       draws keep the random stream unchanged) */
    ER_D void stratify(const Params& P, uint32_t view, uint32_t pixel, uint32_t index)
    {
        tau_u = -1.0f;
        if (!P.stratify) return;
        float u[7];
        er_stratified_sample(P.seed, view, pixel, index, u);
        light_uvw.x = u[0];
        light_uvw.y = u[1];
        light_num = u[2];
        brdf_dir.x = u[3];
        brdf_dir.y = u[4];
        brdf_component = u[5];
        tau_u = u[6];
    }
};

/* mixture pdf of the full-MIS BSDF sampler (Lambertian and Blinn lobes with
   probability 1/2 each, Source/shader.h:364-371; uniform sphere for the phase
   function, :293-299) */
ER_D float mis_bsdf_pdf(const Shader& sh, v3 Wo, v3 Wi)
{
    if (sh.type == 0) {
        const v3 Wol = world_to_local(sh, Wo), Wil = world_to_local(sh, Wi);
        const float pl = same_hemisphere(Wol, Wil) ? fabsf(Wil.z) * ER_INV_PI_F : 0.0f;
        const float pm = same_hemisphere(Wol, Wil) ? blinn_pdf(sh.exponent, Wol, Wil) : 0.0f;
        return 0.5f * (pl + pm);
    }
    return ER_INV_FOUR_PI_TRUE;
}

/* Lambertian::SampleF / Blinn::SampleF / IsotropicPhase::SampleF
   (Source/shader.h:46-56, :142-164, :293-299) */
ER_COLD v3 sample_bsdf_dir(const Shader& sh, v3 Wo, const Metro& ms)
{
    if (sh.type == 0) {
        const v3 Wol = world_to_local(sh, Wo);
        v3 Wil;
        if (ms.brdf_component <= 0.5f) {
            const v2 d = concentric_sample_disk(ms.brdf_dir);
            Wil = V3(d.x, d.y, sqrtf(smax(0.f, 1.f - d.x * d.x - d.y * d.y)));
            if (Wol.z < 0.0f) Wil.z *= -1.0f;
        } else {
            const float e = sh.exponent;
            const float costheta = pow_c(ms.brdf_dir.x, 1.f / (e + 1));
            const float sintheta = sqrtf(smax(0.f, 1.f - costheta * costheta));
            const float phi = ms.brdf_dir.y * 2.f * ER_PI_F;
            const v2 scv = sincos_c(phi);
            const float sn = scv.x, cs = scv.y;
            v3 wh = V3(sintheta * cs, sintheta * sn, costheta);
            if (!same_hemisphere(Wol, wh)) wh = vneg(wh);
            Wil = vadd(vneg(Wol), vscale(wh, 2.f * vdot(Wol, wh)));
        }
        return local_to_world(sh, Wil);
    }
    const float z = 1.f - 2.f * ms.brdf_dir.x;
    const float r = sqrtf(smax(0.f, 1.f - z * z));
    const float phi = 2.f * ER_PI_F * ms.brdf_dir.y;
    const v2 scv = sincos_c(phi);
    const float sn = scv.x, cs = scv.y;
    return V3(r * cs, r * sn, z);
}

/* EstimateDirectLight - Source/transport.h:58-113: the live light-sampling
   half (mis 0, march), or both halves with power-heuristic weights (mis 1),
   with the ratio-tracked transmittance under delta tracking */
ER_D c3 estimate_direct_light(const Params& P, const Light& L, int slot, const Metro& ms, const Event& SE, Rng& rng,
                              const Shader& sh)
{
    v3 Wi;
    c3 Li, Ld = C3(0, 0, 0);
    Surf SS;
    sample_light(P, L, ms.light_uvw, SS, SE, Wi, Li);
    const c3 F = shader_f(sh, SE.Wo, Wi);
    const bool full = P.mis == 1;
    const bool delta = P.free_flight == 1;
    const float BsdfPdf = full ? mis_bsdf_pdf(sh, SE.Wo, Wi) : shader_pdf(sh, SE.Wo, Wi);
    if (!full && !delta) {
        if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f && visibility(P, SE.P, SS.P, rng) > 0.0f) {
            const float LightPdf = vlen2(vsub(SE.P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L.area);
            const float Weight = power_heuristic(LightPdf, BsdfPdf);
            if (sh.type == 0) Ld = cadd(Ld, cscale(cmul(F, Li), vabsdot(Wi, SE.N) * Weight / LightPdf));
            else Ld = cadd(Ld, cdivs(cmul(F, Li), LightPdf));
        }
        return Ld;
    }
    if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f) {
        const float Tr = visibility(P, SE.P, SS.P, rng);
        if (Tr > 0.0f) {
            const float LightPdf = vlen2(vsub(SE.P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L.area);
            c3 c;
            if (full) {
                const float w = power_heuristic(LightPdf, BsdfPdf);
                c = cscale(cmul(F, Li), sh.type == 0 ? vabsdot(Wi, SE.N) * w / LightPdf : w / LightPdf);
            } else if (sh.type == 0) {
                c = cscale(cmul(F, Li), vabsdot(Wi, SE.N) * power_heuristic(LightPdf, BsdfPdf) / LightPdf);
            } else {
                c = cdivs(cmul(F, Li), LightPdf);
            }
            Ld = cadd(Ld, cscale(c, Tr));
        }
    }
    if (!full) return Ld;
    const v3 Wb = sample_bsdf_dir(sh, SE.Wo, ms);
    const c3 Fb = shader_f(sh, SE.Wo, Wb);
    const float pb = mis_bsdf_pdf(sh, SE.Wo, Wb);
    if (cblack(Fb) || !(pb > 0.0f)) return Ld;
    Ray R2;
    R2.O = SE.P;
    R2.D = Wb;
    R2.MinT = 0.0f;
    R2.MaxT = 1000000.0f;
    Event SE2;
    SE2.type = 1; SE2.valid = false; SE2.T = 0.0f; SE2.Le = C3(0, 0, 0);
    SE2.P = V3(0, 0, 0); SE2.N = V3(0, 0, 0); SE2.Wo = V3(0, 0, 0);
    int hit = -1;
    LightHit lh;
    intersect_lights_geom(P, R2, SE2, false, hit, lh);
    if (!SE2.valid || P.light_ids[hit] != P.light_ids[slot]) return Ld;
    SE2.Le = light_emission(P, P.lights[hit], lh);
    if (cblack(SE2.Le)) return Ld;
    const float Tr = visibility(P, SE.P, SE2.P, rng);
    if (Tr > 0.0f) {
        const float LightPdf = vlen2(vsub(SE.P, SE2.P)) / (vabsdot(SE2.N, vneg(Wb)) * L.area);
        const float w = power_heuristic(pb, LightPdf);
        const c3 c = cscale(cmul(Fb, SE2.Le), sh.type == 0 ? vabsdot(Wb, SE.N) * w / pb : w / pb);
        Ld = cadd(Ld, cscale(c, Tr));
    }
    return Ld;
}

/* the object shader of UniformSampleOneLight (Source/transport.h:141-149):
   BRDF with the object's diffuse and specular textures at the hit, IOR 15 and
   the exponent of the glossiness texture's luminance (ColorXYZf::Y) */
ER_D void object_shader(const Params& P, const Event& SE, const ObjHit& hit, Shader& sh)
{
    const Object& O = P.objects[hit.id];
    const c3 Kd = evaluate_texture(P, O.diffuse_texture_id, hit.UV);
    const c3 Ks = evaluate_texture(P, O.specular_texture_id, hit.UV);
    const c3 G = evaluate_texture(P, O.glossiness_texture_id, hit.UV);
    float Y = 0.0f;
    Y += 0.212671f * G.r;
    Y += 0.715160f * G.g;
    Y += 0.072169f * G.b;
    shader_init(sh, 0, SE.N, SE.Wo, Kd, Ks, 15.0f, 1000000.0f * pow_c(Y, 7.0f));
}

/* UniformSampleOneLight - Source/transport.h:115-156 (volume and object events) */
ER_D c3 uniform_sample_one_light(const Params& P, const Event& SE, Rng& rng, const Metro& ms, const ObjHit& hit)
{
    c3 Ld = C3(0, 0, 0);
    const float I = get_intensity(P, SE.P);
    ShadeTF tf;
    shade_tf(P, I, tf);
    Ld = cadd(Ld, tf.Le);
    if (P.light_count <= 0) return Ld;
    const int idx = (int)floorf(ms.light_num * (float)P.light_count);
    if (idx < 0 || idx >= P.light_count || !P.light_valid[idx]) return Ld;
    const Light& L = P.lights[idx];
    Shader sh;
    if (SE.type == 2) {
        object_shader(P, SE, hit, sh);
    } else {
        const int type = P.apply_shading_type ? select_shader_type(P, SE, I, rng) : 0;
        shader_init(sh, type, SE.N, SE.Wo, tf.Kd, tf.Ks, P.volume_ior, tf.exponent);
    }
    Ld = cadd(Ld, estimate_direct_light(P, L, idx, ms, SE, rng, sh));
    return cscale(Ld, (float)P.light_count);
}

/* SampleCamera - Source/singlescattering.h:29-50 */
ER_D Ray sample_camera(const Params& P, int u, int v, v2 film_uv, v2 lens_uv)
{
    Ray R;
    const float sp0 = P.screen00 + (P.inv_screen0 * ((float)u + film_uv.x * 1.0f / (float)P.film[0]));
    const float sp1 = P.screen10 + (P.inv_screen1 * ((float)v + film_uv.y * 1.0f / (float)P.film[1]));
    R.O = vload(P.pos);
    R.D = vnorm(vsub(vadd(vload(P.N), vscale(vload(P.U), sp0)), vscale(vload(P.V), sp1)));
    R.MinT = P.clip_near;
    R.MaxT = P.clip_far;
    if (P.aperture != 0.0f) {
        const v2 d = concentric_sample_disk(lens_uv);
        const float lx = d.x * P.aperture, ly = d.y * P.aperture;
        const v3 LI = vadd(vscale(vload(P.U), lx), vscale(vload(P.V), ly));
        R.O = vadd(R.O, LI);
        R.D = vnorm(vsub(vscale(R.D, P.focal_distance), LI));
    }
    return R;
}

/* SingleScattering - Source/singlescattering.h:76-102.  `sample` >= 0 marks
   sample `sample` of view `view` of a multi-sample render (stratified light
   samples when enabled); -1 a frame of the reference's pipeline. */
ER_D float4 single_scattering(const Params& P, int x, int y, Rng& rng, uint32_t view = 0, int64_t sample = -1)
{
    c3 Lv = C3(0, 0, 0);
    Metro ms;
    ms.large_step(rng);
    ms.tau_u = -1.0f;
    if (sample >= 0) ms.stratify(P, view, (uint32_t)y * (uint32_t)P.film[0] + (uint32_t)x, (uint32_t)sample);
    const Ray R = sample_camera(P, x, y, ms.film_uv, ms.lens_uv);
    Event se0, se1, se2, SE;
    se0.type = 0; se0.valid = false; se0.T = 0.0f; se0.Le = C3(0, 0, 0);
    se0.P = V3(0, 0, 0); se0.N = V3(0, 0, 0); se0.Wo = V3(0, 0, 0);
    se1 = se0; se1.type = 1;
    se2.type = 2; se2.valid = false; se2.T = 0.0f;
    ObjHit hit;
    hit.UV.x = 0.0f; hit.UV.y = 0.0f; hit.id = 0;
    if (P.free_flight == 1) sample_volume_delta(P, R, rng, se0, ms.tau_u);
    else sample_volume(P, R, rng, se0);
    int lslot = -1;
    LightHit lh;
    intersect_lights_geom(P, R, se1, true, lslot, lh);
    if (P.object_count > 0) intersect_objects(P, R, se2, hit);
    SE = se0; SE.valid = false; SE.type = 0;
    float T = FLT_MAX;
    if (se0.valid && se0.T < T) { SE = se0; T = se0.T; }
    if (se1.valid && se1.T < T) { SE = se1; T = se1.T; }
    if (se2.valid && se2.T < T) { SE = se2; T = se2.T; }
    if (SE.valid && SE.type == 1) SE.Le = light_emission(P, P.lights[lslot], lh);
    if (SE.valid && SE.type == 0) Lv = cadd(Lv, uniform_sample_one_light(P, SE, rng, ms, hit));
    if (SE.valid && SE.type == 1) Lv = cadd(Lv, SE.Le);
    if (SE.valid && SE.type == 2) Lv = cadd(Lv, uniform_sample_one_light(P, SE, rng, ms, hit));
    return make_float4(Lv.r, Lv.g, Lv.b, SE.valid ? 1.0f : 0.0f);
}

}  // namespace erd

#endif
