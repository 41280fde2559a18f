/*
 * er_wavefront.cu - the single-scattering estimator as a pipeline of small
 * kernels over a batch of views (compiled with --fmad=false).
 *
 * The one-kernel path (k_trace_sum) inlines camera sampling, free flight,
 * shading, light sampling, MIS and two shadow traversals into one kernel of
 * 255 registers whose code does not fit the instruction cache; under ncu it
 * runs 8 warps per SM with 11 of 32 lanes active.  Here each stage is its
 * own kernel with its own register and code footprint:
 *
 *   k_wf_primary : MetroSample, SampleCamera, free flight, IntersectLights
 *                  (Source/singlescattering.h:76-101).  Misses and light
 *                  hits finish here; volume events go to the event queue.
 *   k_wf_shade   : UniformSampleOneLight up to the shadow rays
 *                  (Source/transport.h:115-156, :58-113): event normal,
 *                  emission, light pick, shader selection, light sample,
 *                  BSDF sample and its light hit.  Unoccluded contributions
 *                  and the two shadow segments go to the shadow queue.
 *   k_wf_shadow  : the shadow segments (march or ratio tracking) and the
 *                  final sum of the sample.
 *   k_wf_reduce  : per-pixel sum over the window's samples in sample order.
 *
 * Batching: every view of a batch (its own tracer: camera, film, transfer
 * functions, lights, volume) has a record in a view table in HBM.  The
 * samples of all views form one index space (view by view, sample-major
 * inside a view: item = s * npix + pixel), cut on the host into windows of
 * whole sample rows; each window is one pass of the four stages over items
 * of many views, so uneven views load-balance inside each launch.  The
 * reduction keeps each pixel's samples in order, so a view's sum is the same
 * whether it is rendered alone or in a batch.
 *
 * Every RNG draw happens in the order of the one-kernel path (the RNG state
 * travels with the queue records) and every float operation is the same, so
 * the sums are bit-identical to k_trace_sum's and to the CPU oracle's.
 */
#include <cstring>
#include <mutex>

#include "er_kernels.h"
#include "er_path.cuh"

using namespace erd;

namespace {

ER_D float u2f(uint32_t u) { return __uint_as_float(u); }
ER_D uint32_t f2u(float f) { return __float_as_uint(f); }

/* warp-aggregated slot in a queue for the lanes with `want` set */
ER_D uint32_t queue_slot(bool want, uint32_t* counter)
{
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    uint32_t base = 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    if (mask && lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader < 0 ? 0 : leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

/* the view record: a kernel parameter for a one-view launch, else the table */
template <bool ONE>
ER_D const WfView& view_of(const WfView* __restrict__ views, const WfView& one, uint32_t v)
{
    if (ONE) return one;
    return views[v];
}

/* the pixel of slot j of a sample row: row by row, or (tile_order) in
   tiles of 32 pixels, row by row of tiles, so that a warp's 32 lanes trace a
   block of neighbouring pixels (tile_order 1: 8x4, 2: 4x8, 3: 16x2); a
   bijection of [0, W H), so the reduce stage maps the slots back */
ER_D uint32_t slot_pixel(const Params& P, uint32_t j)
{
    const int W = P.film[0], H = P.film[1];
    const int lw = P.tile_order == 1 ? 3 : (P.tile_order == 2 ? 2 : 4);     /* log2 of the tile width */
    const uint32_t tx = 1u << lw, ty = 32u >> lw;
    if (!P.tile_order || ((uint32_t)W & (tx - 1u)) || ((uint32_t)H & (ty - 1u))) return j;
    const uint32_t t = j >> 5, u = j & 31u;
    const uint32_t tw = (uint32_t)W >> lw;
    const uint32_t x = (t % tw) * tx + (u & (tx - 1u)), y = (t / tw) * ty + (u >> lw);
    return y * (uint32_t)W + x;
}

/* segment of a window holding window-local item i (segments are sorted by offset) */
ER_D int find_segment(const WfSegment* __restrict__ segs, int nseg, uint32_t i)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (segs[mid].offset <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace

/* top bit of an event record's view word: a surface-object event */
#define WF_OBJECT_EVENT 0x80000000u

/* ---- stage 1: camera ray, free flight, visible lights and objects ---- */

/* MINB: resident 256-thread blocks per SM the register allocation targets
   (2: 128 registers, 3: ~80, 4: 64, 6: 40, 8: 32); picked at run time */
/* OBJ: the variant that also intersects surface objects (scenes without
   objects run the lean one) */
template <int MINB, bool ONE, bool OBJ, bool SKIP>
__global__ void __launch_bounds__(256, MINB) k_wf_primary(const WfView* __restrict__ views, const WfSegment* __restrict__ segs, int nseg,
                                                           const WfView one, const WfSegment one_seg, uint32_t items,
                                                           float4* __restrict__ results, float4* __restrict__ events,
                                                           uint32_t* __restrict__ n_events)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < items; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < items;
        bool push = false;
        Event SE;
        ObjHit hit;
        Metro ms;
        Rng rng;
        rng.s0 = 0u;
        rng.s1 = 0u;
        int v = 0;
        if (live) {
            const WfSegment sg = ONE ? one_seg : segs[find_segment(segs, nseg, i)];
            v = sg.view;
            const WfView& V = view_of<ONE>(views, one, v);
            const Params& P = V.P;
            const uint32_t local = i - sg.offset;
            const uint32_t npix = (uint32_t)(P.film[0] * P.film[1]);
            const int s = sg.s0 + (int)(local / npix);
            const int pix = (int)slot_pixel(P, local % npix);
            const int x = pix % P.film[0], y = pix / P.film[0];
            er_seed_lanes(P.seed, V.view_id, (uint32_t)pix, V.first + (uint32_t)s, &rng.s0, &rng.s1);
            ms.large_step(rng);
            ms.stratify(P, V.view_id, (uint32_t)pix, V.first + (uint32_t)s);
            const Ray R = sample_camera(P, x, y, ms.film_uv, ms.lens_uv);
            Event se0, se1;
            se0.type = 0; se0.valid = false; se0.T = 0.0f; se0.Le = C3(0, 0, 0);
            se0.P = V3(0, 0, 0); se0.N = V3(0, 0, 0); se0.Wo = V3(0, 0, 0);
            se1 = se0; se1.type = 1;
            /* the event normal (no RNG) is computed by the shade stage */
            if (P.free_flight == 1) sample_volume_delta<false, SKIP>(P, R, rng, se0, ms.tau_u);
            else sample_volume<false>(P, R, rng, se0);
            int lslot = -1;
            LightHit lh;
            intersect_lights_geom(P, R, se1, true, lslot, lh);
            SE = se0; SE.valid = false; SE.type = 0;
            float T = FLT_MAX;
            if (se0.valid && se0.T < T) { SE = se0; T = se0.T; }
            if (se1.valid && se1.T < T) { SE = se1; T = se1.T; }
            if (OBJ && P.object_count > 0) {
                Event se2;
                se2.type = 2; se2.valid = false; se2.T = 0.0f;
                intersect_objects(P, R, se2, hit);
                if (se2.valid && se2.T < T) { SE = se2; T = se2.T; }
            }
            if (SE.valid && SE.type == 1) SE.Le = light_emission(P, P.lights[lslot], lh);
            if (!SE.valid) {
                results[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            } else if (SE.type == 1) {
                const c3 Lv = cadd(C3(0, 0, 0), SE.Le);
                results[i] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
            } else {
                push = true;
                /* an object event parks its surface parameters in the sample's
                   result slot, which the shade stage reads before it writes
                   the sample's value there */
                if (OBJ && SE.type == 2) results[i] = make_float4(hit.UV.x, hit.UV.y, u2f((uint32_t)hit.id), 0.0f);
            }
        }
        const uint32_t slot = queue_slot(push, n_events);
        if (push) {
            /* volume events: the normal is computed by the shade stage; object
               events carry theirs and set the top bit of the view word */
            const bool obj = OBJ && SE.type == 2;
            float4* e = events + (size_t)slot * 5;
            e[0] = make_float4(u2f(i), u2f(rng.s0), u2f(rng.s1), ms.light_num);
            e[1] = make_float4(SE.P.x, SE.P.y, SE.P.z, ms.brdf_component);
            e[2] = obj ? make_float4(SE.N.x, SE.N.y, SE.N.z, ms.brdf_dir.x) : make_float4(0.0f, 0.0f, 0.0f, ms.brdf_dir.x);
            e[3] = make_float4(SE.Wo.x, SE.Wo.y, SE.Wo.z, ms.brdf_dir.y);
            e[4] = make_float4(ms.light_uvw.x, ms.light_uvw.y, ms.light_uvw.z, u2f((uint32_t)v | (obj ? WF_OBJECT_EVENT : 0u)));
        }
    }
}

/* persistent stages: a warp stops tracking to refill when fewer than
   refill / 8 of the lanes that were tracking still are (a launch argument,
   WavefrontBuffers::refill_eighths, 2 by default; measured in er_runtime.cu
   refill_eighths) */

/* queue slot among the lanes that are here together (persistent stages,
   where lanes reach their queue pushes at different loop trips) */
ER_D uint32_t queue_slot_active(bool want, uint32_t* counter)
{
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, want);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (mask && lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(active, base, leader < 0 ? (__ffs(active) - 1) : leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

/* ---- stage 1, persistent lanes (delta tracking) ----

   The work of k_wf_primary with lanes tracking one tentative collision or
   majorant brick per inner loop trip: when most of a warp's tracking lanes
   have ended their rays, the warp finishes those samples and gives the
   lanes the next items of the window (consecutive ones, one atomic per
   warp), while the other lanes keep their rays.  The MetroSample values an event
   record carries are drawn again from the sample's seed when the sample
   finishes instead of being held through the tracking. */
template <int MINB, bool ONE, bool OBJ, bool SKIP>
__global__ void __launch_bounds__(256, MINB) k_wf_primary_pt(const WfView* __restrict__ views, const WfSegment* __restrict__ segs,
                                                              int nseg, const WfView one, const WfSegment one_seg, uint32_t items,
                                                              float4* __restrict__ results, float4* __restrict__ events,
                                                              uint32_t* __restrict__ n_events, uint32_t* __restrict__ fetch, int refill)
{
    const int lane = threadIdx.x & 31;
    uint32_t i = 0;
    bool tracking = false, exhausted = false;
    int seg = 0;
    Rng rng;
    rng.s0 = 0u;
    rng.s1 = 0u;
    Ray R;
    DeltaTracker k;
    k.done = true;
    k.hit = false;
    for (;;) {
        /* lanes without a sample take the next items of the window together
           (one atomic per warp), so a warp's new samples are neighbours */
        const unsigned needy = __ballot_sync(0xffffffffu, !tracking && !exhausted);
        if (needy) {
            const int leader = __ffs(needy) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(needy));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!tracking && !exhausted) {
                i = base + (uint32_t)__popc(needy & ((1u << lane) - 1u));
                exhausted = i >= items;
            }
        }
        if (!tracking && !exhausted) {
            seg = ONE ? 0 : find_segment(segs, nseg, i);
            const WfSegment sg = ONE ? one_seg : segs[seg];
            const WfView& V = view_of<ONE>(views, one, sg.view);
            const Params& P = V.P;
            const uint32_t local = i - sg.offset;
            const uint32_t npix = (uint32_t)(P.film[0] * P.film[1]);
            const int s = sg.s0 + (int)(local / npix);
            const int pix = (int)slot_pixel(P, local % npix);
            er_seed_lanes(P.seed, V.view_id, (uint32_t)pix, V.first + (uint32_t)s, &rng.s0, &rng.s1);
            Metro ms;
            ms.large_step(rng);
            ms.stratify(P, V.view_id, (uint32_t)pix, V.first + (uint32_t)s);
            R = sample_camera(P, pix % P.film[0], pix / P.film[0], ms.film_uv, ms.lens_uv);
            delta_begin(P, R, rng, k, ms.tau_u);
            tracking = true;
        }
        if (!__any_sync(0xffffffffu, tracking)) break;
        const WfSegment sg = ONE ? one_seg : segs[seg];
        const WfView& V = view_of<ONE>(views, one, sg.view);
        const Params& P = V.P;
        /* track until most of the lanes that were tracking have ended */
        const int n_work = __popc(__ballot_sync(0xffffffffu, tracking && !k.done));
        while (tracking && !k.done) {
            delta_step<SKIP>(P, R, rng, k);
            if (k.done || 8 * __popc(__activemask()) < refill * n_work) break;
        }
        if (!tracking || !k.done) continue;
        /* the sample's nearest event: volume, visible lights, objects */
        Event SE, se1;
        SE.type = 0; SE.valid = false; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
        SE.P = V3(0, 0, 0); SE.N = V3(0, 0, 0); SE.Wo = V3(0, 0, 0);
        se1 = SE; se1.type = 1;
        if (k.hit) {
            SE.valid = true;
            SE.T = k.t;
            SE.P = vadd(R.O, vscale(R.D, k.t));
            SE.N = V3(0.0f, 0.0f, 0.0f);
            SE.Wo = vneg(R.D);
        }
        const Event se0 = SE;
        int lslot = -1;
        LightHit lh;
        intersect_lights_geom(P, R, se1, true, lslot, lh);
        SE.valid = false; SE.type = 0;
        float T = FLT_MAX;
        if (se0.valid && se0.T < T) { SE = se0; T = se0.T; }
        if (se1.valid && se1.T < T) { SE = se1; T = se1.T; }
        ObjHit hit;
        if (OBJ && P.object_count > 0) {
            Event se2;
            se2.type = 2; se2.valid = false; se2.T = 0.0f;
            intersect_objects(P, R, se2, hit);
            if (se2.valid && se2.T < T) { SE = se2; T = se2.T; }
        }
        if (SE.valid && SE.type == 1) SE.Le = light_emission(P, P.lights[lslot], lh);
        bool push = false;
        if (!SE.valid) {
            results[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else if (SE.type == 1) {
            const c3 Lv = cadd(C3(0, 0, 0), SE.Le);
            results[i] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
        } else {
            push = true;
            if (OBJ && SE.type == 2) results[i] = make_float4(hit.UV.x, hit.UV.y, u2f((uint32_t)hit.id), 0.0f);
        }
        const uint32_t slot = queue_slot_active(push, n_events);
        if (push) {
            const uint32_t local = i - sg.offset;
            const uint32_t npix = (uint32_t)(P.film[0] * P.film[1]);
            Rng r0;
            const uint32_t sidx = V.first + (uint32_t)(sg.s0 + (int)(local / npix));
            er_seed_lanes(P.seed, V.view_id, slot_pixel(P, local % npix), sidx, &r0.s0, &r0.s1);
            Metro ms;
            ms.large_step(r0);
            ms.stratify(P, V.view_id, slot_pixel(P, local % npix), sidx);
            const bool obj = OBJ && SE.type == 2;
            float4* e = events + (size_t)slot * 5;
            e[0] = make_float4(u2f(i), u2f(rng.s0), u2f(rng.s1), ms.light_num);
            e[1] = make_float4(SE.P.x, SE.P.y, SE.P.z, ms.brdf_component);
            e[2] = obj ? make_float4(SE.N.x, SE.N.y, SE.N.z, ms.brdf_dir.x) : make_float4(0.0f, 0.0f, 0.0f, ms.brdf_dir.x);
            e[3] = make_float4(SE.Wo.x, SE.Wo.y, SE.Wo.z, ms.brdf_dir.y);
            e[4] = make_float4(ms.light_uvw.x, ms.light_uvw.y, ms.light_uvw.z, u2f((uint32_t)sg.view | (obj ? WF_OBJECT_EVENT : 0u)));
        }
        tracking = false;
    }
}

/* ---- stage 2: shading up to the shadow segments ---- */

/* flags of a shadow job */
#define WF_RAY1 1u
#define WF_RAY2 2u

/* MINB: resident 128-thread blocks per SM (2: 255 registers, 3: 168, 4: 128, 6: 80) */
template <bool ONE, int MINB, bool OBJ>
__global__ void __launch_bounds__(128, MINB) k_wf_shade(const WfView* __restrict__ views, const WfView one, const float4* __restrict__ events,
                                                  const uint32_t* __restrict__ n_events, float4* __restrict__ results,
                                                  float4* __restrict__ jobs, uint32_t* __restrict__ n_jobs)
{
    const uint32_t n = *n_events;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t e_i = base + threadIdx.x;
        const bool live = e_i < n;
        bool push = false;
        uint32_t sample = 0, flags = 0, v = 0;
        Rng rng;
        rng.s0 = 0u;
        rng.s1 = 0u;
        Event SE;
        c3 Le = C3(0, 0, 0), c1 = C3(0, 0, 0), c2 = C3(0, 0, 0);
        v3 S1 = V3(0, 0, 0), S2 = V3(0, 0, 0);
        float count = 0.0f;
        if (live) {
            const float4* e = events + (size_t)e_i * 5;
            const float4 e0 = e[0], e1 = e[1], e2 = e[2], e3 = e[3], e4 = e[4];
            sample = f2u(e0.x);
            rng.s0 = f2u(e0.y);
            rng.s1 = f2u(e0.z);
            const uint32_t vw = f2u(e4.w);
            v = OBJ ? (vw & ~WF_OBJECT_EVENT) : vw;
            const bool obj = OBJ && (vw & WF_OBJECT_EVENT) != 0u;
            const Params& P = view_of<ONE>(views, one, v).P;
            Metro ms;
            ms.light_num = e0.w;
            ms.brdf_component = e1.w;
            ms.brdf_dir.x = e2.w;
            ms.brdf_dir.y = e3.w;
            ms.light_uvw = V3(e4.x, e4.y, e4.z);
            SE.type = 0; SE.valid = true; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
            SE.P = V3(e1.x, e1.y, e1.z);
            /* NormalizedGradient of SampleVolume (Source/raymarching.h:70); with
               central differences its six intensities also give the gradient
               magnitude of the shader switch */
            float gm = -1.0f;
            ObjHit hit;
            if (obj) {
                const float4 o = results[sample];
                SE.type = 2;
                hit.UV.x = o.x;
                hit.UV.y = o.y;
                hit.id = (int)f2u(o.z);
                SE.N = V3(e2.x, e2.y, e2.z);
            } else if (P.gradient_mode == 1) {
                Grad6 g6;
                gradient_samples(P, SE.P, g6);
                SE.N = vnorm(gradient_cd6(g6));
                if (P.apply_shading_type && P.shading_type >= 2 && P.shading_type <= 4) gm = gradient_magnitude6(P, g6);
            } else {
                SE.N = normalized_gradient(P, SE.P);
            }
            SE.Wo = V3(e3.x, e3.y, e3.z);
            /* UniformSampleOneLight - Source/transport.h:115-156 */
            const float I = get_intensity(P, SE.P);
            ShadeTF tf;
            shade_tf(P, I, tf);
            Le = cadd(C3(0, 0, 0), tf.Le);
            bool early = P.light_count <= 0;
            int idx = 0;
            if (!early) {
                idx = (int)floorf(ms.light_num * (float)P.light_count);
                early = idx < 0 || idx >= P.light_count || !P.light_valid[idx];
            }
            if (early) {
                const c3 Lv = cadd(C3(0, 0, 0), Le);
                results[sample] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
            } else {
                const Light& L = P.lights[idx];
                Shader sh;
                if (obj) {
                    object_shader(P, SE, hit, sh);
                } else {
                    const int type = P.apply_shading_type ? select_shader_type(P, SE, I, rng, gm) : 0;
                    shader_init(sh, type, SE.N, SE.Wo, tf.Kd, tf.Ks, P.volume_ior, tf.exponent);
                }
                count = (float)P.light_count;
                /* EstimateDirectLight - Source/transport.h:58-113, without the visibility terms */
                v3 Wi;
                c3 Li;
                Surf SS;
                sample_light(P, L, ms.light_uvw, SS, SE, Wi, Li);
                const c3 F = shader_f(sh, SE.Wo, Wi);
                const bool full = P.mis == 1;
                const float BsdfPdf = full ? mis_bsdf_pdf(sh, SE.Wo, Wi) : shader_pdf(sh, SE.Wo, Wi);
                if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f) {
                    const float LightPdf = vlen2(vsub(SE.P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L.area);
                    if (full) {
                        const float w = power_heuristic(LightPdf, BsdfPdf);
                        c1 = cscale(cmul(F, Li), sh.type == 0 ? vabsdot(Wi, SE.N) * w / LightPdf : w / LightPdf);
                    } else if (sh.type == 0) {
                        c1 = cscale(cmul(F, Li), vabsdot(Wi, SE.N) * power_heuristic(LightPdf, BsdfPdf) / LightPdf);
                    } else {
                        c1 = cdivs(cmul(F, Li), LightPdf);
                    }
                    S1 = SS.P;
                    flags |= WF_RAY1;
                }
                if (full) {
                    const v3 Wb = sample_bsdf_dir(sh, SE.Wo, ms);
                    const c3 Fb = shader_f(sh, SE.Wo, Wb);
                    const float pb = mis_bsdf_pdf(sh, SE.Wo, Wb);
                    if (!cblack(Fb) && pb > 0.0f) {
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
                        if (SE2.valid && P.light_ids[hit] == P.light_ids[idx]) SE2.Le = light_emission(P, P.lights[hit], lh);
                        if (SE2.valid && P.light_ids[hit] == P.light_ids[idx] && !cblack(SE2.Le)) {
                            const float LightPdf = vlen2(vsub(SE.P, SE2.P)) / (vabsdot(SE2.N, vneg(Wb)) * L.area);
                            const float w = power_heuristic(pb, LightPdf);
                            c2 = cscale(cmul(Fb, SE2.Le), sh.type == 0 ? vabsdot(Wb, SE.N) * w / pb : w / pb);
                            S2 = SE2.P;
                            flags |= WF_RAY2;
                        }
                    }
                }
                if (flags == 0) {
                    const c3 Lv = cadd(C3(0, 0, 0), cscale(cadd(Le, C3(0, 0, 0)), count));
                    results[sample] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
                } else {
                    push = true;
                }
            }
        }
        const uint32_t slot = queue_slot(push, n_jobs);
        if (push) {
            float4* j = jobs + (size_t)slot * 6;
            j[0] = make_float4(u2f(sample), u2f(rng.s0), u2f(rng.s1), u2f(flags));
            j[1] = make_float4(SE.P.x, SE.P.y, SE.P.z, count);
            j[2] = make_float4(S1.x, S1.y, S1.z, Le.r);
            j[3] = make_float4(c1.r, c1.g, c1.b, Le.g);
            j[4] = make_float4(S2.x, S2.y, S2.z, Le.b);
            j[5] = make_float4(c2.r, c2.g, c2.b, u2f(v));
        }
    }
}

/* ---- stage 2 sorted by shader: classification, then shading ---- */

/* When a launch's shader switch mixes BRDF and phase events (hybrid,
   modulation and threshold shading), the shade stage runs as two kernels:
   k_wf_classify does the part every event shares (normal and gradient
   magnitude from the six central-difference lookups, intensity, transfer
   functions, light choice, the shader switch with its random draw) and
   appends a shading record to the queue of its shader - BRDF records from
   the front of the record buffer, phase records from its back - and
   k_wf_shade_sorted shades the records in that order, so a warp evaluates
   one shader instead of both.  The operations and random draws are those of
   k_wf_shade, in the same order: the sums are bit-identical.

   record (5 float4): (sample, rng.s0, rng.s1, view), (P, I | light << 16 |
   shader << 28), (N, brdf_component), (Wo, brdf_dir.x), (light_uvw,
   brdf_dir.y); I is an integer intensity (< 2^16), light < 2^12 */
template <bool ONE>
__global__ void __launch_bounds__(128, 6) k_wf_classify(const WfView* __restrict__ views, const WfView one, const float4* __restrict__ events,
                                                        const uint32_t* __restrict__ n_events, float4* __restrict__ results,
                                                        float4* __restrict__ records, uint32_t cap, uint32_t* __restrict__ n_records)
{
    const uint32_t n = *n_events;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t e_i = base + threadIdx.x;
        bool push = false;
        int type = 0, idx = 0;
        uint32_t sample = 0, v = 0;
        float I = 0.0f;
        Rng rng;
        rng.s0 = 0u;
        rng.s1 = 0u;
        Event SE;
        Metro ms;
        if (e_i < n) {
            const float4* e = events + (size_t)e_i * 5;
            const float4 e0 = e[0], e1 = e[1], e2 = e[2], e3 = e[3], e4 = e[4];
            sample = f2u(e0.x);
            rng.s0 = f2u(e0.y);
            rng.s1 = f2u(e0.z);
            v = f2u(e4.w);
            const Params& P = view_of<ONE>(views, one, v).P;
            ms.light_num = e0.w;
            ms.brdf_component = e1.w;
            ms.brdf_dir.x = e2.w;
            ms.brdf_dir.y = e3.w;
            ms.light_uvw = V3(e4.x, e4.y, e4.z);
            SE.type = 0; SE.valid = true; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
            SE.P = V3(e1.x, e1.y, e1.z);
            float gm = -1.0f;
            if (P.gradient_mode == 1) {
                Grad6 g6;
                gradient_samples(P, SE.P, g6);
                SE.N = vnorm(gradient_cd6(g6));
                if (P.apply_shading_type && P.shading_type >= 2 && P.shading_type <= 4) gm = gradient_magnitude6(P, g6);
            } else {
                SE.N = normalized_gradient(P, SE.P);
            }
            SE.Wo = V3(e3.x, e3.y, e3.z);
            I = get_intensity(P, SE.P);
            ShadeTF tf;
            shade_tf(P, I, tf);
            bool early = P.light_count <= 0;
            if (!early) {
                idx = (int)floorf(ms.light_num * (float)P.light_count);
                early = idx < 0 || idx >= P.light_count || !P.light_valid[idx];
            }
            if (early) {
                const c3 Lv = cadd(C3(0, 0, 0), cadd(C3(0, 0, 0), tf.Le));
                results[sample] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
            } else {
                type = P.apply_shading_type ? select_shader_type(P, SE, I, rng, gm) : 0;
                push = true;
            }
        }
        const uint32_t s_brdf = queue_slot(push && type == 0, n_records);
        const uint32_t s_phase = queue_slot(push && type != 0, n_records + 1);
        if (push) {
            float4* r = records + (size_t)(type == 0 ? s_brdf : cap - 1u - s_phase) * 5;
            r[0] = make_float4(u2f(sample), u2f(rng.s0), u2f(rng.s1), u2f(v));
            r[1] = make_float4(SE.P.x, SE.P.y, SE.P.z, u2f((uint32_t)I | ((uint32_t)idx << 16) | ((uint32_t)type << 28)));
            r[2] = make_float4(SE.N.x, SE.N.y, SE.N.z, ms.brdf_component);
            r[3] = make_float4(SE.Wo.x, SE.Wo.y, SE.Wo.z, ms.brdf_dir.x);
            r[4] = make_float4(ms.light_uvw.x, ms.light_uvw.y, ms.light_uvw.z, ms.brdf_dir.y);
        }
    }
}

/* MINB: resident 128-thread blocks per SM, as k_wf_shade */
template <bool ONE, int MINB>
__global__ void __launch_bounds__(128, MINB) k_wf_shade_sorted(const WfView* __restrict__ views, const WfView one,
                                                               const float4* __restrict__ records, uint32_t cap,
                                                               const uint32_t* __restrict__ n_records, float4* __restrict__ results,
                                                               float4* __restrict__ jobs, uint32_t* __restrict__ n_jobs)
{
    const uint32_t nb = n_records[0];
    const uint32_t n = nb + n_records[1];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool push = false;
        uint32_t sample = 0, flags = 0, v = 0;
        Rng rng;
        rng.s0 = 0u;
        rng.s1 = 0u;
        Event SE;
        c3 Le = C3(0, 0, 0), c1 = C3(0, 0, 0), c2 = C3(0, 0, 0);
        v3 S1 = V3(0, 0, 0), S2 = V3(0, 0, 0);
        float count = 0.0f;
        if (i < n) {
            const float4* r = records + (size_t)(i < nb ? i : cap - 1u - (i - nb)) * 5;
            const float4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3], r4 = r[4];
            sample = f2u(r0.x);
            rng.s0 = f2u(r0.y);
            rng.s1 = f2u(r0.z);
            v = f2u(r0.w);
            const Params& P = view_of<ONE>(views, one, v).P;
            const uint32_t meta = f2u(r1.w);
            const float I = (float)(meta & 0xffffu);
            const int idx = (int)((meta >> 16) & 0xfffu);
            const int type = (int)(meta >> 28);
            Metro ms;
            ms.brdf_component = r2.w;
            ms.brdf_dir.x = r3.w;
            ms.brdf_dir.y = r4.w;
            ms.light_uvw = V3(r4.x, r4.y, r4.z);
            SE.type = 0; SE.valid = true; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
            SE.P = V3(r1.x, r1.y, r1.z);
            SE.N = V3(r2.x, r2.y, r2.z);
            SE.Wo = V3(r3.x, r3.y, r3.z);
            ShadeTF tf;
            shade_tf(P, I, tf);
            Le = cadd(C3(0, 0, 0), tf.Le);
            {
                const Light& L = P.lights[idx];
                Shader sh;
                shader_init(sh, type, SE.N, SE.Wo, tf.Kd, tf.Ks, P.volume_ior, tf.exponent);
                count = (float)P.light_count;
                /* EstimateDirectLight - Source/transport.h:58-113, without the visibility terms */
                v3 Wi;
                c3 Li;
                Surf SS;
                sample_light(P, L, ms.light_uvw, SS, SE, Wi, Li);
                const c3 F = shader_f(sh, SE.Wo, Wi);
                const bool full = P.mis == 1;
                const float BsdfPdf = full ? mis_bsdf_pdf(sh, SE.Wo, Wi) : shader_pdf(sh, SE.Wo, Wi);
                if (!cblack(Li) && !cblack(F) && BsdfPdf > 0.0f) {
                    const float LightPdf = vlen2(vsub(SE.P, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L.area);
                    if (full) {
                        const float w = power_heuristic(LightPdf, BsdfPdf);
                        c1 = cscale(cmul(F, Li), sh.type == 0 ? vabsdot(Wi, SE.N) * w / LightPdf : w / LightPdf);
                    } else if (sh.type == 0) {
                        c1 = cscale(cmul(F, Li), vabsdot(Wi, SE.N) * power_heuristic(LightPdf, BsdfPdf) / LightPdf);
                    } else {
                        c1 = cdivs(cmul(F, Li), LightPdf);
                    }
                    S1 = SS.P;
                    flags |= WF_RAY1;
                }
                if (full) {
                    const v3 Wb = sample_bsdf_dir(sh, SE.Wo, ms);
                    const c3 Fb = shader_f(sh, SE.Wo, Wb);
                    const float pb = mis_bsdf_pdf(sh, SE.Wo, Wb);
                    if (!cblack(Fb) && pb > 0.0f) {
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
                        if (SE2.valid && P.light_ids[hit] == P.light_ids[idx]) SE2.Le = light_emission(P, P.lights[hit], lh);
                        if (SE2.valid && P.light_ids[hit] == P.light_ids[idx] && !cblack(SE2.Le)) {
                            const float LightPdf = vlen2(vsub(SE.P, SE2.P)) / (vabsdot(SE2.N, vneg(Wb)) * L.area);
                            const float w = power_heuristic(pb, LightPdf);
                            c2 = cscale(cmul(Fb, SE2.Le), sh.type == 0 ? vabsdot(Wb, SE.N) * w / pb : w / pb);
                            S2 = SE2.P;
                            flags |= WF_RAY2;
                        }
                    }
                }
                if (flags == 0) {
                    const c3 Lv = cadd(C3(0, 0, 0), cscale(cadd(Le, C3(0, 0, 0)), count));
                    results[sample] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
                } else {
                    push = true;
                }
            }
        }
        const uint32_t slot = queue_slot(push, n_jobs);
        if (push) {
            float4* j = jobs + (size_t)slot * 6;
            j[0] = make_float4(u2f(sample), u2f(rng.s0), u2f(rng.s1), u2f(flags));
            j[1] = make_float4(SE.P.x, SE.P.y, SE.P.z, count);
            j[2] = make_float4(S1.x, S1.y, S1.z, Le.r);
            j[3] = make_float4(c1.r, c1.g, c1.b, Le.g);
            j[4] = make_float4(S2.x, S2.y, S2.z, Le.b);
            j[5] = make_float4(c2.r, c2.g, c2.b, u2f(v));
        }
    }
}

/* ---- stage 3: shadow segments and the sample's sum ---- */

template <int MINB, bool ONE, bool OBJ, bool SKIP>
__global__ void __launch_bounds__(256, MINB) k_wf_shadow(const WfView* __restrict__ views, const WfView one, const float4* __restrict__ jobs,
                                                          const uint32_t* __restrict__ n_jobs, float4* __restrict__ results)
{
    const uint32_t n = *n_jobs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j_i = blockIdx.x * blockDim.x + threadIdx.x; j_i < n; j_i += stride) {
        const float4* j = jobs + (size_t)j_i * 6;
        const float4 j0 = j[0], j1 = j[1], j2 = j[2], j3 = j[3], j4 = j[4], j5 = j[5];
        const Params& P = view_of<ONE>(views, one, f2u(j5.w)).P;
        const bool ref_mode = P.mis != 1 && P.free_flight != 1;
        const uint32_t sample = f2u(j0.x);
        Rng rng;
        rng.s0 = f2u(j0.y);
        rng.s1 = f2u(j0.z);
        const uint32_t flags = f2u(j0.w);
        const v3 Pp = V3(j1.x, j1.y, j1.z);
        const float count = j1.w;
        const c3 Le = C3(j2.w, j3.w, j4.w);
        c3 dl = C3(0, 0, 0);
        if (flags & WF_RAY1) {
            const float Tr = visibility<OBJ, SKIP>(P, Pp, V3(j2.x, j2.y, j2.z), rng);
            if (Tr > 0.0f) {
                const c3 c1 = C3(j3.x, j3.y, j3.z);
                dl = ref_mode ? cadd(dl, c1) : cadd(dl, cscale(c1, Tr));
            }
        }
        if (flags & WF_RAY2) {
            const float Tr = visibility<OBJ, SKIP>(P, Pp, V3(j4.x, j4.y, j4.z), rng);
            if (Tr > 0.0f) dl = cadd(dl, cscale(C3(j5.x, j5.y, j5.z), Tr));
        }
        const c3 Lv = cadd(C3(0, 0, 0), cscale(cadd(Le, dl), count));
        results[sample] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
    }
}

/* ---- stage 3, persistent lanes (delta tracking: ratio-tracked shadows) ----

   The same jobs and arithmetic as k_wf_shadow, with the work split
   differently: lanes track one collision or majorant brick per inner loop
   trip; when most of a warp's tracking lanes have ended their segments,
   the warp starts their next segments or takes new jobs (consecutive ones,
   one atomic per warp) and tracks on.  In k_wf_shadow a warp runs until its
   longest segment ends while the other lanes idle (5.5 of 32 lanes active
   per instruction on the c2 workload). */
template <int MINB, bool ONE, bool OBJ, bool SKIP>
__global__ void __launch_bounds__(256, MINB) k_wf_shadow_pt(const WfView* __restrict__ views, const WfView one,
                                                             const float4* __restrict__ jobs, const uint32_t* __restrict__ n_jobs,
                                                             float4* __restrict__ results, uint32_t* __restrict__ fetch, int refill)
{
    const uint32_t n = *n_jobs;
    const int lane = threadIdx.x & 31;
    uint32_t j_i = 0;
    bool exhausted = false;
    /* phase 0: take a job; 1, 2: tracking shadow segment 1 or 2; 3: write the sample */
    int phase = 0;
    uint32_t flags = 0, v = 0;
    Rng rng;
    rng.s0 = 0u;
    rng.s1 = 0u;
    c3 dl = C3(0, 0, 0);
    Ray R;
    RatioTracker k;
    k.done = true;
    k.Tr = 1.0f;
    for (;;) {
        /* lanes without a job take the next jobs together (one atomic per warp) */
        const unsigned needy = __ballot_sync(0xffffffffu, phase == 0 && !exhausted);
        if (needy) {
            const int leader = __ffs(needy) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(needy));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (phase == 0 && !exhausted) {
                j_i = base + (uint32_t)__popc(needy & ((1u << lane) - 1u));
                exhausted = j_i >= n;
            }
        }
        if (phase == 0 && !exhausted) {
            const float4* j = jobs + (size_t)j_i * 6;
            const float4 j0 = j[0];
            rng.s0 = f2u(j0.y);
            rng.s1 = f2u(j0.z);
            flags = f2u(j0.w);
            v = f2u(j[5].w);
            dl = C3(0, 0, 0);
            phase = (flags & WF_RAY1) ? 1 : ((flags & WF_RAY2) ? 2 : 3);
            if (phase != 3) {
                /* Visible (Source/transport.h:46-56) up to the tracking */
                const Params& P = view_of<ONE>(views, one, v).P;
                const float4 j1 = j[1], js = j[phase == 1 ? 2 : 4];
                k.done = true;
                k.Tr = 1.0f;
                if (P.shadows) {
                    R = shadow_ray(P, V3(j1.x, j1.y, j1.z), V3(js.x, js.y, js.z));
                    if (intersects_light(P, R) || (OBJ && P.object_count > 0 && intersects_object(P, R))) k.Tr = 0.0f;
                    else ratio_begin(P, R, rng, k);
                }
            }
        }
        if (!__any_sync(0xffffffffu, phase != 0)) break;
        const bool seg_phase = phase == 1 || phase == 2;
        const Params& P = view_of<ONE>(views, one, v).P;
        /* track until most of the lanes that were tracking have ended */
        const int n_work = __popc(__ballot_sync(0xffffffffu, seg_phase && !k.done));
        while (seg_phase && !k.done) {
            ratio_step<SKIP>(P, R, rng, k);
            if (k.done || 8 * __popc(__activemask()) < refill * n_work) break;
        }
        if (seg_phase && k.done) {
            const float4* j = jobs + (size_t)j_i * 6;
            const float Tr = k.Tr;
            if (Tr > 0.0f) {
                const float4 c = j[phase == 1 ? 3 : 5];
                dl = cadd(dl, cscale(C3(c.x, c.y, c.z), Tr));
            }
            if (phase == 1 && (flags & WF_RAY2)) {
                phase = 2;
                const float4 j1 = j[1], js = j[4];
                k.done = true;
                k.Tr = 1.0f;
                if (P.shadows) {
                    R = shadow_ray(P, V3(j1.x, j1.y, j1.z), V3(js.x, js.y, js.z));
                    if (intersects_light(P, R) || (OBJ && P.object_count > 0 && intersects_object(P, R))) k.Tr = 0.0f;
                    else ratio_begin(P, R, rng, k);
                }
            } else {
                phase = 3;
            }
        }
        if (phase == 3) {
            const float4* j = jobs + (size_t)j_i * 6;
            const float4 j0 = j[0], j1 = j[1], j2 = j[2], j3 = j[3], j4 = j[4];
            const c3 Le = C3(j2.w, j3.w, j4.w);
            const c3 Lv = cadd(C3(0, 0, 0), cscale(cadd(Le, dl), j1.w));
            results[f2u(j0.x)] = make_float4(Lv.r, Lv.g, Lv.b, 1.0f);
            phase = 0;
        }
    }
}

/* ---- stage 4: per-pixel sum in sample order (blockIdx.y = segment) ---- */

/* partial_in holds the sums of the previous window's last view when this
   window's first segment continues it; partial_out receives the sums of this
   window's last view when the next window continues it */
template <bool ONE>
__global__ void k_wf_reduce(const WfView* __restrict__ views, const WfSegment* __restrict__ segs, const WfView one,
                            const WfSegment one_seg, const float4* __restrict__ results, const float4* __restrict__ partial_in,
                            float4* __restrict__ partial_out)
{
    const WfSegment sg = ONE ? one_seg : segs[blockIdx.y];
    const WfView& V = view_of<ONE>(views, one, sg.view);
    const int npix = V.P.film[0] * V.P.film[1];
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= npix) return;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    if (sg.s0 > 0) {
        const float4 p = partial_in[slot];
        a0 = p.x; a1 = p.y; a2 = p.z; a3 = p.w;
    }
    for (int s = sg.s0; s < sg.s1; s++) {
        const float4 o = results[(size_t)sg.offset + (size_t)(s - sg.s0) * npix + slot];
        a0 += o.x; a1 += o.y; a2 += o.z; a3 += o.w;
    }
    if (sg.s1 < V.spp) {
        partial_out[slot] = make_float4(a0, a1, a2, a3);
        return;
    }
    const uint32_t pix = slot_pixel(V.P, (uint32_t)slot);
    float4 r = make_float4(a0, a1, a2, a3);
    if (V.accumulate) {
        const float4 q = V.sum[pix];
        r = make_float4(q.x + a0, q.y + a1, q.z + a2, q.w + a3);
    }
    V.sum[pix] = r;
}

/* ---- host side ---- */

void er_wavefront_plan(const int* npix, const int* spp, int n_views, size_t window_cap, WavefrontPlan& plan)
{
    plan.segs.clear();
    plan.window_first.clear();
    plan.window_items.clear();
    plan.view_npix.assign(npix, npix + n_views);
    plan.max_items = 0;
    plan.max_npix = 0;
    size_t used = 0;
    for (int v = 0; v < n_views; v++) {
        if (npix[v] > plan.max_npix) plan.max_npix = npix[v];
        int s = 0;
        while (s < spp[v]) {
            if (plan.window_first.empty() || used + (size_t)npix[v] > window_cap) {
                plan.window_first.push_back((int)plan.segs.size());
                plan.window_items.push_back(0);
                used = 0;
            }
            size_t rows = (window_cap - used) / (size_t)npix[v];
            if (rows < 1) rows = 1;
            if (rows > (size_t)(spp[v] - s)) rows = (size_t)(spp[v] - s);
            WfSegment g;
            g.view = v;
            g.s0 = s;
            g.s1 = s + (int)rows;
            g.offset = (uint32_t)used;
            plan.segs.push_back(g);
            used += rows * (size_t)npix[v];
            plan.window_items.back() = (uint32_t)used;
            if (used > plan.max_items) plan.max_items = used;
            s += (int)rows;
        }
    }
}

namespace {

/* stage timing (er_profile_*): CUDA events around every stage launch on the
   launching stream, read back and accumulated by er_wavefront_profile_read */
struct StageProfiler {
    std::mutex m;
    bool enabled = false;
    struct Mark { cudaEvent_t a, b; int stage; };
    std::vector<Mark> pending;
    std::vector<cudaEvent_t> pool;
    double ms[WF_STAGES] = {0.0, 0.0, 0.0, 0.0};
    int64_t launches[WF_STAGES] = {0, 0, 0, 0};
    cudaEvent_t get()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
};

StageProfiler& profiler()
{
    static StageProfiler* p = new StageProfiler();
    return *p;
}

/* records the start of a stage; returns the event or nullptr when off */
cudaEvent_t stage_begin(cudaStream_t s)
{
    StageProfiler& P = profiler();
    std::lock_guard<std::mutex> lock(P.m);
    if (!P.enabled) return nullptr;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs != cudaStreamCaptureStatusNone) return nullptr;   /* not inside graphs */
    cudaEvent_t a = P.get();
    cudaEventRecord(a, s);
    return a;
}

void stage_end(cudaEvent_t a, int stage, cudaStream_t s)
{
    if (!a) return;
    StageProfiler& P = profiler();
    std::lock_guard<std::mutex> lock(P.m);
    cudaEvent_t b = P.get();
    cudaEventRecord(b, s);
    P.pending.push_back({a, b, stage});
}

int sm_count()
{
    int sm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    return sm > 0 ? sm : 132;
}

/* occupancy variants of the delta-tracking stages (persistent or per-thread,
   all with the empty-space jump): 2, 3, 4 or 6 resident blocks per SM (other
   values run 4) */
int narrow_minb(int m) { return (m == 2 || m == 3 || m == 6) ? m : 4; }

template <bool ONE>
cudaError_t launch_windows(const WfView* d_views, const WfSegment* d_segs, const WfView& one, const WavefrontPlan& plan,
                           const WavefrontBuffers& B, cudaStream_t s)
{
    const int sm = sm_count();
    const int nw = (int)plan.window_first.size();
    for (int w = 0; w < nw; w++) {
        const int s0 = plan.window_first[w];
        const int s1 = (w + 1 < nw) ? plan.window_first[w + 1] : (int)plan.segs.size();
        const int nseg = s1 - s0;
        const uint32_t items = plan.window_items[w];
        const WfSegment* dseg = ONE ? nullptr : d_segs + s0;
        const WfSegment one_seg = plan.segs[s0];
        float4* p_in = B.partial + (size_t)((w + 1) & 1) * plan.max_npix;
        float4* p_out = B.partial + (size_t)(w & 1) * plan.max_npix;
        cudaError_t e = cudaMemsetAsync(B.counters, 0, 6 * sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
        const uint32_t g1 = (items + 255) / 256 < (uint32_t)sm * 64 ? (items + 255) / 256 : (uint32_t)sm * 64;
        cudaEvent_t t0 = stage_begin(s);
#define ER_PRIMARY(M, O, K) k_wf_primary<M, ONE, O, K><<<g1, 256, 0, s>>>(d_views, dseg, nseg, one, one_seg, items, B.results, B.events, B.counters)
#define ER_PRIMARY_PT(M, O, K) k_wf_primary_pt<M, ONE, O, K><<<sm * M, 256, 0, s>>>(d_views, dseg, nseg, one, one_seg, items, B.results, B.events, B.counters, B.counters + 2, B.refill_eighths)
        if (B.pt_primary) {
            /* delta tracking: persistent lanes, one resident wave */
            if (B.objects) ER_PRIMARY_PT(4, true, true);
            else {
                /* persistent lanes run only with delta tracking, which always jumps */
                switch (narrow_minb(B.tune_primary)) {
                case 2: ER_PRIMARY_PT(2, false, true); break;
                case 3: ER_PRIMARY_PT(3, false, true); break;
                case 6: ER_PRIMARY_PT(6, false, true); break;
                default: ER_PRIMARY_PT(4, false, true); break;
                }
            }
        } else if (B.objects) ER_PRIMARY(4, true, true);
        else if (B.skip_primary) {
            switch (narrow_minb(B.tune_primary)) {
            case 2: ER_PRIMARY(2, false, true); break;
            case 3: ER_PRIMARY(3, false, true); break;
            case 6: ER_PRIMARY(6, false, true); break;
            default: ER_PRIMARY(4, false, true); break;
            }
        } else {
            switch (B.tune_primary) {
            case 2: ER_PRIMARY(2, false, false); break;
            case 3: ER_PRIMARY(3, false, false); break;
            case 6: ER_PRIMARY(6, false, false); break;
            case 8: ER_PRIMARY(8, false, false); break;
            default: ER_PRIMARY(4, false, false); break;
            }
        }
#undef ER_PRIMARY_PT
#undef ER_PRIMARY
        stage_end(t0, 0, s);
        t0 = stage_begin(s);
#define ER_SHADE(M, O) k_wf_shade<ONE, M, O><<<sm * 16, 128, 0, s>>>(d_views, one, B.events, B.counters, B.results, B.jobs, B.counters + 1)
#define ER_SORTED(M) k_wf_shade_sorted<ONE, M><<<sm * 16, 128, 0, s>>>(d_views, one, B.records, cap, B.counters + 4, B.results, B.jobs, \
                                                                    B.counters + 1)
        const uint32_t cap = (uint32_t)plan.max_items;
        if (B.objects) ER_SHADE(2, true);
        else if (B.sort_shade) {
            /* shader switch mixing BRDF and phase events: classify, then shade by shader */
            k_wf_classify<ONE><<<sm * 16, 128, 0, s>>>(d_views, one, B.events, B.counters, B.results, B.records, cap, B.counters + 4);
            switch (B.tune_shade) {
            case 3: ER_SORTED(3); break;
            case 4: ER_SORTED(4); break;
            case 6: ER_SORTED(6); break;
            default: ER_SORTED(2); break;
            }
        } else switch (B.tune_shade) {
        case 3: ER_SHADE(3, false); break;
        case 4: ER_SHADE(4, false); break;
        case 6: ER_SHADE(6, false); break;
        default: ER_SHADE(2, false); break;
        }
#undef ER_SORTED
#undef ER_SHADE
        stage_end(t0, 1, s);
        t0 = stage_begin(s);
#define ER_SHADOW(M, O, K) k_wf_shadow<M, ONE, O, K><<<sm * 8, 256, 0, s>>>(d_views, one, B.jobs, B.counters + 1, B.results)
#define ER_SHADOW_PT(M, O, K) k_wf_shadow_pt<M, ONE, O, K><<<sm * M, 256, 0, s>>>(d_views, one, B.jobs, B.counters + 1, B.results, B.counters + 3, B.refill_eighths)
        if (B.pt_shadow) {
            /* ratio-tracked shadows: persistent lanes, one resident wave */
            if (B.objects) ER_SHADOW_PT(4, true, true);
            else {
                /* persistent lanes run only with delta tracking, which always jumps */
                switch (narrow_minb(B.tune_shadow)) {
                case 2: ER_SHADOW_PT(2, false, true); break;
                case 3: ER_SHADOW_PT(3, false, true); break;
                case 6: ER_SHADOW_PT(6, false, true); break;
                default: ER_SHADOW_PT(4, false, true); break;
                }
            }
        } else if (B.objects) ER_SHADOW(4, true, true);
        else if (B.skip_shadow) {
            switch (narrow_minb(B.tune_shadow)) {
            case 2: ER_SHADOW(2, false, true); break;
            case 3: ER_SHADOW(3, false, true); break;
            case 6: ER_SHADOW(6, false, true); break;
            default: ER_SHADOW(4, false, true); break;
            }
        } else {
            switch (B.tune_shadow) {
            case 2: ER_SHADOW(2, false, false); break;
            case 3: ER_SHADOW(3, false, false); break;
            case 6: ER_SHADOW(6, false, false); break;
            case 8: ER_SHADOW(8, false, false); break;
            default: ER_SHADOW(4, false, false); break;
            }
        }
#undef ER_SHADOW_PT
#undef ER_SHADOW
        stage_end(t0, 2, s);
        int max_npix = 0;
        for (int g = s0; g < s1; g++) {
            const int np = plan.view_npix[plan.segs[g].view];
            if (np > max_npix) max_npix = np;
        }
        t0 = stage_begin(s);
        k_wf_reduce<ONE><<<dim3((max_npix + 255) / 256, ONE ? 1 : nseg), 256, 0, s>>>(d_views, dseg, one, one_seg, B.results, p_in, p_out);
        stage_end(t0, 3, s);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t er_launch_wavefront_one(const WfView& view, const WavefrontPlan& plan, const WavefrontBuffers& B, cudaStream_t s)
{
    return launch_windows<true>(nullptr, nullptr, view, plan, B, s);
}

cudaError_t er_launch_wavefront_batch(const WfView* d_views, const WfSegment* d_segs, const WavefrontPlan& plan,
                                      const WavefrontBuffers& B, cudaStream_t s)
{
    WfView unused;
    memset(&unused, 0, sizeof(unused));
    return launch_windows<false>(d_views, d_segs, unused, plan, B, s);
}

void er_wavefront_profile_enable(bool on)
{
    StageProfiler& P = profiler();
    std::lock_guard<std::mutex> lock(P.m);
    P.enabled = on;
}

cudaError_t er_wavefront_profile_read(double* ms, int64_t* launches)
{
    StageProfiler& P = profiler();
    std::lock_guard<std::mutex> lock(P.m);
    cudaError_t err = cudaSuccess;
    for (const auto& k : P.pending) {
        cudaError_t e = cudaEventSynchronize(k.b);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, k.a, k.b);
        if (e != cudaSuccess) err = e;
        P.ms[k.stage] += t;
        P.launches[k.stage]++;
        P.pool.push_back(k.a);
        P.pool.push_back(k.b);
    }
    P.pending.clear();
    for (int i = 0; i < WF_STAGES; i++) {
        ms[i] = P.ms[i];
        launches[i] = P.launches[i];
        P.ms[i] = 0.0;
        P.launches[i] = 0;
    }
    return err;
}
