/*
 * er_runtime.cu - host runtime behind the C ABI of include/er_capi.h.
 *
 * Replaces the reference's List<D,H> bind lists and RenderEstimate pipeline
 * (Source/list.cuh:27-173, Source/core.cu:50-155) with:
 *   - std::map registries with the same ID semantics (ID = counter++, update
 *     in place, no reuse, at most 31 items per list checked before the
 *     update-or-insert decision as Source/list.cuh:63-83 does);
 *   - per-tracer device blocks (transfer functions, resolved lights,
 *     textures, sigma table, film buffers) rebuilt only when an item the
 *     tracer depends on changed, instead of re-uploading every list every
 *     frame (Source/core.cu:128, Source/list.cuh:108-148);
 *   - asynchronous, stream-ordered launches (the reference synchronises
 *     around every call, Source/wrapper.cuh:53-141).
 *
 * Host arithmetic that feeds the kernels (camera frame, volume geometry,
 * light areas) follows Source/camera.h:61-96, Source/volume.h:100-129 and
 * Source/shape.h:92-103 operation for operation; this file is compiled with
 * -ffp-contract=off so the host never fuses those multiply-adds.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "er_capi.h"
#include "er_kernels.h"
#include "er_math.h"

namespace {

thread_local std::string g_last_error = "";

er_status fail(er_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

#define ER_CUDA(call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            if (e_ == cudaErrorMemoryAllocation)                                                      \
                return fail(ER_ERR_OUT_OF_MEMORY, "%s: %s", #call, cudaGetErrorString(e_));           \
            return fail(ER_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));                        \
        }                                                                                             \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t ensure(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        else p = nullptr;
        return e;
    }
};

/* FNV-1a, 64 bit */
constexpr uint64_t kFnvBasis = 14695981039346656037ull;
uint64_t fnv1a(uint64_t h, const void* data, size_t n)
{
    const unsigned char* p = (const unsigned char*)data;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

/* items of one wavefront window: 8M samples, 1.5 GB of queues */
constexpr size_t kWindowCap = (size_t)8 << 20;

/* the persistent stages' refill threshold in eighths of a warp's tracking
   lanes: 2, or ER_PT_REFILL (1..7) for measurements (with the empty-space
   jump and tight bricks, C2 / C3 at 2, 3, 4, 5 eighths: 1336 / 2322, 1333 /
   2266, 1317 / 2183, 1278 / 2051 Msamples/s) */
int refill_eighths()
{
    static int v = 0;
    if (!v) {
        const char* e = getenv("ER_PT_REFILL");
        const int r = e ? atoi(e) : 2;
        v = (r >= 1 && r <= 7) ? r : 2;
    }
    return v;
}

/* lanes of the wavefront's tracking stages in 4x8 pixel tiles (the default;
   C2 row order / 8x4 / 4x8 / 16x2: 1346 / 1463-1475 / 1499 / 1405
   Msamples/s), or for measurements (ER_TILE_ORDER) row by row (0), 8x4 (1)
   or 16x2 (3) tiles */
int tile_order()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("ER_TILE_ORDER");
        const int r = e ? atoi(e) : 2;
        v = (r >= 0 && r <= 3) ? r : 2;
    }
    return v;
}

/* queues of the wavefront stages, grown to the largest plan seen */
struct WfQueues {
    DevBuf<float4> results, events, jobs, partial, records;
    DevBuf<uint32_t> counters;
    cudaError_t ensure(const WavefrontPlan& plan, WavefrontBuffers& B)
    {
        cudaError_t e;
        if ((e = results.ensure(plan.max_items)) != cudaSuccess) return e;
        if ((e = events.ensure(5 * plan.max_items)) != cudaSuccess) return e;
        if ((e = jobs.ensure(6 * plan.max_items)) != cudaSuccess) return e;
        if ((e = partial.ensure(2 * (size_t)plan.max_npix)) != cudaSuccess) return e;
        if ((e = counters.ensure(6)) != cudaSuccess) return e;
        B.results = results.p;
        B.events = events.p;
        B.jobs = jobs.p;
        B.partial = partial.p;
        B.records = nullptr;
        B.sort_shade = 0;
        B.refill_eighths = refill_eighths();
        B.counters = counters.p;
        B.tune_primary = 4;
        B.tune_shadow = 4;
        B.tune_shade = 2;
        B.objects = 0;
        B.pt_primary = 0;
        B.pt_shadow = 0;
        B.skip_primary = 0;
        B.skip_shadow = 0;
        return cudaSuccess;
    }
    /* the shading records of the sorted shade stage, when a view mixes shaders */
    cudaError_t ensure_sorted(const WavefrontPlan& plan, bool mixed, WavefrontBuffers& B)
    {
        B.sort_shade = 0;
        if (!mixed) return cudaSuccess;
        cudaError_t e = records.ensure(5 * plan.max_items);
        if (e != cudaSuccess) return e;
        B.records = records.p;
        B.sort_shade = 1;
        return cudaSuccess;
    }
};

/* the shader switch picks BRDF or phase per event (hybrid, modulation,
   threshold), so the sorted shade stage pays */
bool mixes_shaders(const erd::Params& P)
{
    return P.apply_shading_type && P.shading_type >= ER_SHADING_HYBRID && P.shading_type <= ER_SHADING_THRESHOLD;
}

float smin_h(float a, float b) { return (b < a) ? b : a; }
float smax_h(float a, float b) { return (a < b) ? b : a; }

struct V3h { float x, y, z; };
V3h v3h(float x, float y, float z) { V3h r = {x, y, z}; return r; }
V3h sub(V3h a, V3h b) { return v3h(a.x - b.x, a.y - b.y, a.z - b.z); }
float len(V3h a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
V3h norm(V3h a) { const float L = len(a); return v3h(a.x / L, a.y / L, a.z / L); }
V3h cross(V3h a, V3h b) { return v3h((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)); }

/* Shape::Update (Source/shape.h:92-103) */
float shape_area(const er_shape& s)
{
    const float PI = 3.141592654f;
    switch (s.type) {
    case ER_SHAPE_PLANE: return s.size[0] * s.size[1];
    case ER_SHAPE_DISK: return PI * (s.outer_radius * s.outer_radius);
    case ER_SHAPE_RING: return PI * (s.outer_radius * s.outer_radius) - PI * (s.inner_radius * s.inner_radius);
    case ER_SHAPE_BOX: return (2.0f * s.size[0] * s.size[1]) + (2.0f * s.size[0] * s.size[2]) + (2.0f * s.size[1] * s.size[2]);
    case ER_SHAPE_SPHERE: return 4.0f * PI * (s.outer_radius * s.outer_radius);
    case ER_SHAPE_CYLINDER: return (2.0f * PI * (s.outer_radius * s.outer_radius)) + (2.0f * PI * s.outer_radius * s.size[2]);
    default: return s.area;
    }
}

struct VolumeItem {
    int res[3];
    float spacing[3];
    int normalize;
    uint16_t vmax = 0;
    uint64_t signature = 0;        /* sampled content hash (tuning cache key) */
    uint64_t edits = 0;            /* region edits from device voxels (folded into the signature) */
    DevBuf<uint16_t> vox;
    DevBuf<uint2> quad;            /* corner quads (NULL when they do not fit in memory) */
    int qb_nbx = 0;                /* quads in 8^3 bricks: bricks along x (0: x fastest) */
    unsigned long long qb_slab = 0;
    DevBuf<unsigned int> gm_max_bits;
    DevBuf<unsigned int> box_max;  /* largest voxel of an uploaded box */
    float gm_max = -1.0f;          /* lazily computed maximum gradient magnitude */
};

struct BitmapItem {
    int res[2];
    DevBuf<uchar4> pixels;
};

struct TracerItem {
    er_tracer_desc d;
    int W = 0, H = 0;
    int no_iterations = 0;
    double n_samples = 0.0;        /* samples per pixel accumulated by er_render_spp */
    DevBuf<float4> frame, running, sum;
    DevBuf<uchar4> display, display_tmp, display_filtered;
    DevBuf<uint32_t> lanes;
    DevBuf<erd::Tfs> tfs;
    DevBuf<erd::Plf> opacity;
    DevBuf<erd::Light> lights;
    DevBuf<erd::Object> objects;
    DevBuf<erd::Clip> clips;
    DevBuf<erd::Bitmap> bitmaps;
    DevBuf<int> light_valid;
    DevBuf<erd::Texture> textures;
    DevBuf<float> sigma;
    DevBuf<float4> shade_tab;      /* shading transfer functions per integer intensity */
    DevBuf<int> light_ids;
    DevBuf<float> majorant, rmq;   /* majorant: per brick, or -(distance to a non-empty brick) when empty */
    DevBuf<uint8_t> skip_tmp;
    DevBuf<uint32_t> minmax;
    DevBuf<int> err;
    DevBuf<float> autofocus;       /* er_get_auto_focus_distance's result */
    WfQueues wf;
    DevBuf<float4> tune_sum;       /* probe renders of the autotuner */
    erd::Params P;
    uint64_t built_version = 0;
    uint64_t build_serial = 0;     /* distinct for every build of any tracer */
    bool built = false;
};

/* a planned multi-view batch (er_batch_create) */
struct BatchItem {
    std::vector<er_batch_view> views;
    std::vector<er_camera_desc> cameras;
    int flags = 0;
    size_t window_cap = kWindowCap;
    int tune_primary = 4, tune_shadow = 4, tune_shade = 2, tune_stages = 0;
    bool tune_explicit = false;    /* set by er_batch_set_tuning; else the first view's tracer settings */
    bool stages_explicit = false;  /* set by er_batch_set_stages / er_batch_autotune */
    uint64_t planned_version = 0;  /* context version the plan was made at */
    bool planned = false;
    WavefrontPlan plan;
    std::vector<WfView> host_views;
    DevBuf<WfView> d_views;
    DevBuf<WfSegment> d_segs;
    WfQueues wf;
    WavefrontBuffers B;
    int max_w = 0, max_h = 0;
    bool any_display = false;
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void drop_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    ~BatchItem()
    {
        drop_graph();
        if (capture_stream) cudaStreamDestroy(capture_stream);
    }
};

template <class T>
struct Registry {
    std::map<int, std::unique_ptr<T>> items;
    int counter = 0;
};

struct Context {
    std::recursive_mutex m;
    cudaStream_t stream = 0;
    int device = 0;
    uint64_t version = 1;          /* bumped by every bind/unbind */
    Registry<TracerItem> tracers;
    Registry<VolumeItem> volumes;
    Registry<er_light_desc> lights;
    Registry<er_texture_desc> textures;
    Registry<BitmapItem> bitmaps;
    Registry<er_object_desc> objects;
    Registry<er_clipping_object_desc> clipping;
    Registry<BatchItem> batches;   /* not a reference list: no 31-item capacity */
};

Context& ctx()
{
    static Context* c = new Context();
    return *c;
}

/* List::Bind capacity rule (Source/list.cuh:63-67): refused when
   Map.size() + 1 >= 32, before the update-or-insert decision */
template <class T>
er_status reserve_id(Registry<T>& r, int32_t* id, bool* is_new)
{
    if (!id) return fail(ER_ERR_INVALID_ARGUMENT, "id pointer is NULL");
    if (r.items.size() + 1 >= (size_t)(ER_MAX_ITEMS_PER_LIST + 1)) return fail(ER_ERR_LIST_FULL, "bind list is full (%d items)", ER_MAX_ITEMS_PER_LIST);
    const bool exists = *id >= 0 && r.items.count(*id) != 0;
    *is_new = !exists;
    if (!exists) *id = r.counter++;
    return ER_OK;
}

template <class T>
er_status unbind(Registry<T>& r, int32_t id)
{
    auto it = r.items.find(id);
    if (id < 0 || it == r.items.end()) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", id);
    r.items.erase(it);
    ctx().version++;
    return ER_OK;
}

void to_plf(erd::Plf& o, const er_plf& s)
{
    o.count = s.count;
    o.range0 = s.node_range[0];
    o.range1 = s.node_range[1];
    for (int i = 0; i < 128; i++) { o.pos[i] = s.position[i]; o.val[i] = s.value[i]; }
}

/* Shape (Source/shape.h): transforms, type, sizes and the area */
void to_shape(erd::Light& o, const er_shape& sh)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) { o.tm[i][j] = sh.tm[i][j]; o.inv_tm[i][j] = sh.inv_tm[i][j]; }
    o.one_sided = sh.one_sided;
    o.type = sh.type;
    for (int i = 0; i < 3; i++) o.size[i] = sh.size[i];
    o.area = shape_area(sh);
    o.inner_radius = sh.inner_radius;
    o.outer_radius = sh.outer_radius;
}

void to_light(erd::Light& o, const er_light_desc& s)
{
    to_shape(o, s.shape);
    o.visible = s.visible;
    o.texture_id = s.texture_id;
    o.multiplier = s.multiplier;
    o.unit = s.unit;
}

void to_texture(erd::Texture& o, const er_texture_desc& s)
{
    o.type = s.type;
    o.output_level = s.output_level;
    o.bitmap_id = s.bitmap_id;
    o.proc_type = s.procedural.type;
    for (int i = 0; i < 3; i++) {
        o.uniform[i] = s.procedural.uniform_color[i];
        o.checker1[i] = s.procedural.checker_color1[i];
        o.checker2[i] = s.procedural.checker_color2[i];
        to_plf(o.gradient[i], s.procedural.gradient.plf[i]);
    }
    o.offset[0] = s.offset[0]; o.offset[1] = s.offset[1];
    o.repeat[0] = s.repeat[0]; o.repeat[1] = s.repeat[1];
    o.flip[0] = s.flip[0]; o.flip[1] = s.flip[1];
}

/* Volume::operator=(const ErVolume&) - Source/volume.h:100-129 */
void volume_geometry(const VolumeItem& v, erd::Params& P)
{
    float scale = 0.0f;
    if (v.normalize) {
        const float p0 = (float)v.res[0] * v.spacing[0], p1 = (float)v.res[1] * v.spacing[1], p2 = (float)v.res[2] * v.spacing[2];
        scale = 1.0f / smax_h(p0, smax_h(p1, p2));
    }
    float sp[3], size[3];
    for (int i = 0; i < 3; i++) sp[i] = v.spacing[i] * scale;
    for (int i = 0; i < 3; i++) size[i] = (float)v.res[i] * sp[i];
    for (int i = 0; i < 3; i++) {
        P.res[i] = v.res[i];
        P.spacing[i] = sp[i];
        P.inv_size[i] = 1.0f / size[i];
        P.minp[i] = size[i] * -0.5f;
        P.half_size[i] = size[i] * 0.5f;
    }
    P.min_step = smin_h(sp[0], smin_h(sp[1], sp[2]));
    P.vox = v.vox.p;
    P.quad = v.quad.p;
    P.qb_nbx = v.qb_nbx;
    P.qb_slab = v.qb_slab;
}

/* Camera::Update - Source/camera.h:61-96 */
void camera_frame(const er_camera_desc& c, erd::Params& P)
{
    const V3h pos = v3h(c.pos[0], c.pos[1], c.pos[2]);
    const V3h target = v3h(c.target[0], c.target[1], c.target[2]);
    const V3h up = v3h(c.up[0], c.up[1], c.up[2]);
    const V3h N = norm(sub(target, pos));
    const V3h U = norm(cross(N, up));
    const V3h V = norm(cross(N, U));
    float fd = c.focal_distance;
    if (fd == -1.0f) fd = len(sub(target, pos));
    const float sc = er_tanf((0.5f * c.fov / 57.29577951308232f));
    const float aspect = (float)c.film_size[1] / (float)c.film_size[0];
    float s00, s01, s10, s11;
    if (aspect > 1.0f) { s00 = -sc; s01 = sc; s10 = -sc * aspect; s11 = sc * aspect; }
    else { s00 = -sc / aspect; s01 = sc / aspect; s10 = -sc; s11 = sc; }
    P.film[0] = c.film_size[0];
    P.film[1] = c.film_size[1];
    P.pos[0] = pos.x; P.pos[1] = pos.y; P.pos[2] = pos.z;
    P.N[0] = N.x; P.N[1] = N.y; P.N[2] = N.z;
    P.U[0] = U.x; P.U[1] = U.y; P.U[2] = U.z;
    P.V[0] = V.x; P.V[1] = V.y; P.V[2] = V.z;
    P.screen00 = s00;
    P.screen10 = s10;
    P.inv_screen0 = (s01 - s00) / (float)c.film_size[0];
    P.inv_screen1 = (s11 - s10) / (float)c.film_size[1];
    P.clip_near = c.clip_near;
    P.clip_far = c.clip_far;
    P.aperture = c.aperture_size;
    P.focal_distance = fd;
}

er_status check_settings(const er_tracer_desc& d)
{
    const er_render_settings& s = d.settings;
    if (!(s.step_factor_primary > 0.0f) || !(s.step_factor_shadow > 0.0f) || !std::isfinite(s.step_factor_primary) ||
        !std::isfinite(s.step_factor_shadow))
        return fail(ER_ERR_INVALID_ARGUMENT, "step factors must be finite and positive");
    if (!(s.density_scale > 0.0f) || !std::isfinite(s.density_scale)) return fail(ER_ERR_INVALID_ARGUMENT, "density_scale must be finite and positive");
    if (d.camera.film_size[0] <= 0 || d.camera.film_size[1] <= 0 || d.camera.film_size[0] > 32768 || d.camera.film_size[1] > 32768)
        return fail(ER_ERR_INVALID_ARGUMENT, "film size %d x %d out of range", d.camera.film_size[0], d.camera.film_size[1]);
    if (d.light_count < 0 || d.light_count > ER_MAX_INDICES) return fail(ER_ERR_INVALID_ARGUMENT, "light_count %d out of range", d.light_count);
    return ER_OK;
}

er_status init_lanes(TracerItem& t)
{
    const size_t n = (size_t)t.W * t.H;
    std::vector<uint32_t> h(2 * n);
    for (size_t p = 0; p < n; p++) er_seed_lanes(t.d.settings.seed, 0u, (uint32_t)p, 0xffffffffu, &h[p], &h[n + p]);
    ER_CUDA(cudaMemcpyAsync(t.lanes.p, h.data(), 2 * n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return ER_OK;
}

/* which tracking stages run persistent lanes (ER_PERSISTENT_*; delta
   tracking only).  Delta-tracking stages always compile the empty-space
   jump: it sets the face times the tracker continues from, so every path
   (and the oracle) takes it; the ER_TUNE_NO_SKIP_* bits are accepted and
   ignored. */
void persistent_stages(int mode, bool all_delta, WavefrontBuffers& B)
{
    B.skip_primary = all_delta;
    B.skip_shadow = all_delta;
    mode &= 3;
    B.pt_primary = all_delta && (mode == ER_PERSISTENT_BOTH || mode == ER_PERSISTENT_PRIMARY);
    B.pt_shadow = all_delta && (mode == ER_PERSISTENT_SHADOW || mode == ER_PERSISTENT_BOTH);
}

er_status reset_tracer_buffers(TracerItem& t)
{
    const size_t n = (size_t)t.W * t.H;
    cudaStream_t s = ctx().stream;
    ER_CUDA(cudaMemsetAsync(t.running.p, 0, n * sizeof(float4), s));
    ER_CUDA(cudaMemsetAsync(t.sum.p, 0, n * sizeof(float4), s));
    ER_CUDA(cudaMemsetAsync(t.frame.p, 0, n * sizeof(float4), s));
    ER_CUDA(cudaMemsetAsync(t.display.p, 0, n * sizeof(uchar4), s));
    ER_CUDA(cudaMemsetAsync(t.display_filtered.p, 0, n * sizeof(uchar4), s));
    t.no_iterations = 0;
    t.n_samples = 0.0;
    return init_lanes(t);
}

/* Assembles the kernel parameters of a tracer; uploads the dependent blocks
   when any bound item changed since the last build. */
er_status build(TracerItem& t)
{
    Context& C = ctx();
    if (t.built && t.built_version == C.version) return ER_OK;
    const er_tracer_desc& d = t.d;
    auto vit = C.volumes.items.find(d.volume_id);
    if (vit == C.volumes.items.end()) return fail(ER_ERR_INVALID_ID, "tracer references volume ID:%d which does not exist", d.volume_id);
    VolumeItem& v = *vit->second;
    if (d.settings.free_flight != ER_FREE_FLIGHT_MARCH && d.settings.free_flight != ER_FREE_FLIGHT_DELTA)
        return fail(ER_ERR_INVALID_ARGUMENT, "free_flight %d is not an ER_FREE_FLIGHT_* value", d.settings.free_flight);
    if (d.settings.mis != ER_MIS_LIGHT_ONLY && d.settings.mis != ER_MIS_FULL)
        return fail(ER_ERR_INVALID_ARGUMENT, "mis %d is not an ER_MIS_* value", d.settings.mis);
    const int brick = d.settings.majorant_brick > 0 ? d.settings.majorant_brick : 8;
    if (brick > 64) return fail(ER_ERR_INVALID_ARGUMENT, "majorant_brick %d out of range [1, 64]", brick);
    /* a volume bound without NormalizeSize has an empty box: no scatter
       event reads the gradient-magnitude range */
    const bool needs_gm = d.settings.apply_shading_type && d.settings.shading_type >= ER_SHADING_HYBRID &&
                          d.settings.shading_type <= ER_SHADING_THRESHOLD && v.normalize;
    if (needs_gm && v.gm_max < 0.0f) {
        /* GradientMagnitudeRange of the shader switch: maximum voxel-centre
           gradient magnitude (Source/gradientmagnitude.cuh:46-71) */
        float m = 0.0f;
        er_status gs = er_gradient_magnitude(vit->first, nullptr, &m);
        if (gs != ER_OK) return gs;
    }
    erd::Params P;
    memset(&P, 0, sizeof(P));
    volume_geometry(v, P);
    camera_frame(d.camera, P);
    const er_render_settings& s = d.settings;
    P.step_primary = s.step_factor_primary;
    P.step_shadow = s.step_factor_shadow;
    P.density_scale = s.density_scale;
    P.max_shadow_distance = s.max_shadow_distance;
    P.shadows = s.shadows;
    P.gradient_mode = s.gradient_computation;
    P.shading_type = s.shading_type;
    P.apply_shading_type = s.apply_shading_type;
    P.opacity_modulated = s.opacity_modulated;
    P.gradient_factor = s.gradient_factor;
    P.gradient_threshold = s.gradient_threshold;
    P.mis = s.mis;
    P.volume_ior = s.volume_ior > 0.0f ? s.volume_ior : 15.0f;
    P.seed = s.seed;
    P.stratify = s.stratify ? 1 : 0;
    P.gm_inv_max = (v.gm_max > 0.0f) ? 1.0f / v.gm_max : 0.0f;

    /* transfer functions */
    erd::Tfs tf;
    for (int c = 0; c < 3; c++) {
        to_plf(tf.diffuse[c], d.diffuse.plf[c]);
        to_plf(tf.specular[c], d.specular.plf[c]);
        to_plf(tf.emission[c], d.emission.plf[c]);
    }
    to_plf(tf.glossiness, d.glossiness);
    to_plf(tf.opacity, d.opacity);
    cudaStream_t st = C.stream;
    ER_CUDA(t.tfs.ensure(1));
    ER_CUDA(cudaMemcpyAsync(t.tfs.p, &tf, sizeof(tf), cudaMemcpyHostToDevice, st));
    /* sigma table over [0, max voxel] */
    const int n = (int)v.vmax + 1;
    ER_CUDA(t.sigma.ensure((size_t)n));
    ER_CUDA(t.opacity.ensure(1));
    ER_CUDA(cudaMemcpyAsync(t.opacity.p, &tf.opacity, sizeof(erd::Plf), cudaMemcpyHostToDevice, st));
    ER_CUDA(er_launch_sigma_table(t.opacity.p, s.density_scale, t.sigma.p, n, st));
    P.sigma = t.sigma.p;
    P.sigma_n = n;
    ER_CUDA(t.shade_tab.ensure(3 * (size_t)n));
    ER_CUDA(er_launch_shade_table(t.tfs.p, t.shade_tab.p, n, st));
    P.shade_tab = t.shade_tab.p;
    P.free_flight = s.free_flight;
    P.tile_order = tile_order();
    if (s.free_flight == ER_FREE_FLIGHT_DELTA) {
        int nb[3];
        for (int i = 0; i < 3; i++) nb[i] = (v.res[i] + brick - 1) / brick;
        const size_t total = (size_t)nb[0] * nb[1] * nb[2];
        int levels = 1;
        while ((1 << levels) <= n) levels++;
        ER_CUDA(t.majorant.ensure(total));
        ER_CUDA(t.minmax.ensure(total));
        ER_CUDA(t.rmq.ensure((size_t)levels * n));
        ER_CUDA(er_launch_majorant(v.vox.p, v.res, brick, nb, t.sigma.p, n, t.rmq.p, levels, t.minmax.p, s.density_scale,
                                   t.majorant.p, st));
        /* empty bricks carry minus their distance to the nearest non-empty
           one (read by the skipping stages, ignored by the others) */
        ER_CUDA(t.skip_tmp.ensure(2 * total));
        ER_CUDA(er_launch_empty_skip(t.majorant.p, nb, t.skip_tmp.p, st));
        P.brick = brick;
        for (int i = 0; i < 3; i++) P.nb[i] = nb[i];
        P.majorant = t.majorant.p;
    }
    /* lights in LightIDs order */
    const int lc = d.light_count;
    std::vector<erd::Light> L((size_t)std::max(lc, 1));
    std::vector<int> valid((size_t)std::max(lc, 1), 0);
    int max_tex = -1;
    for (auto& kv : C.textures.items) max_tex = std::max(max_tex, kv.first);
    for (int i = 0; i < lc; i++) {
        auto it = C.lights.items.find(d.light_ids[i]);
        if (it == C.lights.items.end()) continue;
        to_light(L[i], *it->second);
        valid[i] = 1;
    }
    /* sphere lights with a rigid transform: the inner ball of the shadow
       rays' occlusion early-out (intersects_light) */
    for (int i = 0; i < lc; i++) {
        erd::Light& l = L[i];
        l.inner_r2 = -1.0f;
        if (!valid[i] || l.type != ER_SHAPE_SPHERE || !(l.outer_radius > 0.0f)) continue;
        /* the exact test maps the ray with InvTM: the sphere is centred where
           InvTM sends a point to the origin, c = -R^T t for InvTM = (R, t) */
        bool rigid = true;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                double d = 0.0;
                for (int k = 0; k < 3; k++) d += (double)l.inv_tm[k][r] * (double)l.inv_tm[k][c];
                if (std::fabs(d - (r == c ? 1.0 : 0.0)) > 1e-5) rigid = false;
            }
        if (!rigid) continue;
        for (int k = 0; k < 3; k++) {
            double c = 0.0;
            for (int r = 0; r < 3; r++) c -= (double)l.inv_tm[r][k] * (double)l.inv_tm[r][3];
            l.inner_c[k] = (float)c;
        }
        const double ri = 0.9 * (double)l.outer_radius;
        l.inner_r2 = (float)(ri * ri);
    }
    /* lights whose texture is uniform (or unbound: black) get its value here,
       as EvaluateTexture computes it: colour * OutputLevel in float
       (Source/textures.h:63-111) */
    for (int i = 0; i < lc; i++) {
        if (!valid[i]) continue;
        erd::Light& l = L[i];
        l.tex_const = 0;
        auto tt = C.textures.items.find(l.texture_id);
        if (l.texture_id < 0 || tt == C.textures.items.end()) {
            l.tex_const = 1;
            l.tex_rgb[0] = l.tex_rgb[1] = l.tex_rgb[2] = 0.0f;
        } else if (tt->second->type == ER_TEXTURE_PROCEDURAL && tt->second->procedural.type == ER_PROCEDURAL_UNIFORM) {
            const volatile float lvl = tt->second->output_level;
            l.tex_const = 1;
            for (int c = 0; c < 3; c++) {
                const volatile float u = tt->second->procedural.uniform_color[c];
                l.tex_rgb[c] = u * lvl;
            }
        }
    }
    std::vector<int> lids((size_t)std::max(lc, 1), -1);
    for (int i = 0; i < lc; i++) lids[i] = d.light_ids[i];
    ER_CUDA(t.lights.ensure(L.size()));
    ER_CUDA(t.light_valid.ensure(valid.size()));
    ER_CUDA(t.light_ids.ensure(lids.size()));
    ER_CUDA(cudaMemcpyAsync(t.lights.p, L.data(), L.size() * sizeof(erd::Light), cudaMemcpyHostToDevice, st));
    ER_CUDA(cudaMemcpyAsync(t.light_valid.p, valid.data(), valid.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    ER_CUDA(cudaMemcpyAsync(t.light_ids.p, lids.data(), lids.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    P.light_count = lc;
    P.lights = t.lights.p;
    P.light_valid = t.light_valid.p;
    P.light_ids = t.light_ids.p;
    /* surface objects: IntersectObjects reads gpObjects[i] for i below
       ObjectIDs.Count (Source/objects.h:45-62), i.e. the first Count bound
       objects in bind-list (ID) order */
    std::vector<erd::Object> O;
    for (auto& kv : C.objects.items) {
        if ((int)O.size() >= d.object_count) break;
        erd::Object o;
        memset(&o, 0, sizeof(o));
        to_shape(o.shape, kv.second->shape);
        o.diffuse_texture_id = kv.second->diffuse_texture_id;
        o.specular_texture_id = kv.second->specular_texture_id;
        o.glossiness_texture_id = kv.second->glossiness_texture_id;
        O.push_back(o);
    }
    P.object_count = (int)O.size();
    if (!O.empty()) {
        ER_CUDA(t.objects.ensure(O.size()));
        ER_CUDA(cudaMemcpyAsync(t.objects.p, O.data(), O.size() * sizeof(erd::Object), cudaMemcpyHostToDevice, st));
        P.objects = t.objects.p;
    }
    /* clipping objects named by ClippingObjectIDs (Source/ertracer.h:100-116);
       IDs that name no bound clipping object are skipped */
    std::vector<erd::Clip> K;
    const int cc = std::min(std::max(d.clipping_object_count, 0), ER_MAX_INDICES);
    for (int i = 0; i < cc; i++) {
        auto it = C.clipping.items.find(d.clipping_object_ids[i]);
        if (d.clipping_object_ids[i] < 0 || it == C.clipping.items.end()) continue;
        erd::Clip k;
        memset(&k, 0, sizeof(k));
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) k.inv_tm[r][c] = it->second->shape.inv_tm[r][c];
        k.type = it->second->shape.type;
        for (int c = 0; c < 3; c++) k.size[c] = it->second->shape.size[c];
        k.outer_radius = it->second->shape.outer_radius;
        k.invert = it->second->invert ? 1 : 0;
        K.push_back(k);
    }
    P.clip_count = (int)K.size();
    if (!K.empty()) {
        ER_CUDA(t.clips.ensure(K.size()));
        ER_CUDA(cudaMemcpyAsync(t.clips.p, K.data(), K.size() * sizeof(erd::Clip), cudaMemcpyHostToDevice, st));
        P.clips = t.clips.p;
    }
    P.box_empty = v.normalize ? 0 : 1;
    /* textures indexed by texture ID; unbound IDs evaluate to black */
    const int ntex = max_tex + 1;
    std::vector<erd::Texture> T((size_t)std::max(ntex, 1));
    for (auto& tx : T) { memset(&tx, 0, sizeof(tx)); tx.type = -1; tx.output_level = 0.0f; }
    for (auto& kv : C.textures.items) to_texture(T[kv.first], *kv.second);
    ER_CUDA(t.textures.ensure(T.size()));
    ER_CUDA(cudaMemcpyAsync(t.textures.p, T.data(), T.size() * sizeof(erd::Texture), cudaMemcpyHostToDevice, st));
    P.textures = t.textures.p;
    P.n_textures = ntex;
    /* bitmaps indexed by bitmap ID (ErTexture::BitmapID); unbound IDs read black */
    int max_bmp = -1;
    for (auto& kv : C.bitmaps.items) max_bmp = std::max(max_bmp, kv.first);
    P.n_bitmaps = max_bmp + 1;
    P.bitmaps = nullptr;
    if (P.n_bitmaps > 0) {
        std::vector<erd::Bitmap> B((size_t)P.n_bitmaps);
        for (auto& b : B) { b.pixels = nullptr; b.res[0] = b.res[1] = 0; }
        for (auto& kv : C.bitmaps.items) {
            erd::Bitmap& b = B[(size_t)kv.first];
            b.pixels = kv.second->pixels.p;
            b.res[0] = kv.second->res[0];
            b.res[1] = kv.second->res[1];
        }
        ER_CUDA(t.bitmaps.ensure(B.size()));
        ER_CUDA(cudaMemcpyAsync(t.bitmaps.p, B.data(), B.size() * sizeof(erd::Bitmap), cudaMemcpyHostToDevice, st));
        P.bitmaps = t.bitmaps.p;
    }
    P.tfs = t.tfs.p;
    ER_CUDA(t.err.ensure(1));
    P.err = t.err.p;
    /* the host copies above read stack vectors: finish them before returning */
    ER_CUDA(cudaStreamSynchronize(st));
    t.P = P;
    t.built = true;
    t.built_version = C.version;
    static uint64_t serial = 0;
    t.build_serial = ++serial;
    return ER_OK;
}

er_status check_device_error(TracerItem& t)
{
    if (!t.err.p) return ER_OK;
    int e = 0;
    ER_CUDA(cudaMemcpyAsync(&e, t.err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    if (e) {
        ER_CUDA(cudaMemsetAsync(t.err.p, 0, sizeof(int), ctx().stream));
        return fail(ER_ERR_TIMEOUT, "a fixed-step march exceeded its step budget (step below the float resolution of the ray parameter)");
    }
    return ER_OK;
}

TracerItem* find_tracer(int id)
{
    auto it = ctx().tracers.items.find(id);
    return (id < 0 || it == ctx().tracers.items.end()) ? nullptr : it->second.get();
}

BilateralTables bilateral_tables(const er_render_settings& s)
{
    BilateralTables T;
    memset(&T, 0, sizeof(T));
    int r = s.bilateral_radius;
    r = r < 0 ? 0 : (r > 127 ? 127 : r);
    T.radius = r;
    const float sd = s.bilateral_sigma_d > 0.0f ? s.bilateral_sigma_d : 1.0f;
    const float sr = s.bilateral_sigma_r > 0.0f ? s.bilateral_sigma_r : 1.0f;
    for (int k = -r; k <= r; k++) T.spatial[r + k] = er_expf(-((float)(k * k)) / (2.0f * sd * sd));
    for (int d = 0; d < 256; d++) T.range[d] = er_expf(-((float)(d * d)) / (2.0f * sr * sr));
    return T;
}

/* multi-sample transport: the wavefront stages (default) or the one-kernel path */
er_status trace_sum(TracerItem& t, int spp, uint32_t view, uint32_t first, float4* sum, int accumulate, cudaStream_t s)
{
    if (t.d.settings.engine == 1) {
        ER_CUDA(er_launch_trace_sum(t.P, spp, view, first, sum, accumulate, s));
        return ER_OK;
    }
    const int npix = t.W * t.H;
    WavefrontPlan plan;
    er_wavefront_plan(&npix, &spp, 1, kWindowCap, plan);
    WavefrontBuffers B;
    ER_CUDA(t.wf.ensure(plan, B));
    B.tune_primary = t.d.settings.tune_primary > 0 ? t.d.settings.tune_primary : 4;
    B.tune_shadow = t.d.settings.tune_shadow > 0 ? t.d.settings.tune_shadow : 4;
    B.tune_shade = t.d.settings.tune_shade > 0 ? t.d.settings.tune_shade : 2;
    B.objects = t.P.object_count > 0;
    persistent_stages(t.d.settings.tune_stages, t.P.free_flight == ER_FREE_FLIGHT_DELTA, B);
    ER_CUDA(t.wf.ensure_sorted(plan, mixes_shaders(t.P), B));
    WfView V;
    memset(&V, 0, sizeof(V));
    V.P = t.P;
    V.view_id = view;
    V.first = first;
    V.spp = spp;
    V.accumulate = accumulate;
    V.sum = sum;
    ER_CUDA(er_launch_wavefront_one(V, plan, B, s));
    return ER_OK;
}

er_status finish_display(TracerItem& t)
{
    if (t.d.settings.bilateral) {
        const BilateralTables T = bilateral_tables(t.d.settings);
        ER_CUDA(er_launch_bilateral(t.display.p, t.display_tmp.p, t.display_filtered.p, t.W, t.H, T, ctx().stream));
    }
    return ER_OK;
}

er_status batch_enqueue(BatchItem& b, cudaStream_t s);

/* builds the batch's tracers, uploads its view and segment tables, sizes its
   queues and, for ER_BATCH_GRAPH, captures one launch as a CUDA graph */
er_status batch_plan(BatchItem& b)
{
    Context& C = ctx();
    const int n = (int)b.views.size();
    b.drop_graph();
    b.planned = false;
    b.host_views.assign((size_t)n, WfView());
    std::vector<int> npix((size_t)n), spp((size_t)n);
    b.max_w = b.max_h = 0;
    b.any_display = false;
    for (int v = 0; v < n; v++) {
        const er_batch_view& bv = b.views[(size_t)v];
        TracerItem* t = find_tracer(bv.tracer_id);
        if (!t) return fail(ER_ERR_INVALID_ID, "batch view %d: resource item with ID:%d does not exist", v, bv.tracer_id);
        er_status st = build(*t);
        if (st != ER_OK) return st;
        WfView& V = b.host_views[(size_t)v];
        memset(&V, 0, sizeof(V));
        V.P = t->P;
        int W = t->W, H = t->H;
        if (bv.camera) {
            const er_camera_desc& c = *bv.camera;
            if (c.film_size[0] <= 0 || c.film_size[1] <= 0 || c.film_size[0] > 32768 || c.film_size[1] > 32768)
                return fail(ER_ERR_INVALID_ARGUMENT, "batch view %d: film size %d x %d out of range", v, c.film_size[0], c.film_size[1]);
            if (!bv.d_sum_xyza || bv.display)
                return fail(ER_ERR_INVALID_ARGUMENT, "batch view %d: a camera override needs its own sum buffer and no display", v);
            camera_frame(c, V.P);
            W = c.film_size[0];
            H = c.film_size[1];
        }
        V.view_id = bv.view;
        V.first = bv.first_sample;
        V.spp = bv.spp;
        V.accumulate = bv.accumulate;
        V.sum = bv.d_sum_xyza ? (float4*)bv.d_sum_xyza : t->sum.p;
        V.display = bv.display ? 1 : 0;
        V.filter = t->d.settings.frame_filter >= 0 ? 1 : 0;
        V.exposure = t->d.camera.exposure;
        V.running = t->running.p;
        V.rgba = t->display.p;
        npix[(size_t)v] = W * H;
        spp[(size_t)v] = bv.spp;
        b.max_w = std::max(b.max_w, W);
        b.max_h = std::max(b.max_h, H);
        b.any_display = b.any_display || V.display;
    }
    for (int v = 0; v < n; v++)
        for (int u = 0; u < v; u++)
            if (b.host_views[(size_t)v].sum == b.host_views[(size_t)u].sum)
                return fail(ER_ERR_INVALID_ARGUMENT, "batch views %d and %d share a sum buffer", u, v);
    er_wavefront_plan(npix.data(), spp.data(), n, b.window_cap, b.plan);
    ER_CUDA(b.wf.ensure(b.plan, b.B));
    ER_CUDA(b.d_views.ensure((size_t)n));
    ER_CUDA(b.d_segs.ensure(b.plan.segs.size()));
    cudaStream_t st = C.stream;
    ER_CUDA(cudaMemcpyAsync(b.d_views.p, b.host_views.data(), (size_t)n * sizeof(WfView), cudaMemcpyHostToDevice, st));
    ER_CUDA(cudaMemcpyAsync(b.d_segs.p, b.plan.segs.data(), b.plan.segs.size() * sizeof(WfSegment), cudaMemcpyHostToDevice, st));
    ER_CUDA(cudaStreamSynchronize(st));
    if (!b.tune_explicit) {
        const er_render_settings& s0 = find_tracer(b.views[0].tracer_id)->d.settings;
        b.tune_primary = s0.tune_primary > 0 ? s0.tune_primary : 4;
        b.tune_shadow = s0.tune_shadow > 0 ? s0.tune_shadow : 4;
        b.tune_shade = s0.tune_shade > 0 ? s0.tune_shade : 2;
    }
    if (!b.stages_explicit) b.tune_stages = find_tracer(b.views[0].tracer_id)->d.settings.tune_stages;
    b.B.tune_primary = b.tune_primary;
    b.B.tune_shadow = b.tune_shadow;
    b.B.tune_shade = b.tune_shade;
    b.B.objects = 0;
    bool all_delta = true, mixed = false;
    for (const WfView& hv : b.host_views) {
        b.B.objects |= hv.P.object_count > 0;
        all_delta = all_delta && hv.P.free_flight == ER_FREE_FLIGHT_DELTA;
        mixed = mixed || mixes_shaders(hv.P);
    }
    persistent_stages(b.tune_stages, all_delta, b.B);
    ER_CUDA(b.wf.ensure_sorted(b.plan, mixed, b.B));
    if (b.flags & ER_BATCH_GRAPH) {
        if (!b.capture_stream) ER_CUDA(cudaStreamCreateWithFlags(&b.capture_stream, cudaStreamNonBlocking));
        ER_CUDA(cudaStreamBeginCapture(b.capture_stream, cudaStreamCaptureModeThreadLocal));
        er_status rs = batch_enqueue(b, b.capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b.capture_stream, &g);
        if (rs != ER_OK) {
            if (g) cudaGraphDestroy(g);
            return rs;
        }
        ER_CUDA(ce);
        b.graph = g;
        ER_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
    }
    b.planned = true;
    b.planned_version = C.version;
    return ER_OK;
}

/* the launch sequence of a batch: wavefront windows, display pass, bilateral */
er_status batch_enqueue(BatchItem& b, cudaStream_t s)
{
    ER_CUDA(er_launch_wavefront_batch(b.d_views.p, b.d_segs.p, b.plan, b.B, s));
    if (b.any_display) {
        ER_CUDA(er_launch_post_batch(b.d_views.p, (int)b.views.size(), b.max_w, b.max_h, s));
        for (const er_batch_view& bv : b.views) {
            if (!bv.display) continue;
            TracerItem* t = find_tracer(bv.tracer_id);
            if (t && t->d.settings.bilateral) {
                const BilateralTables T = bilateral_tables(t->d.settings);
                ER_CUDA(er_launch_bilateral(t->display.p, t->display_tmp.p, t->display_filtered.p, t->W, t->H, T, s));
            }
        }
    }
    return ER_OK;
}

BatchItem* find_batch(int id)
{
    auto it = ctx().batches.items.find(id);
    return (id < 0 || it == ctx().batches.items.end()) ? nullptr : it->second.get();
}

/* ---- autotuner ---- */

std::string tune_cache_path()
{
    const char* e = getenv("ER_TUNE_CACHE");
    if (e && *e) return std::string(e);
    const char* home = getenv("HOME");
    if (!home || !*home) return std::string();
    return std::string(home) + "/.cache/exposurerender_gb300/autotune.txt";
}

/* device, volume content and every setting that changes the work of a sample */
uint64_t tune_key(const TracerItem& t, const VolumeItem& v, int probe_spp)
{
    cudaDeviceProp prop;
    memset(&prop, 0, sizeof(prop));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    uint64_t h = fnv1a(kFnvBasis, prop.name, strnlen(prop.name, sizeof(prop.name)));
    h = fnv1a(h, &prop.multiProcessorCount, sizeof(int));
    h = fnv1a(h, &v.signature, sizeof(v.signature));
    h = fnv1a(h, v.spacing, sizeof(v.spacing));
    er_render_settings s = t.d.settings;
    s.majorant_brick = 0;
    s.tune_primary = s.tune_shadow = s.tune_shade = 0;
    s.tune_stages = 0;
    s.seed = 0;
    s.bilateral = 0;
    s.bilateral_radius = 0;
    s.bilateral_sigma_d = s.bilateral_sigma_r = 0.0f;
    s.frame_filter = 0;
    h = fnv1a(h, &s, sizeof(s));
    h = fnv1a(h, &t.d.opacity, sizeof(t.d.opacity));
    h = fnv1a(h, &t.d.glossiness, sizeof(t.d.glossiness));
    h = fnv1a(h, t.d.camera.film_size, sizeof(t.d.camera.film_size));
    h = fnv1a(h, &t.d.light_count, sizeof(t.d.light_count));
    h = fnv1a(h, &probe_spp, sizeof(probe_spp));
    return h;
}

bool tune_cache_lookup(uint64_t key, er_tune_result& r)
{
    const std::string path = tune_cache_path();
    if (path.empty() || path == "off") return false;
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    bool found = false;
    char line[256];
    while (fgets(line, sizeof(line), f)) {
        unsigned long long k = 0;
        int b = 0, p = 0, sh = 0, sd = 0, pt = 0;
        float m = 0.0f;
        /* lines carry the persistent-lane choice after the throughput */
        if (sscanf(line, "%llx %d %d %d %d %f %d", &k, &b, &p, &sh, &sd, &m, &pt) == 7 && (uint64_t)k == key) {
            r.majorant_brick = b;
            r.tune_primary = p;
            r.tune_shadow = sh;
            r.tune_shade = sd;
            r.msamples_per_s = m;
            r.tune_stages = pt;
            found = true;          /* the last entry for a key wins */
        }
    }
    fclose(f);
    return found;
}

void tune_cache_store(uint64_t key, const er_tune_result& r)
{
    const std::string path = tune_cache_path();
    if (path.empty() || path == "off") return;
    /* create the parent directories */
    for (size_t i = 1; i < path.size(); i++)
        if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
    FILE* f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%016llx %d %d %d %d %.3f %d\n", (unsigned long long)key, r.majorant_brick, r.tune_primary, r.tune_shadow, r.tune_shade,
            r.msamples_per_s, r.tune_stages);
    fclose(f);
}

/* Msamples/s of one probe render with the tracer's current settings */
er_status time_probe(TracerItem& t, int spp, float* msps)
{
    t.built = false;
    er_status st = build(t);
    if (st != ER_OK) return st;
    const size_t npix = (size_t)t.W * t.H;
    /* at least 2^21 samples per probe: a smaller launch does not fill the
       persistent stages' resident wave and misranks them */
    const size_t min_samples = (size_t)1 << 21;
    if ((size_t)spp * npix < min_samples) spp = (int)std::min<size_t>((min_samples + npix - 1) / npix, 4096);
    ER_CUDA(t.tune_sum.ensure(npix));
    cudaStream_t s = ctx().stream;
    st = trace_sum(t, spp, 0x7fffffffu, 0u, t.tune_sum.p, 0, s);
    if (st != ER_OK) return st;
    cudaEvent_t a = nullptr, b = nullptr;
    ER_CUDA(cudaEventCreate(&a));
    ER_CUDA(cudaEventCreate(&b));
    ER_CUDA(cudaEventRecord(a, s));
    st = trace_sum(t, spp, 0x7fffffffu, (uint32_t)spp, t.tune_sum.p, 0, s);
    ER_CUDA(cudaEventRecord(b, s));
    ER_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != ER_OK) return st;
    *msps = ms > 0.0f ? (float)((double)npix * spp / (ms * 1e3)) : 0.0f;
    return check_device_error(t);
}

}  // namespace

/* last-error text for entry points implemented in other translation units */
void er_internal_set_error(const char* message) { g_last_error = message ? message : ""; }

/* ====================================================================== */
/* C ABI                                                                    */
/* ====================================================================== */

#define ER_LOCK std::lock_guard<std::recursive_mutex> lock_(ctx().m)

extern "C" {

ER_API int er_abi_version(void) { return ER_ABI_VERSION; }

ER_API const char* er_last_error_message(void) { return g_last_error.c_str(); }

ER_API er_status er_set_device(int device)
{
    ER_LOCK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return fail(ER_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) return fail(ER_ERR_INVALID_ARGUMENT, "device %d out of range (%d devices)", device, n);
    ER_CUDA(cudaSetDevice(device));
    ctx().device = device;
    return ER_OK;
}

ER_API er_status er_set_stream(void* stream)
{
    ER_LOCK;
    ctx().stream = (cudaStream_t)stream;
    return ER_OK;
}

ER_API er_status er_synchronize(void)
{
    ER_LOCK;
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    for (auto& kv : ctx().tracers.items) {
        er_status s = check_device_error(*kv.second);
        if (s != ER_OK) return s;
    }
    return ER_OK;
}

ER_API er_status er_reset(void)
{
    ER_LOCK;
    Context& C = ctx();
    cudaStreamSynchronize(C.stream);
    cudaDeviceSynchronize();
    C.batches.items.clear();
    C.batches.counter = 0;
    C.tracers.items.clear();
    C.volumes.items.clear();
    C.lights.items.clear();
    C.textures.items.clear();
    C.bitmaps.items.clear();
    C.objects.items.clear();
    C.clipping.items.clear();
    /* a reset library starts numbering from 0 again, like a fresh process */
    C.tracers.counter = C.volumes.counter = C.lights.counter = C.textures.counter = 0;
    C.bitmaps.counter = C.objects.counter = C.clipping.counter = 0;
    C.version++;
    return ER_OK;
}

ER_API void er_default_render_settings(er_render_settings* s)
{
    if (!s) return;
    memset(s, 0, sizeof(*s));
    s->step_factor_primary = 0.1f;
    s->step_factor_shadow = 0.1f;
    s->shadows = 1;
    s->max_shadow_distance = 1.0f;
    s->shading_type = 0;
    s->density_scale = 100.0f;
    s->opacity_modulated = 1;
    s->gradient_computation = 1;
    s->gradient_threshold = 0.5f;
    s->gradient_factor = 0.5f;
    s->volume_ior = 15.0f;
    s->frame_filter = 1;
    s->bilateral_radius = 2;
    s->bilateral_sigma_d = 1.5f;
    s->bilateral_sigma_r = 20.0f;
    s->seed = 1u;
    s->majorant_brick = 8;
}

ER_API void er_plf_init(er_plf* p)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->node_range[0] = FLT_MAX;
    p->node_range[1] = FLT_MIN;
}

ER_API void er_plf_add_node(er_plf* p, float position, float value)
{
    if (!p) return;
    if (p->count + 1 >= ER_MAX_TF_NODES) return;
    p->position[p->count] = position;
    p->value[p->count] = value;
    if (position < p->node_range[0]) p->node_range[0] = position;
    if (position > p->node_range[1]) p->node_range[1] = position;
    p->count++;
}

/* ---- bind lists ---- */

/* Copies the box [lo, lo + n) of voxels (x fastest, packed) from host or
   device memory into a bound volume, refreshes the corner quads it changes
   (one voxel below the box in x and y as well) and returns the largest voxel
   of the refreshed box.  Synchronous. */
er_status upload_box(VolumeItem& v, const int lo[3], const int n[3], const uint16_t* src, cudaMemcpyKind kind, cudaStream_t s,
                     unsigned int* box_max)
{
    cudaMemcpy3DParms p;
    memset(&p, 0, sizeof(p));
    p.srcPtr = make_cudaPitchedPtr((void*)src, (size_t)n[0] * sizeof(uint16_t), (size_t)n[0], (size_t)n[1]);
    p.dstPtr = make_cudaPitchedPtr(v.vox.p, (size_t)v.res[0] * sizeof(uint16_t), (size_t)v.res[0], (size_t)v.res[1]);
    p.dstPos = make_cudaPos((size_t)lo[0] * sizeof(uint16_t), (size_t)lo[1], (size_t)lo[2]);
    p.extent = make_cudaExtent((size_t)n[0] * sizeof(uint16_t), (size_t)n[1], (size_t)n[2]);
    p.kind = kind;
    ER_CUDA(cudaMemcpy3DAsync(&p, s));
    int qlo[3] = { lo[0] > 0 ? lo[0] - 1 : 0, lo[1] > 0 ? lo[1] - 1 : 0, lo[2] };
    int qn[3] = { n[0] + (lo[0] - qlo[0]), n[1] + (lo[1] - qlo[1]), n[2] };
    ER_CUDA(v.box_max.ensure(1));
    ER_CUDA(cudaMemsetAsync(v.box_max.p, 0, sizeof(unsigned int), s));
    ER_CUDA(er_launch_box_quads_max(v.vox.p, v.res, qlo, qn, v.quad.p, v.qb_nbx, v.qb_slab, v.box_max.p, s));
    ER_CUDA(cudaMemcpyAsync(box_max, v.box_max.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    ER_CUDA(cudaStreamSynchronize(s));
    return ER_OK;
}

ER_API er_status er_bind_volume(const er_volume_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d || !d->voxels) return fail(ER_ERR_INVALID_ARGUMENT, "volume descriptor or voxel pointer is NULL");
    for (int i = 0; i < 3; i++)
        if (d->resolution[i] <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "volume resolution must be positive");
    /* a zero, negative or non-finite spacing gives a degenerate box whose
       fixed-step marches take steps of zero or NaN length */
    for (int i = 0; i < 3; i++)
        if (!(d->spacing[i] > 0.0f) || !std::isfinite(d->spacing[i]))
            return fail(ER_ERR_INVALID_ARGUMENT, "volume spacing must be finite and positive");
    /* normalize_size = 0 is accepted: as in the reference, Volume's copy then
       scales the spacing by 0 (Source/volume.h:106-117), the volume has no
       extent and renders show only the lights and objects (box_empty) */
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.volumes, id, &is_new);
    if (st != ER_OK) return st;
    /* a rebind of an ID at the same resolution refills its buffers in place
       (after the work queued on them); otherwise a new item is made */
    std::unique_ptr<VolumeItem> fresh;
    VolumeItem* v = nullptr;
    if (!is_new) {
        VolumeItem& old = *C.volumes.items[*id];
        if (old.res[0] == d->resolution[0] && old.res[1] == d->resolution[1] && old.res[2] == d->resolution[2]) {
            ER_CUDA(cudaStreamSynchronize(C.stream));
            v = &old;
        }
    }
    const size_t n = (size_t)d->resolution[0] * d->resolution[1] * d->resolution[2];
    if (!v) {
        fresh.reset(new VolumeItem());
        v = fresh.get();
        ER_CUDA(v->vox.ensure(n));
        /* corner quads for the transport's lookups, x fastest or (environment
           ER_QUAD_LAYOUT=bricked) in 8^3 bricks; without room for them the
           kernels read the plain voxels (same values, more loads) */
        const char* layout = getenv("ER_QUAD_LAYOUT");
        size_t nq = n;
        if (layout && strcmp(layout, "bricked") == 0) {
            const int nb[3] = { (d->resolution[0] + 7) / 8, (d->resolution[1] + 7) / 8, (d->resolution[2] + 7) / 8 };
            v->qb_nbx = nb[0];
            v->qb_slab = (unsigned long long)nb[0] * (unsigned long long)nb[1] * 512ull;
            nq = (size_t)v->qb_slab * (size_t)nb[2];
        }
        if (v->quad.ensure(nq) != cudaSuccess) cudaGetLastError();
    }
    for (int i = 0; i < 3; i++) { v->res[i] = d->resolution[i]; v->spacing[i] = d->spacing[i]; }
    v->normalize = d->normalize_size;
    v->gm_max = -1.0f;
    /* content signature of the tuning cache: every 61st voxel */
    uint64_t sig = fnv1a(kFnvBasis, d->resolution, sizeof(d->resolution));
    for (size_t i = 0; i < n; i += 61) sig = fnv1a(sig, &d->voxels[i], sizeof(uint16_t));
    v->signature = sig;
    const int lo[3] = { 0, 0, 0 };
    unsigned int vmax = 0;
    er_status us = upload_box(*v, lo, d->resolution, d->voxels, cudaMemcpyHostToDevice, C.stream, &vmax);
    if (us != ER_OK) return us;
    v->vmax = (uint16_t)vmax;
    if (fresh) C.volumes.items[*id] = std::move(fresh);
    C.version++;
    return ER_OK;
}

/* shared by the host and device variants of the region update */
static er_status update_volume_region(int32_t id, const int32_t* offset, const int32_t* size, const uint16_t* voxels,
                                      cudaMemcpyKind kind, cudaStream_t s)
{
    Context& C = ctx();
    auto it = C.volumes.items.find(id);
    if (id < 0 || it == C.volumes.items.end()) return fail(ER_ERR_INVALID_ID, "volume ID:%d does not exist", id);
    if (!offset || !size || !voxels) return fail(ER_ERR_INVALID_ARGUMENT, "offset, size or voxel pointer is NULL");
    VolumeItem& v = *it->second;
    for (int i = 0; i < 3; i++) {
        if (offset[i] < 0 || size[i] <= 0 || (int64_t)offset[i] + size[i] > v.res[i])
            return fail(ER_ERR_INVALID_ARGUMENT, "region [%d, %d) on axis %d is outside the volume's [0, %d)", offset[i],
                        offset[i] + size[i], i, v.res[i]);
    }
    /* the volume may be read by queued work: the edit follows it */
    ER_CUDA(cudaStreamSynchronize(C.stream));
    unsigned int bmax = 0;
    er_status us = upload_box(v, offset, size, voxels, kind, s, &bmax);
    if (us != ER_OK) return us;
    if (bmax > v.vmax) v.vmax = (uint16_t)bmax;
    v.gm_max = -1.0f;
    /* tuning-cache signature: the edit's box, its contents (every 61st of
       the host voxels, as er_bind_volume samples a whole volume) and, for
       device voxels the host cannot read, the volume's edit count */
    v.signature = fnv1a(v.signature, offset, 3 * sizeof(int32_t));
    v.signature = fnv1a(v.signature, size, 3 * sizeof(int32_t));
    const size_t n = (size_t)size[0] * size[1] * size[2];
    if (kind == cudaMemcpyHostToDevice) {
        for (size_t i = 0; i < n; i += 61) v.signature = fnv1a(v.signature, &voxels[i], sizeof(uint16_t));
    } else {
        v.edits++;
        v.signature = fnv1a(v.signature, &v.edits, sizeof(v.edits));
    }
    C.version++;
    return ER_OK;
}

ER_API er_status er_update_volume_region(int32_t volume_id, const int32_t offset[3], const int32_t size[3], const uint16_t* voxels)
{
    ER_LOCK;
    return update_volume_region(volume_id, offset, size, voxels, cudaMemcpyHostToDevice, ctx().stream);
}

ER_API er_status er_update_volume_region_device(int32_t volume_id, const int32_t offset[3], const int32_t size[3],
                                                const uint16_t* d_voxels, void* stream)
{
    ER_LOCK;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx().stream;
    return update_volume_region(volume_id, offset, size, d_voxels, cudaMemcpyDeviceToDevice, s);
}

ER_API er_status er_unbind_volume(int32_t id) { ER_LOCK; return unbind(ctx().volumes, id); }

ER_API er_status er_bind_light(const er_light_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d) return fail(ER_ERR_INVALID_ARGUMENT, "light descriptor is NULL");
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.lights, id, &is_new);
    if (st != ER_OK) return st;
    C.lights.items[*id].reset(new er_light_desc(*d));
    C.version++;
    return ER_OK;
}

ER_API er_status er_unbind_light(int32_t id) { ER_LOCK; return unbind(ctx().lights, id); }

ER_API er_status er_bind_texture(const er_texture_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d) return fail(ER_ERR_INVALID_ARGUMENT, "texture descriptor is NULL");
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.textures, id, &is_new);
    if (st != ER_OK) return st;
    C.textures.items[*id].reset(new er_texture_desc(*d));
    C.version++;
    return ER_OK;
}

ER_API er_status er_unbind_texture(int32_t id) { ER_LOCK; return unbind(ctx().textures, id); }

ER_API er_status er_bind_bitmap(const er_bitmap_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d || !d->pixels || d->resolution[0] <= 0 || d->resolution[1] <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid bitmap descriptor");
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.bitmaps, id, &is_new);
    if (st != ER_OK) return st;
    std::unique_ptr<BitmapItem> b(new BitmapItem());
    b->res[0] = d->resolution[0];
    b->res[1] = d->resolution[1];
    const size_t n = (size_t)b->res[0] * b->res[1];
    ER_CUDA(b->pixels.ensure(n));
    ER_CUDA(cudaMemcpy(b->pixels.p, d->pixels, n * 4, cudaMemcpyHostToDevice));
    C.bitmaps.items[*id] = std::move(b);
    C.version++;
    return ER_OK;
}

ER_API er_status er_unbind_bitmap(int32_t id) { ER_LOCK; return unbind(ctx().bitmaps, id); }

ER_API er_status er_bind_object(const er_object_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d) return fail(ER_ERR_INVALID_ARGUMENT, "object descriptor is NULL");
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.objects, id, &is_new);
    if (st != ER_OK) return st;
    C.objects.items[*id].reset(new er_object_desc(*d));
    C.version++;
    return ER_OK;
}

ER_API er_status er_unbind_object(int32_t id) { ER_LOCK; return unbind(ctx().objects, id); }

ER_API er_status er_bind_clipping_object(const er_clipping_object_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d) return fail(ER_ERR_INVALID_ARGUMENT, "clipping object descriptor is NULL");
    Context& C = ctx();
    bool is_new = false;
    er_status st = reserve_id(C.clipping, id, &is_new);
    if (st != ER_OK) return st;
    C.clipping.items[*id].reset(new er_clipping_object_desc(*d));
    C.version++;
    return ER_OK;
}

ER_API er_status er_unbind_clipping_object(int32_t id) { ER_LOCK; return unbind(ctx().clipping, id); }

ER_API er_status er_bind_tracer(const er_tracer_desc* d, int32_t* id)
{
    ER_LOCK;
    if (!d) return fail(ER_ERR_INVALID_ARGUMENT, "tracer descriptor is NULL");
    er_status st = check_settings(*d);
    if (st != ER_OK) return st;
    Context& C = ctx();
    bool is_new = false;
    st = reserve_id(C.tracers, id, &is_new);
    if (st != ER_OK) return st;
    if (is_new) C.tracers.items[*id].reset(new TracerItem());
    TracerItem& t = *C.tracers.items[*id];
    const bool resize = is_new || t.W != d->camera.film_size[0] || t.H != d->camera.film_size[1];
    const bool reseed = is_new || t.d.settings.seed != d->settings.seed;
    t.d = *d;
    t.built = false;
    C.version++;
    if (resize) {
        /* Tracer::operator= resizes the frame buffer (Source/tracer.h:45-52,
           Source/framebuffer.h:45-68): every buffer is reallocated and cleared */
        t.W = d->camera.film_size[0];
        t.H = d->camera.film_size[1];
        const size_t n = (size_t)t.W * t.H;
        ER_CUDA(t.frame.ensure(n));
        ER_CUDA(t.running.ensure(n));
        ER_CUDA(t.sum.ensure(n));
        ER_CUDA(t.display.ensure(n));
        ER_CUDA(t.display_tmp.ensure(n));
        ER_CUDA(t.display_filtered.ensure(n));
        ER_CUDA(t.lanes.ensure(2 * n));
        ER_CUDA(t.err.ensure(1));
        ER_CUDA(cudaMemsetAsync(t.err.p, 0, sizeof(int), C.stream));
        return reset_tracer_buffers(t);
    }
    if (reseed) return init_lanes(t);
    return ER_OK;
}

ER_API er_status er_unbind_tracer(int32_t id) { ER_LOCK; return unbind(ctx().tracers, id); }

/* ---- rendering ---- */

ER_API er_status er_render_estimate(int32_t tracer_id)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    er_status st = build(*t);
    if (st != ER_OK) return st;
    cudaStream_t s = ctx().stream;
    ER_CUDA(er_launch_trace_frame(t->P, t->lanes.p, t->frame.p, s));
    const int filt = t->d.settings.frame_filter >= 0 ? 1 : 0;
    ER_CUDA(er_launch_post_frame(t->frame.p, t->running.p, t->display.p, t->W, t->H, t->no_iterations, t->d.camera.exposure, filt, s));
    st = finish_display(*t);
    if (st != ER_OK) return st;
    t->no_iterations++;
    return ER_OK;
}

ER_API er_status er_render_spp(int32_t tracer_id, int32_t spp)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (spp <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "spp must be positive");
    er_status st = build(*t);
    if (st != ER_OK) return st;
    cudaStream_t s = ctx().stream;
    const uint32_t first = (uint32_t)t->n_samples;
    st = trace_sum(*t, spp, 0u, first, t->sum.p, t->n_samples > 0.0 ? 1 : 0, s);
    if (st != ER_OK) return st;
    t->n_samples += spp;
    const int filt = t->d.settings.frame_filter >= 0 ? 1 : 0;
    ER_CUDA(er_launch_post_mean(t->sum.p, (float)t->n_samples, t->running.p, t->display.p, t->W, t->H, t->d.camera.exposure, filt, s));
    st = finish_display(*t);
    if (st != ER_OK) return st;
    t->no_iterations += spp;
    return ER_OK;
}

ER_API er_status er_reset_accumulation(int32_t tracer_id)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    return reset_tracer_buffers(*t);
}

ER_API er_status er_get_estimate(int32_t tracer_id, uint8_t* rgba)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!rgba) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    const uchar4* src = t->d.settings.bilateral ? t->display_filtered.p : t->display.p;
    ER_CUDA(cudaMemcpyAsync(rgba, src, (size_t)t->W * t->H * 4, cudaMemcpyDeviceToHost, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return check_device_error(*t);
}

ER_API er_status er_get_frame_estimate(int32_t tracer_id, float* xyza)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!xyza) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    ER_CUDA(cudaMemcpyAsync(xyza, t->frame.p, (size_t)t->W * t->H * sizeof(float4), cudaMemcpyDeviceToHost, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return check_device_error(*t);
}

ER_API er_status er_get_running_estimate(int32_t tracer_id, float* xyza)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!xyza) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    ER_CUDA(cudaMemcpyAsync(xyza, t->running.p, (size_t)t->W * t->H * sizeof(float4), cudaMemcpyDeviceToHost, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return check_device_error(*t);
}

ER_API er_status er_get_seeds(int32_t tracer_id, uint32_t* lanes)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!lanes) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    ER_CUDA(cudaMemcpyAsync(lanes, t->lanes.p, (size_t)t->W * t->H * 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return ER_OK;
}

ER_API er_status er_set_seeds(int32_t tracer_id, const uint32_t* lanes)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!lanes) return fail(ER_ERR_INVALID_ARGUMENT, "input pointer is NULL");
    ER_CUDA(cudaMemcpyAsync(t->lanes.p, lanes, (size_t)t->W * t->H * 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx().stream));
    ER_CUDA(cudaStreamSynchronize(ctx().stream));
    return ER_OK;
}

ER_API er_status er_get_film_size(int32_t tracer_id, int32_t* w, int32_t* h)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (w) *w = t->W;
    if (h) *h = t->H;
    return ER_OK;
}

ER_API er_status er_get_no_iterations(int32_t tracer_id, int32_t* no_iterations)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!no_iterations) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    *no_iterations = t->no_iterations;
    return ER_OK;
}

ER_API er_status er_get_auto_focus_distance(int32_t tracer_id, int32_t film_u, int32_t film_v, float* distance)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!distance) return fail(ER_ERR_INVALID_ARGUMENT, "output pointer is NULL");
    er_status st = build(*t);
    if (st != ER_OK) return st;
    if (film_u < 0 || film_v < 0 || film_u >= t->W || film_v >= t->H)
        return fail(ER_ERR_INVALID_ARGUMENT, "film position (%d, %d) outside the %d x %d film", film_u, film_v, t->W, t->H);
    /* the reference seeds its one-thread kernel with rand(); here the lanes
       come from the tracer's seed and the pixel (view ER_AUTOFOCUS_VIEW) */
    uint32_t l0 = 0, l1 = 0;
    er_seed_lanes(t->d.settings.seed, ER_AUTOFOCUS_VIEW, (uint32_t)film_v * (uint32_t)t->W + (uint32_t)film_u, 0u, &l0, &l1);
    ER_CUDA(t->autofocus.ensure(1));
    cudaStream_t s = ctx().stream;
    ER_CUDA(er_launch_autofocus(t->P, film_u, film_v, l0, l1, t->autofocus.p, s));
    ER_CUDA(cudaMemcpyAsync(distance, t->autofocus.p, sizeof(float), cudaMemcpyDeviceToHost, s));
    ER_CUDA(cudaStreamSynchronize(s));
    return check_device_error(*t);
}

/* ---- device-pointer entry points ---- */

ER_API er_status er_trace_sum_device(int32_t tracer_id, int32_t spp, uint32_t view, uint32_t first_sample, float* d_sum,
                                     int32_t accumulate, void* stream)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!d_sum || spp <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid sum buffer or spp");
    er_status st = build(*t);
    if (st != ER_OK) return st;
    return trace_sum(*t, spp, view, first_sample, (float4*)d_sum, accumulate, (cudaStream_t)stream);
}

ER_API er_status er_batch_create(const er_batch_view* views, int32_t n_views, int32_t flags, int32_t window_items,
                                 int32_t* batch_id)
{
    ER_LOCK;
    if (!views || n_views <= 0 || n_views > 65535 || !batch_id) return fail(ER_ERR_INVALID_ARGUMENT, "invalid batch views");
    if (window_items < 0) return fail(ER_ERR_INVALID_ARGUMENT, "window_items must be >= 0");
    for (int v = 0; v < n_views; v++)
        if (views[v].spp <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "batch view %d: spp must be positive", v);
    std::unique_ptr<BatchItem> b(new BatchItem());
    b->views.assign(views, views + n_views);
    /* the batch keeps its own copies of the camera overrides */
    b->cameras.resize((size_t)n_views);
    for (int v = 0; v < n_views; v++) {
        if (!views[v].camera) continue;
        b->cameras[(size_t)v] = *views[v].camera;
        b->views[(size_t)v].camera = &b->cameras[(size_t)v];
    }
    b->flags = flags;
    b->window_cap = window_items > 0 ? (size_t)window_items : kWindowCap;
    const er_status st = batch_plan(*b);
    if (st != ER_OK) return st;
    const int id = ctx().batches.counter++;
    ctx().batches.items[id] = std::move(b);
    *batch_id = id;
    return ER_OK;
}

ER_API er_status er_batch_launch(int32_t batch_id, void* stream)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    if (!b->planned || b->planned_version != ctx().version) {
        const er_status st = batch_plan(*b);
        if (st != ER_OK) return st;
    }
    if (b->exec) {
        ER_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
        return ER_OK;
    }
    return batch_enqueue(*b, (cudaStream_t)stream);
}

ER_API er_status er_batch_advance(int32_t batch_id, uint32_t samples, void* stream)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    for (size_t v = 0; v < b->views.size(); v++) {
        b->views[v].first_sample += samples;
        b->host_views[v].first += samples;
    }
    /* a pageable source is staged before the call returns */
    ER_CUDA(cudaMemcpyAsync(b->d_views.p, b->host_views.data(), b->host_views.size() * sizeof(WfView), cudaMemcpyHostToDevice,
                            (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_batch_set_tuning(int32_t batch_id, int32_t tune_primary, int32_t tune_shadow)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    auto valid = [](int v) { return v == 0 || v == 2 || v == 3 || v == 4 || v == 6 || v == 8; };
    if (!valid(tune_primary) || !valid(tune_shadow)) return fail(ER_ERR_INVALID_ARGUMENT, "tuning values must be 0, 2, 3, 4, 6 or 8");
    if (tune_primary) b->tune_primary = tune_primary;
    if (tune_shadow) b->tune_shadow = tune_shadow;
    b->tune_explicit = true;
    b->planned = false;   /* re-captured at the next launch */
    return ER_OK;
}

ER_API er_status er_batch_set_stages(int32_t batch_id, int32_t tune_stages)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    if (tune_stages < 0 || tune_stages > (3 | ER_TUNE_NO_SKIP))
        return fail(ER_ERR_INVALID_ARGUMENT, "tune_stages %d is not ER_PERSISTENT_* with ER_TUNE_NO_SKIP_* bits", tune_stages);
    b->tune_stages = tune_stages;
    b->stages_explicit = true;
    b->planned = false;   /* re-captured at the next launch */
    return ER_OK;
}

ER_API er_status er_batch_autotune(int32_t batch_id, void* stream, int32_t* tune_stages, float* msamples_per_s)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    double samples = 0.0;
    for (const er_batch_view& v : b->views) {
        const TracerItem* t = find_tracer(v.tracer_id);
        const int W = v.camera ? v.camera->film_size[0] : (t ? t->W : 0);
        const int H = v.camera ? v.camera->film_size[1] : (t ? t->H : 0);
        samples += (double)W * H * v.spp;
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t a = nullptr, e = nullptr;
    ER_CUDA(cudaEventCreate(&a));
    ER_CUDA(cudaEventCreate(&e));
    /* one timed launch of the whole batch in its current configuration
       (planned and captured first, outside the timed region) */
    auto time_batch = [&](float* rate) -> er_status {
        if (!b->planned || b->planned_version != ctx().version) {
            const er_status ps = batch_plan(*b);
            if (ps != ER_OK) return ps;
        }
        ER_CUDA(cudaEventRecord(a, st));
        const er_status ls = er_batch_launch(batch_id, stream);
        if (ls != ER_OK) return ls;
        ER_CUDA(cudaEventRecord(e, st));
        ER_CUDA(cudaEventSynchronize(e));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, e);
        *rate = ms > 0.0f ? (float)(samples / (ms * 1e3)) : 0.0f;
        return ER_OK;
    };
    auto done = [&](er_status rs) { cudaEventDestroy(a); cudaEventDestroy(e); return rs; };
    float best_rate = 0.0f;
    er_status rs = time_batch(&best_rate);
    if (rs != ER_OK) return done(rs);
    /* each delta-tracking tracer's majorant brick in turn, on whole launches
       (a brick that helps one view can hurt the others of its volume) */
    std::vector<int32_t> tids;
    for (const er_batch_view& v : b->views) {
        const TracerItem* t = find_tracer(v.tracer_id);
        if (t && t->d.settings.free_flight == ER_FREE_FLIGHT_DELTA && std::find(tids.begin(), tids.end(), v.tracer_id) == tids.end())
            tids.push_back(v.tracer_id);
    }
    for (int32_t tid : tids) {
        TracerItem* t = find_tracer(tid);
        const int cur = t->d.settings.majorant_brick > 0 ? t->d.settings.majorant_brick : 8;
        int best_b = cur;
        for (int bb : {1, 2, 4, 8}) {
            if (bb == cur) continue;
            t->d.settings.majorant_brick = bb;
            t->built = false;
            ctx().version++;
            float r = 0.0f;
            rs = time_batch(&r);
            if (rs != ER_OK) return done(rs);
            if (r > best_rate) { best_rate = r; best_b = bb; }
        }
        t->d.settings.majorant_brick = best_b;
        t->built = false;
        ctx().version++;
    }
    /* then the tracking stages' persistent-lane mode */
    const int candidates[] = {ER_PERSISTENT_BOTH, ER_PERSISTENT_SHADOW, ER_PERSISTENT_NONE, ER_PERSISTENT_PRIMARY};
    int best = b->tune_stages;
    for (int c : candidates) {
        rs = er_batch_set_stages(batch_id, c);
        if (rs != ER_OK) return done(rs);
        float r = 0.0f;
        rs = time_batch(&r);
        if (rs != ER_OK) return done(rs);
        if (r > best_rate) { best_rate = r; best = c; }
    }
    rs = er_batch_set_stages(batch_id, best);
    if (rs != ER_OK) return done(rs);
    /* last the occupancy variants of the tracking stages under that mode */
    const int pairs[][2] = {{4, 4}, {3, 3}, {3, 4}, {4, 3}, {2, 3}, {2, 2}, {6, 4}, {4, 6}, {6, 6}};
    int best_p = b->tune_primary, best_s = b->tune_shadow;
    for (const auto& pr : pairs) {
        if (pr[0] == best_p && pr[1] == best_s) continue;
        rs = er_batch_set_tuning(batch_id, pr[0], pr[1]);
        if (rs != ER_OK) return done(rs);
        float r = 0.0f;
        rs = time_batch(&r);
        if (rs != ER_OK) return done(rs);
        if (r > best_rate) { best_rate = r; best_p = pr[0]; best_s = pr[1]; }
    }
    rs = er_batch_set_tuning(batch_id, best_p, best_s);
    if (rs != ER_OK) return done(rs);
    if (tune_stages) *tune_stages = best;
    if (msamples_per_s) *msamples_per_s = best_rate;
    return done(ER_OK);
}

ER_API er_status er_batch_info(int32_t batch_id, int32_t* n_windows, int32_t* n_segments, int64_t* queue_bytes)
{
    ER_LOCK;
    BatchItem* b = find_batch(batch_id);
    if (!b) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    if (n_windows) *n_windows = (int32_t)b->plan.window_first.size();
    if (n_segments) *n_segments = (int32_t)b->plan.segs.size();
    if (queue_bytes) *queue_bytes = (int64_t)((12 * b->plan.max_items + 2 * (size_t)b->plan.max_npix) * sizeof(float4));
    return ER_OK;
}

ER_API er_status er_batch_destroy(int32_t batch_id)
{
    ER_LOCK;
    auto it = ctx().batches.items.find(batch_id);
    if (batch_id < 0 || it == ctx().batches.items.end()) return fail(ER_ERR_INVALID_ID, "batch with ID:%d does not exist", batch_id);
    ER_CUDA(cudaDeviceSynchronize());
    ctx().batches.items.erase(it);
    return ER_OK;
}

ER_API er_status er_autotune_tracer(int32_t tracer_id, int32_t probe_spp, er_tune_result* result)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (probe_spp <= 0 || probe_spp > 4096) return fail(ER_ERR_INVALID_ARGUMENT, "probe_spp %d out of range [1, 4096]", probe_spp);
    er_status st = build(*t);
    if (st != ER_OK) return st;
    Context& C = ctx();
    const VolumeItem& v = *C.volumes.items.find(t->d.volume_id)->second;
    const uint64_t key = tune_key(*t, v, probe_spp);
    er_tune_result r;
    memset(&r, 0, sizeof(r));
    er_render_settings& s = t->d.settings;
    const er_render_settings saved = s;
    if (tune_cache_lookup(key, r)) {
        r.from_cache = 1;
    } else {
        const bool delta = s.free_flight == ER_FREE_FLIGHT_DELTA;
        const bool wavefront = s.engine != 1;
        s.tune_primary = s.tune_primary > 0 ? s.tune_primary : 4;
        s.tune_shadow = s.tune_shadow > 0 ? s.tune_shadow : 4;
        s.tune_shade = s.tune_shade > 0 ? s.tune_shade : 2;
        r.tune_shade = s.tune_shade;
        r.majorant_brick = s.majorant_brick > 0 ? s.majorant_brick : 8;
        r.tune_primary = s.tune_primary;
        r.tune_shadow = s.tune_shadow;
        r.msamples_per_s = -1.0f;
        /* majorant brick first (the dominant term for delta tracking), then
           the occupancy variants at the best brick */
        const int bricks[] = {1, 2, 4, 8, 16};
        const int base_stages = s.tune_stages & 3;
        r.tune_stages = s.tune_stages;
        for (int b : bricks) {
            if (!delta && b != r.majorant_brick) continue;
            s.majorant_brick = b;
            s.tune_stages = base_stages;
            float m = 0.0f;
            st = time_probe(*t, probe_spp, &m);
            if (st != ER_OK) {
                /* a brick size whose grid does not fit (memory, launch limits) is
                   skipped; a fault that poisons the context ends the sweep */
                if (cudaDeviceSynchronize() != cudaSuccess) { s = saved; t->built = false; return st; }
                cudaGetLastError();
                continue;
            }
            r.candidates++;
            if (m > r.msamples_per_s) { r.msamples_per_s = m; r.majorant_brick = b; r.tune_stages = s.tune_stages; }
        }
        if (r.msamples_per_s < 0.0f) { s = saved; t->built = false; return fail(ER_ERR_CUDA, "no majorant brick size could be timed"); }
        s.majorant_brick = r.majorant_brick;
        s.tune_stages = r.tune_stages;
        if (wavefront) {
            /* occupancy pairs, with persistent-lane tracking stages or not (delta tracking) */
            const int variants[][2] = {{4, 4}, {3, 3}, {3, 4}, {4, 3}, {2, 3}, {3, 2}, {2, 2}, {2, 4}, {6, 4}, {4, 6}, {6, 6}};
            const int modes_delta[] = {ER_PERSISTENT_SHADOW, ER_PERSISTENT_BOTH, ER_PERSISTENT_NONE, ER_PERSISTENT_PRIMARY};
            const int modes_march[] = {ER_PERSISTENT_SHADOW};
            const int* modes = delta ? modes_delta : modes_march;
            const int n_modes = delta ? 4 : 1;
            for (int mi = 0; mi < n_modes; mi++) {
                s.tune_stages = modes[mi];
                for (const auto& vv : variants) {
                    s.tune_primary = vv[0];
                    s.tune_shadow = vv[1];
                    float m = 0.0f;
                    st = time_probe(*t, probe_spp, &m);
                    if (st != ER_OK) { s = saved; t->built = false; return st; }
                    r.candidates++;
                    if (m > r.msamples_per_s) {
                        r.msamples_per_s = m;
                        r.tune_primary = vv[0];
                        r.tune_shadow = vv[1];
                        r.tune_stages = modes[mi];
                    }
                }
            }
            s.tune_primary = r.tune_primary;
            s.tune_shadow = r.tune_shadow;
            s.tune_stages = r.tune_stages;
            const int shades[] = {2, 3, 4, 6};
            for (int sd : shades) {
                s.tune_shade = sd;
                float m = 0.0f;
                st = time_probe(*t, probe_spp, &m);
                if (st != ER_OK) { s = saved; t->built = false; return st; }
                r.candidates++;
                if (m > r.msamples_per_s) { r.msamples_per_s = m; r.tune_shade = sd; }
            }
        }
        tune_cache_store(key, r);
    }
    s.majorant_brick = r.majorant_brick;
    s.tune_primary = r.tune_primary;
    s.tune_shadow = r.tune_shadow;
    s.tune_shade = r.tune_shade;
    s.tune_stages = r.tune_stages;
    t->built = false;
    C.version++;            /* batches over this tracer re-plan */
    st = build(*t);
    if (st != ER_OK) return st;
    if (result) *result = r;
    return ER_OK;
}

/* the tracer's parameters with the medium's majorant grid, and the medium */
static er_status medium_params(int32_t tracer_id, const er_medium_desc* m, erd::Params& P, DmParams& M, TracerItem** tp)
{
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!m || !m->d_density || !m->d_opacity) return fail(ER_ERR_INVALID_ARGUMENT, "medium descriptor or its buffers are NULL");
    if (m->model != ER_MEDIUM_SPLINE && m->model != ER_MEDIUM_TRACER)
        return fail(ER_ERR_INVALID_ARGUMENT, "model %d is not an ER_MEDIUM_* value", m->model);
    const er_render_settings& ts = t->d.settings;
    const int shading = !ts.apply_shading_type ? ER_SHADING_BRDF_ONLY : ts.shading_type;
    if (m->model == ER_MEDIUM_TRACER) {
        if (m->n_opacity != t->d.opacity.count || m->n_opacity < 1)
            return fail(ER_ERR_INVALID_ARGUMENT, "n_opacity %d is not the tracer's opacity node count %d", m->n_opacity,
                        t->d.opacity.count);
        if (shading != ER_SHADING_BRDF_ONLY && shading != ER_SHADING_PHASE_ONLY && shading != ER_SHADING_HYBRID)
            return fail(ER_ERR_UNSUPPORTED, "the differentiable tracer model supports the BRDF, phase and hybrid shaders");
        if (shading != ER_SHADING_PHASE_ONLY && ts.gradient_computation != ER_GRADIENT_CENTRAL)
            return fail(ER_ERR_UNSUPPORTED, "the differentiable tracer model takes normals from central differences");
        if (shading == ER_SHADING_HYBRID && !(m->gradient_magnitude_inv > 0.0f && std::isfinite(m->gradient_magnitude_inv)))
            return fail(ER_ERR_INVALID_ARGUMENT, "the hybrid shader needs a finite positive gradient_magnitude_inv");
    } else if (m->n_opacity < 6 || m->n_opacity > ER_MAX_TF_NODES) {
        return fail(ER_ERR_INVALID_ARGUMENT, "n_opacity %d out of range [6, %d]", m->n_opacity, ER_MAX_TF_NODES);
    }
    if (m->brick < 1 || m->brick > 64) return fail(ER_ERR_INVALID_ARGUMENT, "brick %d out of range [1, 64]", m->brick);
    if (!(m->nee_probability > 0.0f && m->nee_probability <= 1.0f))
        return fail(ER_ERR_INVALID_ARGUMENT, "nee_probability must lie in (0, 1]");
    if (!(m->scale > 0.0f) || !std::isfinite(m->scale)) return fail(ER_ERR_INVALID_ARGUMENT, "scale must be finite and positive");
    er_status st = build(*t);
    if (st != ER_OK) return st;
    P = t->P;
    P.brick = m->brick;
    for (int i = 0; i < 3; i++) P.nb[i] = (P.res[i] + m->brick - 1) / m->brick;
    P.majorant = m->d_majorant;
    M.rho = m->d_density;
    M.tf = m->d_opacity;
    M.tf_n = m->n_opacity;
    M.scale = m->scale;
    for (int i = 0; i < 3; i++) M.albedo[i] = m->albedo[i];
    M.q = m->nee_probability;
    M.model = m->model;
    M.gm_inv = m->model == ER_MEDIUM_TRACER ? m->gradient_magnitude_inv : 0.0f;
    M.emissive = 0;
    if (m->model == ER_MEDIUM_TRACER)
        for (int c = 0; c < 3; c++)
            for (int i = 0; i < t->d.emission.plf[c].count; i++)
                if (t->d.emission.plf[c].value[i] != 0.0f) M.emissive = 1;
    *tp = t;
    return ER_OK;
}

ER_API er_status er_medium_majorant(int32_t tracer_id, const er_medium_desc* medium, float margin, float floor_, float* d_majorant,
                                    void* stream)
{
    ER_LOCK;
    erd::Params P;
    DmParams M;
    TracerItem* t = nullptr;
    er_medium_desc m = medium ? *medium : er_medium_desc();
    m.d_majorant = d_majorant;
    er_status st = medium_params(tracer_id, medium ? &m : nullptr, P, M, &t);
    if (st != ER_OK) return st;
    if (!d_majorant) return fail(ER_ERR_INVALID_ARGUMENT, "d_majorant is NULL");
    if (!(margin >= 1.0f) || !(floor_ >= 0.0f)) return fail(ER_ERR_INVALID_ARGUMENT, "margin must be >= 1 and floor >= 0");
    if ((long long)P.nb[0] * P.nb[1] * P.nb[2] > (1ll << 26))
        return fail(ER_ERR_INVALID_ARGUMENT, "%d x %d x %d bricks exceed the majorant build's 2^26", P.nb[0], P.nb[1], P.nb[2]);
    /* model 1 reads the tracer's opacity PLF (device) for its node positions */
    const erd::Plf* plf = M.model == ER_MEDIUM_TRACER
                              ? reinterpret_cast<const erd::Plf*>(reinterpret_cast<const char*>(t->tfs.p) + offsetof(erd::Tfs, opacity))
                              : nullptr;
    ER_CUDA(er_launch_dm_majorant(M.rho, P.res, P.brick, M.tf, M.tf_n, plf, M.scale, margin, floor_, d_majorant,
                                  (cudaStream_t)stream));
    return ER_OK;
}

/* names one walk of the differentiable medium (the tracer's build, the
   medium's buffers and values, spp, view, first sample, and the buffer of
   its samples): an adjoint with the key of the forward just before it
   replays against that forward's shadow jobs (er_medium.cu dm_windows) */
static uint64_t medium_walk_key(const TracerItem* t, const er_medium_desc* m, int32_t spp, uint32_t view, uint32_t first,
                                const float* samples)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    };
    const uintptr_t ptrs[4] = {(uintptr_t)m->d_density, (uintptr_t)m->d_opacity, (uintptr_t)m->d_majorant, (uintptr_t)samples};
    const int32_t ints[6] = {m->n_opacity, m->brick, m->model, spp, (int32_t)view, (int32_t)first};
    const float fl[6] = {m->scale, m->albedo[0], m->albedo[1], m->albedo[2], m->nee_probability, m->gradient_magnitude_inv};
    mix(&t->build_serial, sizeof(t->build_serial));
    mix(ptrs, sizeof(ptrs));
    mix(ints, sizeof(ints));
    mix(fl, sizeof(fl));
    return h ? h : 1;
}

ER_API er_status er_medium_render(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                  uint32_t first_sample, float* d_samples, float* d_sum_rgb, void* stream)
{
    ER_LOCK;
    erd::Params P;
    DmParams M;
    TracerItem* t = nullptr;
    er_status st = medium_params(tracer_id, medium, P, M, &t);
    if (st != ER_OK) return st;
    if (!medium->d_majorant || !d_samples || spp <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid majorant, samples buffer or spp");
    ER_CUDA(er_launch_dm_forward(P, M, spp, view, first_sample, d_samples, d_sum_rgb,
                                 medium_walk_key(t, medium, spp, view, first_sample, d_samples), (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_medium_render_f64(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                      uint32_t first_sample, double* d_samples64, double* d_sum64, void* stream)
{
    ER_LOCK;
    erd::Params P;
    DmParams M;
    TracerItem* t = nullptr;
    er_status st = medium_params(tracer_id, medium, P, M, &t);
    if (st != ER_OK) return st;
    if (!medium->d_majorant || !d_samples64 || !d_sum64 || spp <= 0)
        return fail(ER_ERR_INVALID_ARGUMENT, "invalid majorant, output buffers or spp");
    ER_CUDA(er_launch_dm_forward64(P, M, spp, view, first_sample, d_samples64, d_sum64, (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_medium_adjoint(int32_t tracer_id, const er_medium_desc* medium, int32_t spp, uint32_t view,
                                   uint32_t first_sample, const float* d_dloss_dsum, const float* d_samples,
                                   float* d_grad_density, float* d_grad_opacity, void* stream)
{
    ER_LOCK;
    erd::Params P;
    DmParams M;
    TracerItem* t = nullptr;
    er_status st = medium_params(tracer_id, medium, P, M, &t);
    if (st != ER_OK) return st;
    if (!medium->d_majorant || !d_dloss_dsum || spp <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid majorant, dLoss buffer or spp");
    ER_CUDA(er_launch_dm_adjoint(P, M, spp, view, first_sample, d_dloss_dsum, d_samples, d_grad_density, d_grad_opacity,
                                 medium_walk_key(t, medium, spp, view, first_sample, d_samples), (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_profile_enable(int32_t enable)
{
    er_wavefront_profile_enable(enable != 0);
    return ER_OK;
}

ER_API er_status er_profile_read(double* ms, int64_t* launches)
{
    if (!ms || !launches) return fail(ER_ERR_INVALID_ARGUMENT, "output pointers are NULL");
    ER_CUDA(er_wavefront_profile_read(ms, launches));
    return ER_OK;
}

ER_API er_status er_get_render_settings(int32_t tracer_id, er_render_settings* settings)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!settings) return fail(ER_ERR_INVALID_ARGUMENT, "settings pointer is NULL");
    *settings = t->d.settings;
    return ER_OK;
}

ER_API er_status er_trace_frame_device(int32_t tracer_id, uint32_t* d_lanes, float* d_frame, void* stream)
{
    ER_LOCK;
    TracerItem* t = find_tracer(tracer_id);
    if (!t) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", tracer_id);
    if (!d_lanes || !d_frame) return fail(ER_ERR_INVALID_ARGUMENT, "invalid device buffers");
    er_status st = build(*t);
    if (st != ER_OK) return st;
    ER_CUDA(er_launch_trace_frame(t->P, d_lanes, (float4*)d_frame, (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_post_frame_device(const float* d_frame, float* d_running, uint8_t* d_rgba, int32_t width, int32_t height,
                                      int32_t no_iterations, float exposure, int32_t frame_filter, void* stream)
{
    if (!d_frame || !d_running || !d_rgba || width <= 0 || height <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid post-process arguments");
    ER_CUDA(er_launch_post_frame((const float4*)d_frame, (float4*)d_running, (uchar4*)d_rgba, width, height, no_iterations, exposure,
                                 frame_filter >= 0 ? 1 : 0, (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_tonemap_device(const float* d_xyza, float scale, uint8_t* d_rgba, int32_t width, int32_t height, float exposure,
                                   void* stream)
{
    if (!d_xyza || !d_rgba || width <= 0 || height <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid tone-map arguments");
    ER_CUDA(er_launch_tonemap((const float4*)d_xyza, scale, (uchar4*)d_rgba, width * height, exposure, (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_bilateral_device(const uint8_t* d_in, uint8_t* d_tmp, uint8_t* d_out, int32_t width, int32_t height, int32_t radius,
                                     float sigma_d, float sigma_r, void* stream)
{
    if (!d_in || !d_tmp || !d_out || width <= 0 || height <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "invalid bilateral arguments");
    if (radius < 0 || radius > 127) return fail(ER_ERR_INVALID_ARGUMENT, "bilateral radius %d out of range [0, 127]", radius);
    er_render_settings s;
    er_default_render_settings(&s);
    s.bilateral_radius = radius;
    s.bilateral_sigma_d = sigma_d;
    s.bilateral_sigma_r = sigma_r;
    const BilateralTables T = bilateral_tables(s);
    ER_CUDA(er_launch_bilateral((const uchar4*)d_in, (uchar4*)d_tmp, (uchar4*)d_out, width, height, T, (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_gradient_magnitude(int32_t volume_id, uint16_t* d_gm, float* max_gm)
{
    ER_LOCK;
    auto it = ctx().volumes.items.find(volume_id);
    if (volume_id < 0 || it == ctx().volumes.items.end()) return fail(ER_ERR_INVALID_ID, "resource item with ID:%d does not exist", volume_id);
    VolumeItem& v = *it->second;
    erd::Params P;
    memset(&P, 0, sizeof(P));
    volume_geometry(v, P);
    ER_CUDA(v.gm_max_bits.ensure(1));
    cudaStream_t s = ctx().stream;
    ER_CUDA(cudaMemsetAsync(v.gm_max_bits.p, 0, sizeof(unsigned int), s));
    ER_CUDA(er_launch_gradient_magnitude(P, d_gm, v.gm_max_bits.p, s));
    unsigned int bits = 0;
    ER_CUDA(cudaMemcpyAsync(&bits, v.gm_max_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, s));
    ER_CUDA(cudaStreamSynchronize(s));
    float m;
    memcpy(&m, &bits, sizeof(m));
    v.gm_max = m;
    if (max_gm) *max_gm = m;
    ctx().version++;
    return ER_OK;
}

ER_API er_status er_build_majorant_device(const uint16_t* d_voxels, const int32_t resolution[3], int32_t brick, const float* d_sigma,
                                          int32_t sigma_count, float density_scale, float* d_majorant, void* stream)
{
    ER_LOCK;
    if (!d_voxels || !resolution || !d_sigma || !d_majorant) return fail(ER_ERR_INVALID_ARGUMENT, "NULL argument");
    if (brick < 1 || brick > 64) return fail(ER_ERR_INVALID_ARGUMENT, "brick %d out of range [1, 64]", brick);
    if (sigma_count < 1 || sigma_count > 65536) return fail(ER_ERR_INVALID_ARGUMENT, "sigma_count %d out of range [1, 65536]", sigma_count);
    int res[3], nb[3];
    for (int i = 0; i < 3; i++) {
        if (resolution[i] <= 0) return fail(ER_ERR_INVALID_ARGUMENT, "resolution must be positive");
        res[i] = resolution[i];
        nb[i] = (res[i] + brick - 1) / brick;
    }
    const size_t total = (size_t)nb[0] * nb[1] * nb[2];
    int levels = 1;
    while ((1 << levels) <= sigma_count) levels++;
    /* library-owned scratch, grown on demand */
    static DevBuf<uint32_t> minmax;
    static DevBuf<float> rmq;
    ER_CUDA(minmax.ensure(total));
    ER_CUDA(rmq.ensure((size_t)levels * sigma_count));
    ER_CUDA(er_launch_majorant(d_voxels, res, brick, nb, d_sigma, sigma_count, rmq.p, levels, minmax.p, density_scale, d_majorant,
                               (cudaStream_t)stream));
    return ER_OK;
}

ER_API er_status er_math_eval_device(int32_t fn, int32_t n, const float* d_x, const float* d_y, float* d_out, void* stream)
{
    if (fn < 0 || fn > 7 || n < 0 || !d_x || !d_out || ((fn == 5 || fn == 7) && !d_y))
        return fail(ER_ERR_INVALID_ARGUMENT, "invalid math evaluation arguments");
    if (n == 0) return ER_OK;
    ER_CUDA(er_launch_math_eval(fn, n, d_x, d_y, d_out, (cudaStream_t)stream));
    return ER_OK;
}

}  // extern "C"
