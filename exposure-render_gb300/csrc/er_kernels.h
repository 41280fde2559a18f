/*
 * er_kernels.h - launch functions of the CUDA kernels, called by the host
 * runtime (er_runtime.cpp).
 */
#ifndef ER_KERNELS_H
#define ER_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "er_device.cuh"

/* spatial (KernelD) and range (GaussSimilarity) weights of the bilateral
   filter (Source/filter.h:34-40), passed by value */
struct BilateralTables {
    int radius;
    float spatial[256];
    float range[256];
};

cudaError_t er_launch_trace_frame(const erd::Params& P, uint32_t* lanes, float4* frame, cudaStream_t s);
cudaError_t er_launch_trace_sum(const erd::Params& P, int spp, uint32_t view, uint32_t first, float4* sum, int accumulate,
                                cudaStream_t s);
/* the autofocus distance of film pixel (u, v) into out (one float) */
cudaError_t er_launch_autofocus(const erd::Params& P, int u, int v, uint32_t lane0, uint32_t lane1, float* out, cudaStream_t s);
cudaError_t er_launch_sigma_table(const erd::Plf* opacity, float density_scale, float* table, int n, cudaStream_t s);
/* 3 float4 per integer intensity in [0, n): the shading transfer functions (erd::shade_tf) */
cudaError_t er_launch_shade_table(const erd::Tfs* tfs, float4* tab, int n, cudaStream_t s);

cudaError_t er_launch_post_frame(const float4* frame, float4* running, uchar4* rgba, int W, int H, int n_iter, float exposure,
                                 int filter, cudaStream_t s);
cudaError_t er_launch_post_mean(const float4* sum, float n, float4* running, uchar4* rgba, int W, int H, float exposure, int filter,
                                cudaStream_t s);
cudaError_t er_launch_tonemap(const float4* xyza, float scale, uchar4* rgba, int n, float exposure, cudaStream_t s);
cudaError_t er_launch_bilateral(const uchar4* in, uchar4* tmp, uchar4* out, int W, int H, const BilateralTables& T,
                                cudaStream_t s);
cudaError_t er_launch_gradient_magnitude(const erd::Params& P, uint16_t* gm, unsigned int* max_bits, cudaStream_t s);
cudaError_t er_launch_math_eval(int fn, int n, const float* x, const float* y, float* out, cudaStream_t s);
cudaError_t er_launch_majorant(const uint16_t* vox, const int res[3], int B, const int nb[3], const float* sigma, int n,
                               float* rmq, int levels, uint32_t* minmax, float density_scale, float* majorant, cudaStream_t s);
/* writes -(Chebyshev distance to the nearest non-empty brick, capped at 32)
   into the empty bricks of a majorant grid; tmp holds 2 bytes per brick */
cudaError_t er_launch_empty_skip(float* majorant, const int nb[3], uint8_t* tmp, cudaStream_t s);

/* the differentiable medium (er_medium.cu) */
struct DmParams {
    const float* rho;    /* density grid, the tracer volume's resolution, x fastest */
    const float* tf;     /* tf_n opacity B-spline values (model 0) or opacity node values (model 1) */
    int tf_n;
    float scale;         /* sigma = scale * opacity */
    float albedo[3];
    float q;             /* next-event probability per collision */
    int model;           /* 0: B-spline opacity, isotropic albedo; 1: the tracer's transfer functions and shading */
    int emissive;        /* model 1: the tracer's emission TF is not zero everywhere */
    float gm_inv;        /* model 1, hybrid: 1 / gradient-magnitude range (a constant) */
};
/* key: nonzero name of the walk (tracer build, medium, spp, view, first
   sample); an adjoint with the key and stream of the last one-window call
   replays against that call's kept shadow jobs */
cudaError_t er_launch_dm_forward(const erd::Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, float* samples,
                                 float* sum, uint64_t key, cudaStream_t s);
cudaError_t er_launch_dm_forward64(const erd::Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, double* samples,
                                   double* sum, cudaStream_t s);
cudaError_t er_launch_dm_adjoint(const erd::Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, const float* dimg,
                                 const float* fwd, float* g_rho, float* g_tf, uint64_t key, cudaStream_t s);
/* plf: NULL for model 0 (B-spline values tf); model 1: the tracer's opacity
   PLF (device), whose node values are tf */
cudaError_t er_launch_dm_majorant(const float* rho, const int res[3], int B, const float* tf, int n, const erd::Plf* plf, float scale,
                                  float margin, float floor_, float* out, cudaStream_t s);

/* corner quads (quad may be NULL; laid out by quad_index with qb_nbx,
   qb_slab) and atomicMax of the voxel values over the box [lo, lo + n) */
cudaError_t er_launch_box_quads_max(const uint16_t* vox, const int res[3], const int lo[3], const int n[3], uint2* quad, int qb_nbx,
                                    unsigned long long qb_slab, unsigned int* vmax, cudaStream_t s);

/* sets the text returned by er_last_error_message() on this thread */
void er_internal_set_error(const char* message);

/* one view of a wavefront batch (er_wavefront.cu): the tracer's parameters,
   its RNG stream and its output sums */
struct WfView {
    erd::Params P;
    uint32_t view_id;    /* view index of the counter-based RNG stream */
    uint32_t first;      /* sample index of the view's first sample */
    int spp;             /* samples per pixel rendered by one batch launch */
    int accumulate;      /* add to sum instead of overwriting it */
    float4* sum;         /* film pixels: X, Y, Z and alpha sums */
    /* display pass of a batch (er_post.cu k_post_batch) */
    int display;         /* 1: mean -> frame filter -> tone map */
    int filter;          /* 3x3 Gaussian of the mean */
    float exposure;
    float4* running;     /* film pixels: the filtered mean */
    uchar4* rgba;        /* film pixels: the tone-mapped display */
};

cudaError_t er_launch_post_batch(const WfView* d_views, int n_views, int max_w, int max_h, cudaStream_t s);

/* sample rows [s0, s1) of one view, at item `offset` of its window */
struct WfSegment {
    int view;
    int s0, s1;
    uint32_t offset;
};

/* windows of a batch: each is one pass of the four stages */
struct WavefrontPlan {
    std::vector<WfSegment> segs;          /* all windows' segments, window by window */
    std::vector<int> window_first;        /* first segment of each window */
    std::vector<uint32_t> window_items;   /* items of each window */
    std::vector<int> view_npix;           /* film pixels of each view */
    size_t max_items = 0;                 /* largest window */
    int max_npix = 0;                     /* largest film */
};

/* queues of the wavefront pipeline, sized by a plan */
struct WavefrontBuffers {
    float4* results;     /* max_items */
    float4* events;      /* 5 * max_items */
    float4* jobs;        /* 6 * max_items */
    float4* partial;     /* 2 * max_npix: sums of a view cut by a window boundary */
    float4* records;     /* 5 * max_items when sort_shade: shading records by shader (BRDF from the front, phase from the back) */
    uint32_t* counters;  /* 6: events, shadow jobs, items and jobs taken by the persistent stages, BRDF and phase records */
    int tune_primary;    /* resident blocks per SM targeted by the primary stage (2, 3, 4, 6, 8) */
    int tune_shadow;     /* same for the shadow stage */
    int tune_shade;      /* resident 128-thread blocks per SM of the shade stage (2, 3, 4, 6) */
    int objects;         /* 1 when a view has surface objects: the primary and shade stages run their
                            object-handling variants (at the default occupancy) */
    int pt_primary;      /* the persistent-lane primary stage runs (every view delta-tracks) */
    int pt_shadow;       /* the persistent-lane shadow stage runs (every view delta-tracks) */
    int skip_primary;    /* the free-flight stage compiles the empty-space skip */
    int skip_shadow;     /* the shadow stage compiles the empty-space skip */
    int refill_eighths;  /* persistent stages refill a warp when fewer than this many eighths of its
                            tracking lanes still track (1..7) */
    int sort_shade;      /* a view's shader switch mixes BRDF and phase events: the shade stage runs as
                            k_wf_classify + k_wf_shade_sorted (records must be allocated) */
};

/* cuts the items of views (npix[v] * spp[v] each) into windows of whole
   sample rows of at most window_cap items (one row at least) */
void er_wavefront_plan(const int* npix, const int* spp, int n_views, size_t window_cap, WavefrontPlan& plan);

/* stage timing of the wavefront launches: 0 primary, 1 shade, 2 shadow,
   3 reduce; read returns the accumulated milliseconds and launch counts since
   the previous read (and clears them) */
#define WF_STAGES 4
void er_wavefront_profile_enable(bool on);
cudaError_t er_wavefront_profile_read(double* ms, int64_t* launches);

/* one view with its parameters passed by value (no device tables) */
cudaError_t er_launch_wavefront_one(const WfView& view, const WavefrontPlan& plan, const WavefrontBuffers& B, cudaStream_t s);

/* many views: d_views / d_segs are the plan's tables in device memory */
cudaError_t er_launch_wavefront_batch(const WfView* d_views, const WfSegment* d_segs, const WavefrontPlan& plan,
                                      const WavefrontBuffers& B, cudaStream_t s);

#endif
