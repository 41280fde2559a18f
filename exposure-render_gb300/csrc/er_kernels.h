/*
 * er_kernels.h - launch functions of the CUDA kernels, called by the host
 * runtime (er_runtime.cpp).
 */
#ifndef ER_KERNELS_H
#define ER_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

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
cudaError_t er_launch_sigma_table(const erd::Plf* opacity, float density_scale, float* table, int n, cudaStream_t s);

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

/* sets the text returned by er_last_error_message() on this thread */
void er_internal_set_error(const char* message);

/* queues of the wavefront pipeline (er_wavefront.cu); max_samples bounds one chunk */
struct WavefrontBuffers {
    float4* results;     /* max_samples */
    float4* events;      /* 5 * max_samples */
    float4* jobs;        /* 6 * max_samples */
    float4* partial;     /* film pixels */
    uint32_t* counters;  /* 2 */
    size_t max_samples;
    int tune_primary;    /* resident blocks per SM targeted by the primary stage (1..4) */
    int tune_shadow;     /* same for the shadow stage */
};

size_t er_wavefront_chunk_spp(int npix, int spp, size_t max_samples);
cudaError_t er_launch_wavefront(const erd::Params& P, int spp, uint32_t view, uint32_t first, float4* sum, int accumulate,
                                const WavefrontBuffers& B, cudaStream_t s);

#endif
