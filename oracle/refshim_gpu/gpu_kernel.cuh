/*
 * ORACLE build shim -- gpu/include/gpu_kernel.cuh for a host-only build of the
 * reference's msosm_gpu_batch.cpp (for MSOSM_GPU_BATCH::build_segments,
 * msosm_gpu_batch.cpp:262-295).  Keeps the types and constants the processor
 * uses (gpu_kernel.cuh:5-21: ITEMS_PER_THREAD, BLOCK_SIZE, Segment,
 * DelayBlockMeta), the CUDA_CHECK / CUFFT_CHECK macros and the NVTX range macros
 * (gpu_common.cuh:17-62, here no-ops), and declares the kernel wrappers the
 * processor calls (gpu_kernel.cuh:23-40), which refshim_gpu/kernel_stubs.cpp
 * defines as no-ops: nothing of the GPU path is run, only build_segments.
 */
#pragma once
#include "globals.h"

constexpr int ITEMS_PER_THREAD = 4;
constexpr int BLOCK_SIZE = 256;

typedef struct
{
    int start;
    int len;
    int group;
} Segment;

typedef struct
{
    int seg_offset;
    int seg_count;
} DelayBlockMeta;

#define CUDA_CHECK(call) (void)(call)
#define CUFFT_CHECK(call) (void)(call)
#define PUSH_RANGE(name, cid)
#define POP_RANGE
#define nvtxNameCudaStream(stream, name) (void)(stream)

void GPU_GetDevInfo();
void uint16ToComplex(Complex *dst, uint16_t *src, size_t size, cudaStream_t stream = 0);
void gatherMultiply(const Complex *fft_block, const Complex *dedisp_params, Complex *ifft_input,
                    const DelayBlockMeta *delay_block_meta, const Segment *segments, int &max_seg_count, int &batch,
                    int &numDMs, int &fftpoint, int &read_block_index, int &fft_block_size, cudaStream_t stream = 0);
void discardSamples(Complex *a, Complex *b, int M, int count, cudaStream_t stream = 0);
void discardSamplesToUint16(uint16_t *dst, Complex *src, int M, int count, cudaStream_t stream = 0);
