/*
 * ORACLE build shim -- no-op definitions of the kernel wrappers and helpers the
 * reference's msosm_gpu_batch.cpp references, so that its host-only build links.
 * None of them is called: the library built with them exposes build_segments only.
 */
#include "gpu_kernel.cuh"

bool verbose = false;
void line() {}
void banner() {}
void GPU_GetDevInfo() {}
void uint16ToComplex(Complex *, uint16_t *, size_t, cudaStream_t) {}
void gatherMultiply(const Complex *, const Complex *, Complex *, const DelayBlockMeta *, const Segment *, int &, int &,
                    int &, int &, int &, int &, cudaStream_t)
{
}
void discardSamples(Complex *, Complex *, int, int, cudaStream_t) {}
void discardSamplesToUint16(uint16_t *, Complex *, int, int, cudaStream_t) {}
