// Kernel launch interface of the MS-OSM engine (internal; not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace msosm {

enum InFormat : int
{
    IN_U16 = 0, // uint16_pair offset binary, 0 = no data (gpu_kernel.cu:16-30)
    IN_C64 = 1, // complex64
    IN_I8 = 2,  // int8 interleaved I/Q
};

enum OutMode : int
{
    OUT_NONE = 0,
    OUT_C64 = 1,  // float2 [D][B][M] (fold-mode output buffer of the reference)
    OUT_U16 = 2,  // uint16_pair [D][B][M] (discardSamplesToUint16)
    OUT_FOLD = 4, // |x|^2 phase fold of every DM (fused)
    OUT_POW = 8,  // float |x|^2 [D][B][M] for the second polarisation's fused fold
    OUT_PAIR = 16 // with OUT_FOLD: fold sqrt(partner |a|^2 + |x|^2) (2-pol intensity)
};

// F = N1 * N2, N2 = 2^ceil(L/2), N1 = 2^floor(L/2).
struct Geom
{
    int L, F, M, N1, N2;
};

// Twiddle tables for one transform direction, in device memory.
struct Twiddles
{
    const float2 *twN1; // W_{N1}^m, m < N1
    const float2 *twN2; // W_{N2}^m, m < N2
    const float2 *lo;   // W_F^m, m < N2
    const float2 *hi;   // W_F^(m*N2), m < N1
};

struct FoldArgs
{
    double *sum;         // [D][K] accumulated sums (double, as Fold_GPU)
    unsigned long long *cnt; // [D][K] sample counts
    uint64_t phase0;     // phase of sample 0 of this call, Q0.64 turns
    uint64_t dphase;     // phase advance per sample, Q0.64 turns
    unsigned K;          // bins per series
    // set in captured graphs: phase0 is read from here at run time (the graph's calls
    // advance it), since a replay cannot take a new phase0 from the host
    const uint64_t *phase_dev = nullptr;
};

#ifdef __CUDACC__
__device__ __forceinline__ uint64_t fold_phase0(const FoldArgs &f)
{
    return f.phase_dev ? __ldcg(reinterpret_cast<const unsigned long long *>(f.phase_dev)) : f.phase0;
}
#endif

// Device-resident fold phase of captured graphs: set it (stream-ordered, no host buffer)
// or advance it by one call's samples.
cudaError_t launch_phase_set(uint64_t *phase, uint64_t value, cudaStream_t st);
cudaError_t launch_phase_advance(uint64_t *phase, uint64_t inc, cudaStream_t st);

// Which step of the last failed launch helper on this thread went wrong (the shared-
// memory attribute or the launch itself, with the launch geometry); empty if none.
const char *launch_failure_detail();
void set_launch_failure_detail(const char *kernel, const char *step, unsigned gx, unsigned gy, unsigned block,
                               size_t smem);

// Forward: B overlapping windows of the [tail | new input] stream -> spectra ring slots.
// Pass 1 (decode + column transforms -> T), pass 2 (row transforms -> ring slot rbi+b).
cudaError_t launch_forward_p1(const Geom &g, const Twiddles &tw, int in_format, const void *in, const float2 *tail,
                              float2 *tail_next, float2 *T, int B, cudaStream_t st);
cudaError_t launch_forward_p2(const Geom &g, const Twiddles &tw, const float2 *T, float2 *ring, int rbi, int B,
                              cudaStream_t st);

// Inverse for FFTs g0 .. g0+count-1 (g = d*B + b): gather x response -> inverse -> epilogue.
struct InvArgs
{
    const float2 *ring;
    const float2 *H;        // [D][F]
    const uint16_t *delays; // [D][F]
    float2 *T;              // [count][F] intermediate
    int rbi, fbs, B;
    int out_mode;
    float2 *out_c64;  // [D][B][M]
    uint32_t *out_u16; // [D][B][M]
    FoldArgs fold;
};
// Pass 1 (gather x response + column transforms -> T), pass 2 (row transforms + epilogue).
cudaError_t launch_inverse_p1(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                              cudaStream_t st);
cudaError_t launch_inverse_p2(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                              cudaStream_t st);

// Standalone intensity + phase fold of `size` samples of one or two complex series
// (Fold_GPU::calculate_intensity + fold_data_phase).  kind FOLD_POWER: pol2 ==
// nullptr gives |a|^2, otherwise sqrt(|a|^2+|b|^2) (FOLD_POWER2); FOLD_CROSS folds
// 2 Re(conj(a) b), counted where |a|^2 != 0 (the derivative of |a|^2 when b = da).
// series: number of consecutive series of length `size`.
enum FoldKind : int
{
    FOLD_POWER = 0,
    FOLD_POWER2 = 1,
    FOLD_CROSS = 2,
};
cudaError_t launch_fold(const float2 *pol1, const float2 *pol2, size_t size, int series, const FoldArgs &f,
                        cudaStream_t st, int kind = FOLD_POWER);

// folded[i] = cnt ? sum/cnt : 0 (computeFoldedData_kernel)
cudaError_t launch_fold_finalize(const double *sum, const unsigned long long *cnt, float *folded, size_t n,
                                 cudaStream_t st);

} // namespace msosm
