// Shared device helpers of the MS-OSM kernels.
#pragma once
#include <algorithm>
#include "fft_tile.cuh"
#include "msosm_kernels.cuh"

namespace msosm {

// Columns per CTA and threads per CTA for a sub-transform of length N.  Large
// sub-transforms use 8192-point tiles (64 KB of data); small ones keep 16
// columns so that every global access covers at least 128 contiguous bytes.
template <int N>
struct TileCfg
{
    static constexpr int COLS = (N <= 512) ? 16 : 8192 / N; // 8192-point tiles from N = 512 up
    static constexpr int POINTS = N * COLS;
    static constexpr int THREADS = (POINTS / 16 < 32) ? 32 : (POINTS / 16);
    static constexpr int SMEM_DATA = TileGeom<N, COLS>::SMEM_ELEMS; // float2 elements
    static constexpr size_t SMEM_BYTES = (size_t)(SMEM_DATA + N) * sizeof(float2);
    // two CTAs per SM: one CTA's loads overlap the other's butterflies
    static constexpr int MIN_BLOCKS = 2;
};

// W_F^m from the two-level table: m = hi*N2 + lo.
__device__ __forceinline__ float2 twiddle_F(const float2 *__restrict__ lo, const float2 *__restrict__ hi, unsigned m,
                                            unsigned n2_mask, int n2_shift)
{
    return cmul(__ldg(lo + (m & n2_mask)), __ldg(hi + (m >> n2_shift)));
}

// uint16 offset-binary decode: x - 32768*(x != 0)  (gpu/gpu_kernel.cu:16-30)
__device__ __forceinline__ float2 decode_u16(uint32_t v)
{
    const uint32_t x = v & 0xFFFFu, y = v >> 16;
    return make_float2((float)x - 32768.0f * (float)(x != 0u), (float)y - 32768.0f * (float)(y != 0u));
}

template <int FMT>
__device__ __forceinline__ float2 load_sample(const void *__restrict__ in, size_t i)
{
    if constexpr (FMT == IN_U16)
        return decode_u16(__ldcs(reinterpret_cast<const unsigned int *>(in) + i));
    else if constexpr (FMT == IN_C64)
        return __ldcs(reinterpret_cast<const float2 *>(in) + i);
    else
    {
        const short v = __ldcs(reinterpret_cast<const short *>(in) + i);
        return make_float2((float)(signed char)(v & 0xFF), (float)(signed char)((v >> 8) & 0xFF));
    }
}

// discardSamplesToUint16 epilogue (gpu/gpu_kernel.cu:398-413): round-to-nearest,
// offset 32768 for non-zero values, packed (y << 16) | x.
__device__ __forceinline__ uint32_t encode_u16(float2 v)
{
    const uint32_t x = __float2uint_rn(v.x + (v.x != 0.0f ? 32768.0f : 0.0f));
    const uint32_t y = __float2uint_rn(v.y + (v.y != 0.0f ? 32768.0f : 0.0f));
    return (y << 16) | x;
}

// Add sample p (skipped when exactly zero, as foldDataPhase_kernel does) to
// shared phase bin `bin`.  All 32 lanes must call it together, and the samples of
// each half-warp must be in time order spanning less than one period.  Bins are
// then cyclically non-decreasing along the half-warp, so equal first and last
// bins mean one shared bin: the half-warp is reduced with shuffles and lands as a
// single atomic.
// `nz` says whether the sample counts (p may be a signed term that is zero).
__device__ __forceinline__ void fold_accumulate(float *s_sum, unsigned *s_cnt, unsigned bin, float p, bool nz)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned base = lane & 16u;
    const unsigned half = base ? 0xFFFF0000u : 0x0000FFFFu;
    const unsigned b_first = __shfl_sync(0xFFFFFFFFu, bin, base);
    const unsigned b_last = __shfl_sync(0xFFFFFFFFu, bin, base + 15u);
    const unsigned nzmask = __ballot_sync(0xFFFFFFFFu, nz);
    float s = p;
    s += __shfl_xor_sync(0xFFFFFFFFu, s, 8);
    s += __shfl_xor_sync(0xFFFFFFFFu, s, 4);
    s += __shfl_xor_sync(0xFFFFFFFFu, s, 2);
    s += __shfl_xor_sync(0xFFFFFFFFu, s, 1);
    if (b_first == b_last)
    {
        if ((lane & 15u) == 0u)
        {
            const unsigned c = __popc(nzmask & half);
            if (c)
            {
                atomicAdd(s_sum + bin, s);
                atomicAdd(s_cnt + bin, c);
            }
        }
    }
    else if (nz)
    {
        atomicAdd(s_sum + bin, p);
        atomicAdd(s_cnt + bin, 1u);
    }
}

__device__ __forceinline__ void fold_accumulate(float *s_sum, unsigned *s_cnt, unsigned bin, float p)
{
    fold_accumulate(s_sum, s_cnt, bin, p, p != 0.0f);
}

// Phase bin of a Q0.64 phase: floor(phase * K).
__device__ __forceinline__ unsigned phase_bin(uint64_t ph, unsigned K)
{
    return (unsigned)__umul64hi(ph, (unsigned long long)K);
}

// Raise a kernel's dynamic shared-memory limit.  `granted` is the caller's
// per-kernel cache (a function-local static in each launch wrapper, which is
// instantiated once per kernel), indexed by device.
constexpr int kMaxDevices = 64;
template <class KERNEL>
inline cudaError_t ensure_smem(KERNEL k, size_t bytes, size_t (&granted)[kMaxDevices])
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        dev = 0;
    if (bytes <= 48 * 1024 || bytes <= granted[dev])
        return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        granted[dev] = bytes;
    else
        (void)cudaGetLastError(); // reported through the return value, not left for later calls
    return e;
}

// Prefer a shared-memory carveout that holds `blocks` CTAs of `dyn_bytes` dynamic
// shared memory each (plus static and per-CTA reserved bytes), rounded down to a
// whole percent: the driver rounds a carveout up to the next configuration it has.
template <class KERNEL>
inline cudaError_t prefer_carveout(KERNEL k, size_t dyn_bytes, int blocks)
{
    int dev = 0, per_sm = 0, reserved = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
        return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k)) != cudaSuccess)
        return e;
    if (per_sm <= 0)
        return cudaSuccess;
    const size_t need = (size_t)blocks * (dyn_bytes + fa.sharedSizeBytes + (size_t)reserved);
    const int pct = (int)std::min<size_t>(100, need * 100 / (size_t)per_sm);
    return cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

} // namespace msosm
