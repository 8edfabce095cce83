// Stand-alone intensity + phase fold (Fold_GPU, folding/fold_gpu.cpp:27-60).
//
// Replaces calculateIntensity / calculateIntensity_single (gpu/gpu_kernel.cu:430-460),
// foldDataPhase (gpu_kernel.cu:462-496) and computeFoldedData (gpu_kernel.cu:498-518)
// for callers that fold the processor's complex output themselves (the 2-pol
// path and the reference-shaped Fold_GPU object).  The intensity is computed on
// the fly -- no intensity buffer -- and samples are binned with the same Q0.64
// fixed-point phase as the fused path: bin = floor(frac(t/P) * K) computed
// without per-sample FP64 arithmetic.
#include "msosm_common.cuh"

namespace msosm {

constexpr int FOLD_THREADS = 256;
constexpr unsigned FOLD_SMEM_MAX_BINS = 12288; // 96 KB of bins

template <int KIND, bool SMEM_BINS>
__global__ void __launch_bounds__(FOLD_THREADS)
    fold_kernel(const float2 *__restrict__ a, const float2 *__restrict__ b, size_t size, FoldArgs f, size_t chunk)
{
    extern __shared__ float fsm[];
    float *s_sum = fsm;
    unsigned *s_cnt = reinterpret_cast<unsigned *>(fsm + (SMEM_BINS ? f.K : 0));
    const int s = blockIdx.y;
    const float2 *pa = a + (size_t)s * size;
    const float2 *pb = KIND != FOLD_POWER ? b + (size_t)s * size : nullptr;
    if constexpr (SMEM_BINS)
    {
        for (unsigned i = threadIdx.x; i < f.K; i += FOLD_THREADS)
        {
            s_sum[i] = 0.0f;
            s_cnt[i] = 0u;
        }
        __syncthreads();
    }
    const size_t begin = (size_t)blockIdx.x * chunk;
    const size_t end = begin + chunk < size ? begin + chunk : size;
    // whole warps iterate together so the shuffles in fold_accumulate see all lanes
    for (size_t base = begin; base < end; base += FOLD_THREADS)
    {
        const size_t i = base + threadIdx.x;
        float p = 0.0f;
        bool nz = false;
        unsigned bin = 0;
        if (i < end)
        {
            const float2 x = __ldcs(pa + i);
            if constexpr (KIND == FOLD_POWER2)
            {
                const float2 y = __ldcs(pb + i);
                p = sqrtf(x.x * x.x + x.y * x.y + y.x * y.x + y.y * y.y);
                nz = p != 0.0f;
            }
            else if constexpr (KIND == FOLD_CROSS)
            {
                // 2 Re(conj(a) b), counted where |a|^2 is, so counts match the power fold
                const float2 y = __ldcs(pb + i);
                p = 2.0f * (x.x * y.x + x.y * y.y);
                nz = (x.x * x.x + x.y * x.y) != 0.0f;
            }
            else
            {
                p = x.x * x.x + x.y * x.y;
                nz = p != 0.0f;
            }
            bin = phase_bin(fold_phase0(f) + (uint64_t)i * f.dphase, f.K);
        }
        if constexpr (SMEM_BINS)
            fold_accumulate(s_sum, s_cnt, bin, p, nz);
        else if (nz)
        {
            atomicAdd(f.sum + (size_t)s * f.K + bin, (double)p);
            atomicAdd(f.cnt + (size_t)s * f.K + bin, 1ULL);
        }
    }
    if constexpr (SMEM_BINS)
    {
        __syncthreads();
        double *gs = f.sum + (size_t)s * f.K;
        unsigned long long *gc = f.cnt + (size_t)s * f.K;
        for (unsigned k = threadIdx.x; k < f.K; k += FOLD_THREADS)
        {
            const unsigned c = s_cnt[k];
            if (c)
            {
                atomicAdd(gs + k, (double)s_sum[k]);
                atomicAdd(gc + k, (unsigned long long)c);
            }
        }
    }
}

template <int KIND, bool SMEM_BINS>
static cudaError_t fold_launch(const float2 *a, const float2 *b, size_t size, int series, const FoldArgs &f,
                               cudaStream_t st)
{
    auto k = fold_kernel<KIND, SMEM_BINS>;
    const size_t smem = SMEM_BINS ? (size_t)f.K * 8 : 0;
    static size_t granted[kMaxDevices] = {};
    cudaError_t e = ensure_smem(k, smem, granted);
    if (e != cudaSuccess)
        return e;
    // ~4 chunks per SM across all series; each chunk a multiple of the block size
    const size_t target_blocks = 152 * 4;
    size_t per_series = (target_blocks + series - 1) / series;
    size_t chunk = (size + per_series - 1) / per_series;
    chunk = ((chunk + FOLD_THREADS - 1) / FOLD_THREADS) * FOLD_THREADS;
    if (chunk < 8 * FOLD_THREADS)
        chunk = 8 * FOLD_THREADS;
    const unsigned gx = (unsigned)((size + chunk - 1) / chunk);
    dim3 grid(gx > 0 ? gx : 1, series);
    k<<<grid, FOLD_THREADS, smem, st>>>(a, b, size, f, chunk);
    return cudaGetLastError();
}

template <int KIND>
static cudaError_t fold_kind(const float2 *pol1, const float2 *pol2, size_t size, int series, const FoldArgs &f,
                             cudaStream_t st)
{
    return f.K <= FOLD_SMEM_MAX_BINS ? fold_launch<KIND, true>(pol1, pol2, size, series, f, st)
                                     : fold_launch<KIND, false>(pol1, pol2, size, series, f, st);
}

cudaError_t launch_fold(const float2 *pol1, const float2 *pol2, size_t size, int series, const FoldArgs &f,
                        cudaStream_t st, int kind /* = FOLD_POWER */)
{
    if (size == 0 || series <= 0)
        return cudaSuccess;
    if (kind == FOLD_CROSS)
        return fold_kind<FOLD_CROSS>(pol1, pol2, size, series, f, st);
    if (pol2)
        return fold_kind<FOLD_POWER2>(pol1, pol2, size, series, f, st);
    return fold_kind<FOLD_POWER>(pol1, nullptr, size, series, f, st);
}

__global__ void fold_finalize_kernel(const double *__restrict__ sum, const unsigned long long *__restrict__ cnt,
                                     float *__restrict__ folded, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const unsigned long long c = cnt[i];
    folded[i] = c > 0 ? (float)(sum[i] / (double)c) : 0.0f;
}

cudaError_t launch_fold_finalize(const double *sum, const unsigned long long *cnt, float *folded, size_t n,
                                 cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    fold_finalize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sum, cnt, folded, n);
    return cudaGetLastError();
}

namespace {
__global__ void phase_set_kernel(unsigned long long *p, unsigned long long v) { *p = v; }
__global__ void phase_advance_kernel(unsigned long long *p, unsigned long long inc) { *p += inc; }
} // namespace

cudaError_t launch_phase_set(uint64_t *phase, uint64_t value, cudaStream_t st)
{
    phase_set_kernel<<<1, 1, 0, st>>>(reinterpret_cast<unsigned long long *>(phase), value);
    return cudaGetLastError();
}

cudaError_t launch_phase_advance(uint64_t *phase, uint64_t inc, cudaStream_t st)
{
    phase_advance_kernel<<<1, 1, 0, st>>>(reinterpret_cast<unsigned long long *>(phase), inc);
    return cudaGetLastError();
}

} // namespace msosm
