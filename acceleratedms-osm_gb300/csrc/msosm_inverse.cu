// Per-DM inverse transforms of the MS-OSM stream.
//
// Replaces, for every (DM d, window b), the reference's gatherMultiply_kernel
// (gpu/gpu_kernel.cu:106-210), the batched cufftExecC2C inverse
// (msosm_gpu_batch.cpp:196-199) and discardSamples / discardSamplesToUint16
// (gpu_kernel.cu:346-376, 398-428), plus, when folding, calculateIntensity_single and
// foldDataPhase (gpu_kernel.cu:438-444, 462-496).
//
//   pass 1 (column n1): x[n] = ring[(rbi + b - delay_d[n]) mod fbs][n] * H_d[n]
//           for n = n1 + N1*n2 -- the delayed-bin gather and the response
//           multiply happen on load; N2-point inverse DFT; times W_F^(+n1*k2)
//           into T[n1 + N1*k2].
//   pass 2 (row k2): N1-point inverse DFT; only k1 >= N1/2 (time samples M..2M-1
//           of the window) are kept, scaled by 1/F, and written as complex64 or
//           uint16 pairs at [d][b][o], o = k2 + N2*(k1 - N1/2), and/or folded:
//           |v|^2 into phase bin floor(phase(b*M + o) * K) with the phase in
//           Q0.64 fixed point, accumulated in shared memory, one flush per CTA.
#include "msosm_common.cuh"

namespace msosm {

struct InvLoader
{
    const float2 *ring;
    const float2 *Hd;       // response of this DM
    const uint16_t *dl;     // delays of this DM
    int c0, N1, F, fbs;
    int rb;                 // rbi + b
    __device__ __forceinline__ float2 load(int col, int n2) const
    {
        const int n = c0 + col + N1 * n2;
        int slot = rb - (int)__ldg(dl + n);
        if (slot < 0)
            slot += fbs;
        const float2 s = __ldg(ring + (size_t)slot * F + n);
        const float2 h = __ldg(Hd + n);
        return cmul(s, h);
    }
};

struct InvStoreT
{
    float2 *T;
    const float2 *lo, *hi;
    int c0, N1;
    unsigned n2_mask;
    int n2_shift;
    __device__ __forceinline__ void store(int col, int k2, float2 v) const
    {
        const int n1 = c0 + col;
        const float2 w = twiddle_F(lo, hi, (unsigned)(n1 * k2), n2_mask, n2_shift);
        T[n1 + (size_t)N1 * k2] = cmul(v, w);
    }
};

struct NoLoad
{
    __device__ __forceinline__ float2 load(int, int) const { return make_float2(0.f, 0.f); }
};

template <int MODE>
struct InvEpilogue
{
    float2 *out_c64;   // [d][b] row, M samples
    uint32_t *out_u16; // [d][b] row
    float *s_sum;
    unsigned *s_cnt;
    uint64_t ph_b;     // phase of sample b*M
    uint64_t dphase;
    unsigned K;
    int r0, N1, N2;
    float scale;
    __device__ __forceinline__ void store(int col, int k1, float2 v) const
    {
        if (k1 < (N1 >> 1)) // overlap-save discard (uniform per warp)
            return;
        const int o = r0 + col + N2 * (k1 - (N1 >> 1));
        v.x *= scale;
        v.y *= scale;
        if constexpr ((MODE & OUT_C64) != 0)
            out_c64[o] = v;
        if constexpr ((MODE & OUT_U16) != 0)
            out_u16[o] = encode_u16(v);
        if constexpr ((MODE & OUT_FOLD) != 0)
        {
            const float p = v.x * v.x + v.y * v.y;
            const uint64_t ph = ph_b + (uint64_t)o * dphase;
            fold_accumulate(s_sum, s_cnt, phase_bin(ph, K), p);
        }
    }
};

template <int N>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MIN_BLOCKS)
    inv_pass1_kernel(const float2 *__restrict__ ring, const float2 *__restrict__ H, const uint16_t *__restrict__ delays,
                     float2 *__restrict__ T, const float2 *__restrict__ twN2, const float2 *__restrict__ lo,
                     const float2 *__restrict__ hi, long long g0, int B, int rbi, int fbs, int N1, int F,
                     int n2_shift)
{
    using C = TileCfg<N>;
    extern __shared__ float2 smem[];
    float2 *sm = smem;
    float2 *tw = smem + C::SMEM_DATA;
    load_twiddles<N, C::THREADS>(tw, twN2);
    __syncthreads();
    const int c0 = blockIdx.x * C::COLS;
    const long long gi = g0 + blockIdx.y;
    const int d = (int)(gi / B), b = (int)(gi % B);
    InvLoader ld{ring, H + (size_t)d * F, delays + (size_t)d * F, c0, N1, F, fbs, rbi + b};
    InvStoreT st{T + (size_t)blockIdx.y * F, lo, hi, c0, N1, (unsigned)(N - 1), n2_shift};
    fft_stages<N, C::COLS, C::THREADS, +1, 1, true>(sm, tw, ld, st);
}

template <int N, int MODE>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MIN_BLOCKS)
    inv_pass2_kernel(const float2 *__restrict__ T, const float2 *__restrict__ twN1, long long g0, int B, int M,
                     int N2, float2 *__restrict__ out_c64, uint32_t *__restrict__ out_u16, FoldArgs fold)
{
    using C = TileCfg<N>;
    constexpr int LD = TileGeom<N, C::COLS>::LD;
    extern __shared__ float2 smem[];
    float2 *sm = smem;
    float2 *tw = smem + C::SMEM_DATA;
    float *s_sum = reinterpret_cast<float *>(tw + N);
    unsigned *s_cnt = reinterpret_cast<unsigned *>(s_sum + ((MODE & OUT_FOLD) ? fold.K : 0));
    const int r0 = blockIdx.x * C::COLS;
    const long long gi = g0 + blockIdx.y;
    const int d = (int)(gi / B), b = (int)(gi % B);
    const int F = 2 * M;
    const float2 *src = T + (size_t)blockIdx.y * F + (size_t)r0 * N;
    for (int e = threadIdx.x; e < C::POINTS; e += C::THREADS)
    {
        const int col = e / N, n = e % N;
        sm[n * LD + col] = __ldcg(src + e);
    }
    load_twiddles<N, C::THREADS>(tw, twN1);
    if constexpr ((MODE & OUT_FOLD) != 0)
    {
        for (unsigned i = threadIdx.x; i < fold.K; i += C::THREADS)
        {
            s_sum[i] = 0.0f;
            s_cnt[i] = 0u;
        }
    }
    __syncthreads();
    const size_t row = ((size_t)d * B + b) * M;
    InvEpilogue<MODE> ep{out_c64 ? out_c64 + row : nullptr,
                         out_u16 ? out_u16 + row : nullptr,
                         s_sum,
                         s_cnt,
                         fold_phase0(fold) + (uint64_t)((uint64_t)b * (uint64_t)M) * fold.dphase,
                         fold.dphase,
                         fold.K,
                         r0,
                         N,
                         N2,
                         1.0f / (float)F};
    fft_stages<N, C::COLS, C::THREADS, +1, 1, false>(sm, tw, NoLoad{}, ep);
    if constexpr ((MODE & OUT_FOLD) != 0)
    {
        __syncthreads();
        double *gs = fold.sum + (size_t)d * fold.K;
        unsigned long long *gc = fold.cnt + (size_t)d * fold.K;
        for (unsigned i = threadIdx.x; i < fold.K; i += C::THREADS)
        {
            const unsigned c = s_cnt[i];
            if (c)
            {
                atomicAdd(gs + i, (double)s_sum[i]);
                atomicAdd(gc + i, (unsigned long long)c);
            }
        }
    }
}

template <int N>
static cudaError_t inv_pass1(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                             cudaStream_t st)
{
    using C = TileCfg<N>;
    auto k = inv_pass1_kernel<N>;
    static size_t granted[kMaxDevices] = {};
    cudaError_t e = ensure_smem(k, C::SMEM_BYTES, granted);
    if (e != cudaSuccess)
        return e;
    dim3 grid(g.N1 / C::COLS, count);
    k<<<grid, C::THREADS, C::SMEM_BYTES, st>>>(a.ring, a.H, a.delays, a.T, tw.twN2, tw.lo, tw.hi, g0, a.B, a.rbi,
                                                  a.fbs, g.N1, g.F, __builtin_ctz((unsigned)g.N2));
    return cudaGetLastError();
}

template <int N, int MODE>
static cudaError_t inv_pass2_mode(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                                  cudaStream_t st)
{
    using C = TileCfg<N>;
    auto k = inv_pass2_kernel<N, MODE>;
    const size_t smem = C::SMEM_BYTES + (((MODE & OUT_FOLD) != 0) ? (size_t)a.fold.K * 8 : 0);
    static size_t granted[kMaxDevices] = {};
    cudaError_t e = ensure_smem(k, smem, granted);
    if (e != cudaSuccess)
        return e;
    dim3 grid(g.N2 / C::COLS, count);
    k<<<grid, C::THREADS, smem, st>>>(a.T, tw.twN1, g0, a.B, g.M, g.N2, a.out_c64, a.out_u16, a.fold);
    return cudaGetLastError();
}

template <int N>
static cudaError_t inv_pass2(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                             cudaStream_t st)
{
    switch (a.out_mode)
    {
    case OUT_C64: return inv_pass2_mode<N, OUT_C64>(g, tw, a, g0, count, st);
    case OUT_U16: return inv_pass2_mode<N, OUT_U16>(g, tw, a, g0, count, st);
    case OUT_FOLD: return inv_pass2_mode<N, OUT_FOLD>(g, tw, a, g0, count, st);
    case OUT_C64 | OUT_FOLD: return inv_pass2_mode<N, OUT_C64 | OUT_FOLD>(g, tw, a, g0, count, st);
    case OUT_U16 | OUT_FOLD: return inv_pass2_mode<N, OUT_U16 | OUT_FOLD>(g, tw, a, g0, count, st);
    case OUT_C64 | OUT_U16: return inv_pass2_mode<N, OUT_C64 | OUT_U16>(g, tw, a, g0, count, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_inverse_p1(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                              cudaStream_t st)
{
    switch (g.N2)
    {
    case 16: return inv_pass1<16>(g, tw, a, g0, count, st);
    case 32: return inv_pass1<32>(g, tw, a, g0, count, st);
    case 64: return inv_pass1<64>(g, tw, a, g0, count, st);
    case 128: return inv_pass1<128>(g, tw, a, g0, count, st);
    case 256: return inv_pass1<256>(g, tw, a, g0, count, st);
    case 512: return inv_pass1<512>(g, tw, a, g0, count, st);
    case 1024: return inv_pass1<1024>(g, tw, a, g0, count, st);
    case 2048: return inv_pass1<2048>(g, tw, a, g0, count, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_inverse_p2(const Geom &g, const Twiddles &tw, const InvArgs &a, long long g0, int count,
                              cudaStream_t st)
{
    switch (g.N1)
    {
    case 16: return inv_pass2<16>(g, tw, a, g0, count, st);
    case 32: return inv_pass2<32>(g, tw, a, g0, count, st);
    case 64: return inv_pass2<64>(g, tw, a, g0, count, st);
    case 128: return inv_pass2<128>(g, tw, a, g0, count, st);
    case 256: return inv_pass2<256>(g, tw, a, g0, count, st);
    case 512: return inv_pass2<512>(g, tw, a, g0, count, st);
    case 1024: return inv_pass2<1024>(g, tw, a, g0, count, st);
    case 2048: return inv_pass2<2048>(g, tw, a, g0, count, st);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace msosm
