// Forward transforms of the MS-OSM stream (replaces the reference's
// uint16ToComplex + cufftPlanMany forward, msosm_gpu_batch.cpp:100-107,189-191).
//
// Window b of a call covers samples [b*M, b*M + 2M) of [tail | new input], i.e.
// the previous call's last M samples followed by the B*M new ones
// (msosm_gpu_batch.cpp:153-165).  F = 2M = N1*N2 is done in two passes:
//   pass 1: column n1 -> N2-point DFT over x[n1 + N1*n2], times W_F^(-n1*k2),
//           into T[n1 + N1*k2]; input decode (u16 / c64 / i8) is fused into the
//           load and the tail for the next call is written on the way.
//   pass 2: row k2 -> N1-point DFT over T[n1 + N1*k2] -> X[k2 + N2*k1], written
//           straight into spectra-ring slot rbi + b.
#include "msosm_common.cuh"

#include <cstdio>

namespace msosm {

namespace {
thread_local char g_launch_detail[192] = "";
}

const char *launch_failure_detail() { return g_launch_detail; }

void set_launch_failure_detail(const char *kernel, const char *step, unsigned gx, unsigned gy, unsigned block,
                               size_t smem)
{
    if (!kernel || !*kernel)
    {
        g_launch_detail[0] = '\0'; // cleared
        return;
    }
    std::snprintf(g_launch_detail, sizeof g_launch_detail, "%s: %s (grid %u x %u, %u threads, %zu bytes shared)",
                  kernel, step, gx, gy, block, smem);
}

template <int FMT>
struct FwdLoader
{
    const void *in;
    const float2 *tail;
    float2 *tail_next;
    int c0, b, B, M, N1;
    __device__ __forceinline__ float2 load(int col, int n2) const
    {
        const int nbin = c0 + col + N1 * n2;
        const long long s = (long long)b * M + nbin;
        float2 v;
        if (s < M)
            v = tail[s];
        else
            v = load_sample<FMT>(in, (size_t)(s - M));
        if (b == B - 1 && nbin >= M)
            tail_next[nbin - M] = v;
        return v;
    }
};

struct FwdStoreT
{
    float2 *T; // this window's intermediate
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

struct NoLoader
{
    __device__ __forceinline__ float2 load(int, int) const { return make_float2(0.f, 0.f); }
};

struct RingStore
{
    float2 *dst; // ring slot base
    int r0, N2;
    __device__ __forceinline__ void store(int col, int k1, float2 v) const
    {
        dst[r0 + col + (size_t)N2 * k1] = v;
    }
};

template <int N, int FMT>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MIN_BLOCKS)
    fwd_pass1_kernel(const void *__restrict__ in, const float2 *__restrict__ tail, float2 *__restrict__ tail_next,
                     float2 *__restrict__ T, const float2 *__restrict__ twN2, const float2 *__restrict__ lo,
                     const float2 *__restrict__ hi, int B, int M, int N1, int n2_shift)
{
    using C = TileCfg<N>;
    extern __shared__ float2 smem[];
    float2 *sm = smem;
    float2 *tw = smem + C::SMEM_DATA;
    load_twiddles<N, C::THREADS>(tw, twN2);
    __syncthreads();
    const int c0 = blockIdx.x * C::COLS;
    const int b = blockIdx.y;
    const int F = 2 * M;
    FwdLoader<FMT> ld{in, tail, tail_next, c0, b, B, M, N1};
    FwdStoreT st{T + (size_t)b * F, lo, hi, c0, N1, (unsigned)(N - 1), n2_shift};
    fft_stages<N, C::COLS, C::THREADS, -1, 1, true>(sm, tw, ld, st);
}

template <int N>
__global__ void __launch_bounds__(TileCfg<N>::THREADS, TileCfg<N>::MIN_BLOCKS)
    fwd_pass2_kernel(const float2 *__restrict__ T, float2 *__restrict__ ring, const float2 *__restrict__ twN1,
                     int rbi, int M, int N2)
{
    using C = TileCfg<N>;
    constexpr int LD = TileGeom<N, C::COLS>::LD;
    extern __shared__ float2 smem[];
    float2 *sm = smem;
    float2 *tw = smem + C::SMEM_DATA;
    const int r0 = blockIdx.x * C::COLS;
    const int b = blockIdx.y;
    const int F = 2 * M;
    const float2 *src = T + (size_t)b * F + (size_t)r0 * N;
    for (int e = threadIdx.x; e < C::POINTS; e += C::THREADS)
    {
        const int col = e / N, n = e % N;
        sm[n * LD + col] = __ldcg(src + e);
    }
    load_twiddles<N, C::THREADS>(tw, twN1);
    __syncthreads();
    RingStore st{ring + (size_t)(rbi + b) * F, r0, N2};
    fft_stages<N, C::COLS, C::THREADS, -1, 1, false>(sm, tw, NoLoader{}, st);
}

template <int N, int FMT>
static cudaError_t fwd_pass1(const Geom &g, const Twiddles &tw, const void *in, const float2 *tail, float2 *tail_next,
                             float2 *T, int B, cudaStream_t st)
{
    using C = TileCfg<N>;
    auto k = fwd_pass1_kernel<N, FMT>;
    static size_t granted[kMaxDevices] = {};
    dim3 grid(g.N1 / C::COLS, B);
    cudaError_t e = ensure_smem(k, C::SMEM_BYTES, granted);
    if (e != cudaSuccess)
    {
        set_launch_failure_detail("fwd_pass1", "shared-memory attribute", grid.x, grid.y, C::THREADS, C::SMEM_BYTES);
        return e;
    }
    k<<<grid, C::THREADS, C::SMEM_BYTES, st>>>(in, tail, tail_next, T, tw.twN2, tw.lo, tw.hi, B, g.M, g.N1,
                                                  __builtin_ctz((unsigned)g.N2));
    e = cudaGetLastError();
    if (e != cudaSuccess)
        set_launch_failure_detail("fwd_pass1", "launch", grid.x, grid.y, C::THREADS, C::SMEM_BYTES);
    return e;
}

template <int N>
static cudaError_t fwd_pass2(const Geom &g, const Twiddles &tw, const float2 *T, float2 *ring, int rbi, int B,
                             cudaStream_t st)
{
    using C = TileCfg<N>;
    auto k = fwd_pass2_kernel<N>;
    static size_t granted[kMaxDevices] = {};
    dim3 grid(g.N2 / C::COLS, B);
    cudaError_t e = ensure_smem(k, C::SMEM_BYTES, granted);
    if (e != cudaSuccess)
    {
        set_launch_failure_detail("fwd_pass2", "shared-memory attribute", grid.x, grid.y, C::THREADS, C::SMEM_BYTES);
        return e;
    }
    k<<<grid, C::THREADS, C::SMEM_BYTES, st>>>(T, ring, tw.twN1, rbi, g.M, g.N2);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        set_launch_failure_detail("fwd_pass2", "launch", grid.x, grid.y, C::THREADS, C::SMEM_BYTES);
    return e;
}

template <int FMT>
static cudaError_t fwd_pass1_dispatch(const Geom &g, const Twiddles &tw, const void *in, const float2 *tail,
                                      float2 *tail_next, float2 *T, int B, cudaStream_t st)
{
    switch (g.N2)
    {
    case 16: return fwd_pass1<16, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 32: return fwd_pass1<32, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 64: return fwd_pass1<64, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 128: return fwd_pass1<128, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 256: return fwd_pass1<256, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 512: return fwd_pass1<512, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 1024: return fwd_pass1<1024, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 2048: return fwd_pass1<2048, FMT>(g, tw, in, tail, tail_next, T, B, st);
    case 4096: return fwd_pass1<4096, FMT>(g, tw, in, tail, tail_next, T, B, st);
    default: set_launch_failure_detail("fwd_pass1", "no tile for this size", g.N2, 0, 0, 0); return cudaErrorInvalidValue;
    }
}

static cudaError_t fwd_pass2_dispatch(const Geom &g, const Twiddles &tw, const float2 *T, float2 *ring, int rbi,
                                      int B, cudaStream_t st)
{
    switch (g.N1)
    {
    case 16: return fwd_pass2<16>(g, tw, T, ring, rbi, B, st);
    case 32: return fwd_pass2<32>(g, tw, T, ring, rbi, B, st);
    case 64: return fwd_pass2<64>(g, tw, T, ring, rbi, B, st);
    case 128: return fwd_pass2<128>(g, tw, T, ring, rbi, B, st);
    case 256: return fwd_pass2<256>(g, tw, T, ring, rbi, B, st);
    case 512: return fwd_pass2<512>(g, tw, T, ring, rbi, B, st);
    case 1024: return fwd_pass2<1024>(g, tw, T, ring, rbi, B, st);
    case 2048: return fwd_pass2<2048>(g, tw, T, ring, rbi, B, st);
    case 4096: return fwd_pass2<4096>(g, tw, T, ring, rbi, B, st);
    default: set_launch_failure_detail("fwd_pass2", "no tile for this size", g.N1, 0, 0, 0); return cudaErrorInvalidValue;
    }
}

cudaError_t launch_forward_p1(const Geom &g, const Twiddles &tw, int in_format, const void *in, const float2 *tail,
                              float2 *tail_next, float2 *T, int B, cudaStream_t st)
{
    switch (in_format)
    {
    case IN_U16: return fwd_pass1_dispatch<IN_U16>(g, tw, in, tail, tail_next, T, B, st);
    case IN_C64: return fwd_pass1_dispatch<IN_C64>(g, tw, in, tail, tail_next, T, B, st);
    case IN_I8: return fwd_pass1_dispatch<IN_I8>(g, tw, in, tail, tail_next, T, B, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_forward_p2(const Geom &g, const Twiddles &tw, const float2 *T, float2 *ring, int rbi, int B,
                              cudaStream_t st)
{
    return fwd_pass2_dispatch(g, tw, T, ring, rbi, B, st);
}

} // namespace msosm
