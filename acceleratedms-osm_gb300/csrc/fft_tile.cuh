// Tile FFT building blocks for the MS-OSM engine (sm_103a).
//
// A CTA transforms COLS independent length-N sequences ("columns") held in
// shared memory.  Stages are Stockham autosort stages, each thread owning BPT
// butterflies per stage with all R inputs in registers.  The default plan takes
// radix-8 stages (then 4 or 2 to finish); the "big" plan used by the persistent
// inverse transform takes two register stages of radix 16/32 (N = 512: 16 x 32,
// N = 1024: 32 x 32, N = 256: 16 x 16, N = 2048: 16 x 8 x 16, N = 4096: 16 x 16 x 16;
// see StageRadix).
// Register DFTs of radix 16 and 32 are composites of radix-8/4/2 kernels with
// compile-time twiddle constants.  The first stage may read straight from global memory through a
// loader functor and the last stage may hand its outputs to an epilogue functor
// instead of shared memory, so a pass touches shared memory only between stages.
//
// Shared layout: element (col, n) lives at n*LD + col with LD = COLS + 1.  A
// half-warp covers 16 consecutive columns of one row (column-fast mapping) or 16
// consecutive rows of one column (j-fast mapping, LD odd), so with the pad every
// access is the minimal two wavefronts for 256 bytes.
//
// Stage (R, Ns):  butterfly j (0 <= j < N/R), k = j mod Ns
//   in  : x[j + r*N/R] * W_{Ns*R}^{r*k}          (r = 0..R-1)
//   out : y[(j/Ns)*Ns*R + k + r*Ns] = DFT_R(in)[r]
// W_N^m = exp(SIGN * 2*pi*i*m/N); SIGN = -1 forward, +1 inverse (unnormalised),
// the cuFFT convention the reference's transforms use.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace msosm {

__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * (SIGN * i)
template <int SIGN>
__host__ __device__ __forceinline__ float2 cmul_si(float2 a)
{
    return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int SIGN>
__host__ __device__ __forceinline__ void dft2(float2 *v)
{
    float2 t = csub(v[0], v[1]);
    v[0] = cadd(v[0], v[1]);
    v[1] = t;
}

template <int SIGN>
__host__ __device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3)
{
    float2 a = cadd(v0, v2), b = csub(v0, v2);
    float2 c = cadd(v1, v3), d = cmul_si<SIGN>(csub(v1, v3));
    v0 = cadd(a, c);
    v2 = csub(a, c);
    v1 = cadd(b, d);
    v3 = csub(b, d);
}

template <int SIGN>
__host__ __device__ __forceinline__ void dft4(float2 *v)
{
    dft4<SIGN>(v[0], v[1], v[2], v[3]);
}

template <int SIGN>
__host__ __device__ __forceinline__ void dft8(float2 *v)
{
    const float c = 0.70710678118654752440f;
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<SIGN>(e0, e1, e2, e3);
    dft4<SIGN>(o0, o1, o2, o3);
    // W8^1 * o1 = c*(o.x - s*o.y, s*o.x + o.y); W8^2 = s*i; W8^3 * o = c*(-o.x - s*o.y, s*o.x - o.y)
    const float s = (float)SIGN;
    float2 t1 = make_float2(c * (o1.x - s * o1.y), c * (s * o1.x + o1.y));
    float2 t2 = cmul_si<SIGN>(o2);
    float2 t3 = make_float2(c * (-o3.x - s * o3.y), c * (s * o3.x - o3.y));
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
}

// ---- compile-time twiddles --------------------------------------------------
// cos/sin of 2*pi*e/R evaluated at compile time by Taylor series after reducing
// the angle to [-pi/4, pi/4] with the octant symmetries (|x| <= pi/4: 14 terms
// reach double precision), then rounded to float once.
constexpr double kTwoPi = 6.283185307179586476925286766559;
__host__ __device__ constexpr double taylor_sin(double x)
{
    double term = x, sum = x;
    for (int n = 1; n < 14; n++)
    {
        term *= -x * x / (double)((2 * n) * (2 * n + 1));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double taylor_cos(double x)
{
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 14; n++)
    {
        term *= -x * x / (double)((2 * n - 1) * (2 * n));
        sum += term;
    }
    return sum;
}
// angle 2*pi*e/R with e reduced mod R; octant o = floor(8e/R), remainder angle
__host__ __device__ constexpr double unit_cos(int e, int R)
{
    e = ((e % R) + R) % R;
    const int o8 = 8 * e; // angle = 2*pi*e/R = (pi/4) * (8e/R)
    const int oct = o8 / R;
    const double rem = (kTwoPi / 8.0) * ((double)(o8 - oct * R) / (double)R); // in [0, pi/4)
    // angle = oct*pi/4 + rem
    switch (oct)
    {
    case 0: return taylor_cos(rem);
    case 1: return taylor_sin(kTwoPi / 8.0 - rem);
    case 2: return -taylor_sin(rem);
    case 3: return -taylor_cos(kTwoPi / 8.0 - rem);
    case 4: return -taylor_cos(rem);
    case 5: return -taylor_sin(kTwoPi / 8.0 - rem);
    case 6: return taylor_sin(rem);
    default: return taylor_cos(kTwoPi / 8.0 - rem);
    }
}
__host__ __device__ constexpr double unit_sin(int e, int R) { return unit_cos(4 * e - R, 4 * R); } // sin t = cos(t - pi/2)

// x * W_R^E with W_R = exp(SIGN * 2*pi*i/R), E known at compile time.
template <int SIGN, int R, int E>
__host__ __device__ __forceinline__ float2 cmul_tw(float2 x)
{
    constexpr int e = ((E % R) + R) % R;
    if constexpr (e == 0)
        return x;
    else if constexpr (4 * e == R)
        return cmul_si<SIGN>(x);
    else if constexpr (2 * e == R)
        return make_float2(-x.x, -x.y);
    else if constexpr (4 * e == 3 * R)
        return cmul_si<-SIGN>(x);
    else
    {
        constexpr float c = (float)unit_cos(e, R);
        constexpr float s = (float)(SIGN * unit_sin(e, R));
        return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
    }
}

template <int R, int SIGN>
__host__ __device__ __forceinline__ void dftR(float2 *v);

// Composite R = A*B in registers (decimation in time, natural-order output):
//   u_b[ka] = DFT_A{ v[B*a + b] }_a * W_R^(b*ka),   X[ka + A*kb] = DFT_B{ u_b[ka] }_b
template <int R, int SIGN, int A, int b, int ka>
__host__ __device__ __forceinline__ void dft_twiddle_row(float2 *t)
{
    if constexpr (ka < A)
    {
        constexpr int B = R / A;
        (void)B;
        t[b * A + ka] = cmul_tw<SIGN, R, b * ka>(t[b * A + ka]);
        dft_twiddle_row<R, SIGN, A, b, ka + 1>(t);
    }
}
template <int R, int SIGN, int A, int b>
__host__ __device__ __forceinline__ void dft_first(const float2 *v, float2 *t)
{
    constexpr int B = R / A;
    if constexpr (b < B)
    {
        float2 u[A];
#pragma unroll
        for (int a = 0; a < A; a++)
            u[a] = v[B * a + b];
        dftR<A, SIGN>(u);
#pragma unroll
        for (int k = 0; k < A; k++)
            t[b * A + k] = u[k];
        dft_twiddle_row<R, SIGN, A, b, 0>(t);
        dft_first<R, SIGN, A, b + 1>(v, t);
    }
}
template <int R, int SIGN, int A>
__host__ __device__ __forceinline__ void dft_composite(float2 *v)
{
    constexpr int B = R / A;
    float2 t[R];
    dft_first<R, SIGN, A, 0>(v, t);
#pragma unroll
    for (int ka = 0; ka < A; ka++)
    {
        float2 w[B];
#pragma unroll
        for (int b = 0; b < B; b++)
            w[b] = t[b * A + ka];
        dftR<B, SIGN>(w);
#pragma unroll
        for (int kb = 0; kb < B; kb++)
            v[ka + A * kb] = w[kb];
    }
}

template <int R, int SIGN>
__host__ __device__ __forceinline__ void dftR(float2 *v)
{
    if constexpr (R == 8)
        dft8<SIGN>(v);
    else if constexpr (R == 4)
        dft4<SIGN>(v);
    else if constexpr (R == 2)
        dft2<SIGN>(v);
    else if constexpr (R == 16)
        dft_composite<16, SIGN, 8>(v); // 8 x 2
    else if constexpr (R == 32)
        dft_composite<32, SIGN, 8>(v); // 8 x 4
    else
        dft_composite<R, SIGN, 8>(v); // 8 x R/8
}

// Radix of the stage that starts with sub-transform size Ns.  The default plan is
// radix 8 (then 4 or 2); the BIG plan takes two stages of radix 16/32 where it can
// (threads then hold 32 values, for 256-thread tiles of 8192 points).
template <int N, int Ns, bool BIG = false>
struct StageRadix
{
    static constexpr int rem = N / Ns;
    static constexpr int big = (N == 512)    ? (Ns == 1 ? 16 : 32)
                               : (N == 1024) ? 32
                               : (N == 2048) ? (Ns == 1 ? 16 : (Ns == 16 ? 8 : 16))
                               : (N == 4096) ? 16
                               : (N == 256)  ? 16
                               : (N == 128)  ? (Ns == 1 ? 8 : 16)
                                             : (rem >= 8 ? 8 : rem);
    static constexpr int value = BIG ? (big < rem ? big : rem) : ((rem >= 8) ? 8 : rem);
};

template <int N, int COLS>
struct TileGeom
{
    static constexpr int LD = COLS + 1;
    static constexpr int SMEM_ELEMS = N * LD;
};

// A destination may take a butterfly's R outputs at once (store_group<R, Ns>)
// instead of one at a time, e.g. to derive per-output factors by recurrence.
template <class T, class = void>
struct HasStoreGroup
{
    static constexpr bool value = false;
};
template <class T>
struct HasStoreGroup<T, decltype((void)&T::template store_group<2, 1>, void())>
{
    static constexpr bool value = true;
};

// A source may fill a whole stage's inputs at once (load_stage), e.g. to issue all
// of a thread's independent global loads before using any of them.
template <class T, class = void>
struct HasLoadStage
{
    static constexpr bool value = false;
};
template <class T>
struct HasLoadStage<T, decltype((void)&T::template load_stage<1, 2, 1, 1, 32>, void())>
{
    static constexpr bool value = true;
};

// A final-stage destination may ask for the "j-fast" thread mapping (J_FAST):
// consecutive lanes take consecutive butterflies of one column instead of one
// butterfly of consecutive columns, so a column's outputs leave as contiguous runs.
// Its stage twiddles then come from a [r][k] table (tw_last[r*Ns + k] = W_N^(r*k)),
// which consecutive k read without bank conflicts.
template <class T, class = void>
struct IsJFast
{
    static constexpr bool value = false;
};
template <class T>
struct IsJFast<T, decltype((void)T::J_FAST, void())>
{
    static constexpr bool value = T::J_FAST;
};

// Ns of the last stage of a plan (the stage with Ns * R == N).
template <int N, int Ns, bool BIG, bool DONE = (Ns * StageRadix<N, Ns, BIG>::value == N)>
struct LastNs
{
    static constexpr int value = LastNs<N, Ns * StageRadix<N, Ns, BIG>::value, BIG>::value;
};
template <int N, int Ns, bool BIG>
struct LastNs<N, Ns, BIG, true>
{
    static constexpr int value = Ns;
};

// Shared-memory source/destination for a stage.
template <int N, int COLS>
struct SmemIO
{
    float2 *sm;
    __device__ __forceinline__ float2 load(int col, int n) const { return sm[n * TileGeom<N, COLS>::LD + col]; }
    __device__ __forceinline__ void store(int col, int n, float2 v) const { sm[n * TileGeom<N, COLS>::LD + col] = v; }
};

// One Stockham stage.  SRC/DST provide load(col, n) / store(col, n, v).
// SRC_SMEM / DST_SMEM say whether they alias the CTA's shared tile, which decides
// the barriers.  tw: W_N^m table (SIGN applied), N entries, shared memory;
// tw_last: the [r][k] table of a j-fast final stage.
template <int N, int COLS, int THREADS, int SIGN, int Ns, bool SRC_SMEM, bool DST_SMEM, bool BIG, class SRC, class DST>
__device__ __forceinline__ void fft_stage(const SRC &src, const DST &dst, const float2 *__restrict__ tw,
                                          const float2 *__restrict__ tw_last = nullptr)
{
    constexpr int R = StageRadix<N, Ns, BIG>::value;
    constexpr int NB = COLS * N / R;
    static_assert(NB % THREADS == 0, "butterflies must divide evenly over threads");
    constexpr int BPT = NB / THREADS;
    constexpr int STRIDE = N / R;
    constexpr int TWSTEP = N / (Ns * R);
    constexpr bool JF = IsJFast<DST>::value;
    static_assert(!JF || Ns * R == N, "the j-fast mapping is for a final stage");
    float2 v[BPT][R];
    if constexpr (Ns == 1 && HasLoadStage<SRC>::value)
    {
        // butterfly i of this thread: col = beta % COLS, j = beta / COLS, inputs j + r*STRIDE
        src.template load_stage<BPT, R, STRIDE, COLS, THREADS>(v);
    }
    else
    {
#pragma unroll
        for (int i = 0; i < BPT; i++)
        {
            const int beta = threadIdx.x + i * THREADS;
            const int col = JF ? beta / STRIDE : beta % COLS;
            const int j = JF ? beta % STRIDE : beta / COLS;
            const int k = j & (Ns - 1);
#pragma unroll
            for (int r = 0; r < R; r++)
            {
                float2 a = src.load(col, j + r * STRIDE);
                if constexpr (Ns > 1)
                {
                    if (r > 0)
                        a = cmul(a, JF ? tw_last[r * Ns + k] : tw[r * k * TWSTEP]);
                }
                v[i][r] = a;
            }
        }
    }
    if constexpr (SRC_SMEM && DST_SMEM)
        __syncthreads();
#pragma unroll
    for (int i = 0; i < BPT; i++)
    {
        dftR<R, SIGN>(v[i]);
        const int beta = threadIdx.x + i * THREADS;
        const int col = JF ? beta / STRIDE : beta % COLS;
        const int j = JF ? beta % STRIDE : beta / COLS;
        const int k = j & (Ns - 1);
        const int base = (j / Ns) * Ns * R + k;
        if constexpr (HasStoreGroup<DST>::value)
            dst.template store_group<R, Ns>(col, base, v[i]); // outputs base + r*Ns, r = 0..R-1
        else
        {
#pragma unroll
            for (int r = 0; r < R; r++)
                dst.store(col, base + r * Ns, v[i][r]);
        }
    }
    if constexpr (DST_SMEM)
        __syncthreads();
}

// Run all stages from Ns onwards.  FIRST: the stage at Ns reads from `first`
// (global loader) instead of shared memory.  The final stage hands its outputs to
// `last` (epilogue) instead of shared memory.
// EPI_IN_SMEM: the epilogue writes into the shared tile too, so the final stage
// takes a barrier between its loads and its outputs and another after them.
template <int N, int COLS, int THREADS, int SIGN, int Ns, bool FIRST_FROM_LOADER, bool BIG = false,
          bool EPI_IN_SMEM = false, class LOADER, class EPI>
__device__ __forceinline__ void fft_stages(float2 *sm, const float2 *tw, const LOADER &first, const EPI &last,
                                           const float2 *tw_last = nullptr)
{
    constexpr int R = StageRadix<N, Ns, BIG>::value;
    constexpr bool IS_LAST = (Ns * R == N);
    SmemIO<N, COLS> io{sm};
    if constexpr (FIRST_FROM_LOADER && IS_LAST)
        fft_stage<N, COLS, THREADS, SIGN, Ns, false, EPI_IN_SMEM, BIG>(first, last, tw, tw_last);
    else if constexpr (FIRST_FROM_LOADER)
        fft_stage<N, COLS, THREADS, SIGN, Ns, false, true, BIG>(first, io, tw);
    else if constexpr (IS_LAST)
        fft_stage<N, COLS, THREADS, SIGN, Ns, true, EPI_IN_SMEM, BIG>(io, last, tw, tw_last);
    else
        fft_stage<N, COLS, THREADS, SIGN, Ns, true, true, BIG>(io, io, tw);
    if constexpr (!IS_LAST)
        fft_stages<N, COLS, THREADS, SIGN, Ns * R, false, BIG, EPI_IN_SMEM>(sm, tw, first, last, tw_last);
}

// Twiddle table W_N^m (m < N) into shared memory from a global table of W_N.
template <int N, int THREADS>
__device__ __forceinline__ void load_twiddles(float2 *tw_sm, const float2 *__restrict__ tw_g)
{
    for (int i = threadIdx.x; i < N; i += THREADS)
        tw_sm[i] = __ldg(tw_g + i);
}

} // namespace msosm
