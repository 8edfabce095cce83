// Persistent inverse transform: all (DM, window) transforms of one call in one
// launch, the pass-1 -> pass-2 intermediate kept in a small ring of transform
// slots that stays in L2.
//
// Work items, taken from a global ticket counter in this order:
//   block q = 0 .. G+LAG-1 holds  [ P1(q, tile 0..n1t-1) | P2(q-LAG, tile 0..n2t-1) ]
// P1(f, c): gather x response + N2-point column transforms of transform f,
//           column tile c, into slot f mod S of the ring.
// P2(f, r): N1-point row transforms of row tile r of transform f + the
//           discard / encode / fold epilogue.
// Dependencies, through per-slot completion counters (monotone over the launch):
//   P2(f)  needs all P1(f)              : p1_done[f mod S] >= (f/S + 1) * n1t
//   P1(f)  needs slot f mod S released  : p2_done[f mod S] >= (f/S) * n2t
// Every item waited on holds a smaller ticket (S > LAG).  A CTA holds its current
// item and the next ticket (fetched early to hide the atomic's latency), and starts
// that ticket only after finishing the current item, which has a smaller ticket; so
// the smallest unfinished ticket is always some CTA's current item, with every
// dependence finished: no deadlock whatever the residency.  Waits are nevertheless
// bounded by %globaltimer; on timeout the kernel raises an error flag, every later
// wait returns at once and the host reports the failure.
#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "msosm_common.cuh"
#include "msosm_persist.cuh"
#include "umma.cuh"

namespace msosm {

namespace {

constexpr int P_POINTS = 8192;
constexpr int P_THREADS = 256; // 32 points per thread: radix-16/32 stages in registers

template <int N>
struct PCfg
{
    static constexpr int COLS = P_POINTS / N;
    static constexpr int LD = COLS + 1;
    static constexpr int SMEM_DATA = N * LD;
};

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Called by one thread: wait until *cnt >= target.  False if the launch failed
// meanwhile (another CTA raised the error flag) or this wait timed out (raises it).
// One acquire load when the count is already there (the common case); otherwise
// polls with volatile loads (served by L2, no L1 invalidation), then one acquire
// load orders the caller's later reads after the observed count.
__device__ __forceinline__ bool wait_count(const unsigned *cnt, unsigned target, int *err,
                                           unsigned long long timeout_ns)
{
    if (ld_acquire(cnt) >= target)
        return true;
    const volatile unsigned *vc = cnt;
    const uint64_t t0 = global_ns();
    unsigned backoff = 32;
    while (*vc < target)
    {
        if (*(volatile int *)err)
            return false;
        if (global_ns() - t0 > timeout_ns)
        {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(backoff);
        if (backoff < 1024)
            backoff *= 2;
    }
    (void)ld_acquire(cnt);
    return true;
}

// Streaming read-only loads that skip L1 allocation, leaving L1 to the twiddle tables.
__device__ __forceinline__ float2 ld_na(const float2 *p)
{
    float2 v;
    asm("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_na(const uint16_t *p)
{
    unsigned short v;
    asm("ld.global.nc.L1::no_allocate.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return (int)v;
}

template <class HOOK>
struct PInvLoader
{
    const float2 *ring;
    const float2 *Hd;
    const uint16_t *dl;
    int c0, N1, F, fbs, rb;
    HOOK hook; // run once all of this thread's loads are issued
    // The first stage's inputs in two waves: every delay, then every spectrum and
    // response value, so the delay -> spectrum dependences overlap across elements.
    template <int BPT, int R, int STRIDE, int COLS, int THREADS>
    __device__ __forceinline__ void load_stage(float2 (&v)[BPT][R]) const
    {
        int slot[BPT][R];
#pragma unroll
        for (int i = 0; i < BPT; i++)
        {
            const int beta = threadIdx.x + i * THREADS;
            const int n0 = c0 + beta % COLS + N1 * (beta / COLS);
#pragma unroll
            for (int r = 0; r < R; r++)
                slot[i][r] = ld_na(dl + n0 + N1 * STRIDE * r);
        }
#pragma unroll
        for (int i = 0; i < BPT; i++)
        {
            const int beta = threadIdx.x + i * THREADS;
            const int n0 = c0 + beta % COLS + N1 * (beta / COLS);
#pragma unroll
            for (int r = 0; r < R; r++)
            {
                const int n = n0 + N1 * STRIDE * r;
                int s = rb - slot[i][r];
                if (s < 0)
                    s += fbs;
                v[i][r] = cmul(ld_na(ring + (size_t)s * F + n), ld_na(Hd + n));
            }
        }
        hook();
    }
};

// Pass-1 outputs into the slot, column-major: element (n1, k2) at n1*N2 + k2, so
// that pass 2 reads a row tile's inputs as 128-byte runs straight into registers.
// The last stage runs j-fast, so a column's outputs leave as contiguous runs too.
struct PStoreT
{
    static constexpr bool J_FAST = true;
    float2 *T;
    const float2 *lo, *hi;
    int c0, N2;
    unsigned n2_mask;
    int n2_shift;
    // Last stage: outputs k2 = base + r*Ns.  W_F^(n1*k2) = W_F^(n1*base) * (W_F^(n1*Ns))^r,
    // two table lookups per butterfly and a product chain instead of two per output.
    template <int R, int Ns>
    __device__ __forceinline__ void store_group(int col, int base, const float2 *v) const
    {
        const int n1 = c0 + col;
        float2 w = twiddle_F(lo, hi, (unsigned)(n1 * base), n2_mask, n2_shift);
        const float2 step = twiddle_F(lo, hi, (unsigned)(n1 * Ns), n2_mask, n2_shift);
        float2 *dst = T + (size_t)n1 * N2 + base;
#pragma unroll
        for (int r = 0; r < R; r++)
        {
            dst[Ns * r] = cmul(v[r], w);
            w = cmul(w, step);
        }
    }
};

// Pass-2 inputs of row tile r0 .. r0+COLS-1 from the column-major slot: element
// (row r0 + col, n1) at n1*N2 + r0 + col.  L2-resident, so loaded with .cg.
template <class HOOK>
struct PTLoader
{
    const float2 *Ts;
    int r0, N2;
    HOOK hook; // as in PInvLoader
    template <int BPT, int R, int STRIDE, int COLS, int THREADS>
    __device__ __forceinline__ void load_stage(float2 (&v)[BPT][R]) const
    {
#pragma unroll
        for (int i = 0; i < BPT; i++)
        {
            const int beta = threadIdx.x + i * THREADS;
            const float2 *p = Ts + r0 + beta % COLS + (size_t)N2 * (beta / COLS);
#pragma unroll
            for (int r = 0; r < R; r++)
                v[i][r] = __ldcg(p + (size_t)N2 * STRIDE * r);
        }
        hook();
    }
};

// Placeholder first-stage source of a pass whose first stage reads shared memory.
struct PNoLoad
{
};

// Last pass-2 stage: outputs k1 = base + r*Ns of row (r0 + col); only k1 >= N1/2
// (window samples M..2M-1) survive, i.e. r >= R/2.  Series outputs go straight to
// global memory; for the fold, |v|^2 is parked in a shared tile s_p[(k1 - N1/2)*COLS
// + col], in time order, for fold_tile() to bin.
template <int MODE, int COLS>
struct PEpilogue
{
    float2 *out_c64;
    uint32_t *out_u16;
    float *out_pow;
    const float *pair_pow;
    float *s_p;
    int r0, N1, N2;
    float scale;
    template <int R, int Ns>
    __device__ __forceinline__ void store_group(int col, int base, const float2 *v) const
    {
#pragma unroll
        for (int r = R / 2; r < R; r++)
        {
            const int k1h = base + r * Ns - (N1 >> 1);
            float2 x = v[r];
            // fold-only: |x|^2 is binned unscaled and the bins take the 1/F^2 at the
            // flush (a power of two: the same floats as scaling each sample)
            if constexpr (MODE != OUT_FOLD)
            {
                x.x *= scale;
                x.y *= scale;
            }
            const int o = r0 + col + N2 * k1h;
            if constexpr ((MODE & OUT_C64) != 0)
                out_c64[o] = x;
            if constexpr ((MODE & OUT_U16) != 0)
                out_u16[o] = encode_u16(x);
            if constexpr ((MODE & OUT_POW) != 0)
                out_pow[o] = x.x * x.x + x.y * x.y;
            if constexpr ((MODE & OUT_PAIR) != 0)
            {
                // 2-pol intensity sqrt(|a|^2 + |b|^2) (calculateIntensity_kernel, gpu_kernel.cu:430-436)
                s_p[k1h * COLS + col] = sqrtf(__ldcs(pair_pow + o) + (x.x * x.x + x.y * x.y));
            }
            else if constexpr ((MODE & OUT_FOLD) != 0)
                s_p[k1h * COLS + col] = x.x * x.x + x.y * x.y;
        }
    }
};

// One phase bin of the per-CTA accumulator: the sum and the count side by side, so
// that the whole shared layout sits at compile-time offsets.
struct BinAcc
{
    float sum;
    unsigned cnt;
};

// Bin the staged tile: each thread takes runs of G consecutive time samples; a
// run whose first and last samples share a phase bin (runs are far shorter than a
// period, and phase is monotone within a run) is summed in registers and lands as
// one shared atomic; other runs go sample by sample.  Zero samples are skipped as
// foldDataPhase_kernel does.
template <int COLS, int HALF, int THREADS = P_THREADS>
__device__ __forceinline__ void fold_tile(const float *s_p, BinAcc *s_bins, uint64_t ph_b,
                                          uint64_t dphase, unsigned K, int r0, int N2)
{
    constexpr int SAMPLES = COLS * HALF;
    constexpr int PER_T = SAMPLES / THREADS;
    constexpr int G = PER_T < COLS ? PER_T : COLS;
    static_assert(SAMPLES % THREADS == 0 && PER_T % G == 0, "fold tile shape");
#pragma unroll
    for (int g0 = 0; g0 < PER_T; g0 += G)
    {
        const int e0 = threadIdx.x * PER_T + g0;
        const int k1h = e0 / COLS, c = e0 % COLS;
        const uint64_t ph0 = ph_b + (uint64_t)(r0 + c + N2 * k1h) * dphase;
        const unsigned bf = phase_bin(ph0, K);
        const unsigned bl = phase_bin(ph0 + (uint64_t)(G - 1) * dphase, K);
        float p[G];
#pragma unroll
        for (int i = 0; i < G; i++)
            p[i] = s_p[e0 + i];
        if (bf == bl)
        {
            float s = 0.0f;
            unsigned n = 0;
#pragma unroll
            for (int i = 0; i < G; i++)
            {
                s += p[i];
                n += (p[i] != 0.0f);
            }
            if (n)
            {
                atomicAdd(&s_bins[bf].sum, s);
                atomicAdd(&s_bins[bf].cnt, n);
            }
        }
        else
        {
#pragma unroll
            for (int i = 0; i < G; i++)
            {
                if (p[i] != 0.0f)
                {
                    const unsigned bi = phase_bin(ph0 + (uint64_t)i * dphase, K);
                    atomicAdd(&s_bins[bi].sum, p[i]);
                    atomicAdd(&s_bins[bi].cnt, 1u);
                }
            }
        }
    }
}

// Per-CTA fold accumulator: the shared per-bin sums of one DM trial, carried over
// the CTA's consecutive pass-2 items of that trial and flushed to the global
// double / u64 sums when the trial changes and at the end.  Each thread flushes and
// clears the bins it owns; the callers' barriers order this against fold_tile().
template <int THREADS = P_THREADS>
__device__ __forceinline__ void fold_flush(BinAcc *s_bins, const FoldArgs &fa, int d, double scale2)
{
    double *gs = fa.sum + (size_t)d * fa.K;
    unsigned long long *gc = fa.cnt + (size_t)d * fa.K;
    for (unsigned i = threadIdx.x; i < fa.K; i += THREADS)
    {
        const BinAcc v = s_bins[i];
        if (v.cnt)
        {
            atomicAdd(gs + i, (double)v.sum * scale2);
            atomicAdd(gc + i, (unsigned long long)v.cnt);
            s_bins[i] = BinAcc{0.0f, 0u};
        }
    }
}

// Transform index gi -> (DM trial d, window b): DM trials in groups of G, window-major
// inside a group (G = 1: DM-major), the last group holding the D mod G remaining trials.
// Consecutive transforms then gather from nearly the same spectra-ring lines (neighbouring
// trials' block delays differ by at most a step), which L2 serves to the whole group.
__device__ __forceinline__ void transform_dm_window(unsigned gi, unsigned B, unsigned D, unsigned G, int &d, int &b)
{
    const unsigned full = D / G, per = G * B;
    const unsigned grp = gi / per;
    if (grp < full)
    {
        const unsigned r = gi - grp * per;
        b = (int)(r / G);
        d = (int)(grp * G + r % G);
    }
    else
    {
        const unsigned rem = D - full * G, r = gi - full * per;
        b = (int)(r / rem);
        d = (int)(full * G + r % rem);
    }
}

// The completion count ticket t's item waits on and the value it needs: P1(f) waits
// for slot f mod S to be released by P2(f - S), P2(f) for all P1(f).  False if t
// holds no item of the launch's transforms.
template <int n1t, int n2t>
__device__ __forceinline__ bool ticket_dependence(const PersistArgs &a, long long total, unsigned t,
                                                  const unsigned *&cnt, unsigned &target)
{
    constexpr int per_block = n1t + n2t;
    if ((long long)t >= total)
        return false;
    const long long q = t / per_block;
    const int w = (int)(t % per_block);
    const bool p1 = w < n1t;
    const long long f = p1 ? q : q - a.lag;
    if (f < 0 || f >= a.G)
        return false;
    const unsigned slot = (unsigned)f % (unsigned)a.S; // f < 2^31 (host check)
    const unsigned gen = (unsigned)f / (unsigned)a.S;
    cnt = p1 ? a.p2_done + slot : a.p1_done + slot;
    target = p1 ? gen * n2t : (gen + 1) * n1t;
    return true;
}

// Thread 0, during an item, once its loads are issued: look once (acquire load) at
// the dependence of the next ticket it holds.  Returns that ticket if the dependence
// is already met (counts only grow, so it stays met), else ~0u.  The acquire then
// orders the next item's reads as judge_ticket's wait would, and the item boundary
// skips that round trip.
template <int n1t, int n2t>
__device__ __forceinline__ unsigned ticket_precheck(const PersistArgs &a, long long total, unsigned t)
{
    const unsigned *cnt;
    unsigned target;
    if (!ticket_dependence<n1t, n2t>(a, total, t, cnt, target))
        return ~0u;
    return ld_acquire(cnt) >= target ? t : ~0u;
}

// Thread 0 of a CTA: take the ticket it holds (fetching the next one, whose latency
// overlaps the item), wait for the item's dependences, and return the verdict:
// -1 stop (tickets exhausted; or, with stop_on_error, the launch failed), 0 skip
// (outside the launch's transforms, or a failed wait), 1 run.  ready_t: a ticket
// whose dependence ticket_precheck() already saw met (no wait for it).
template <int n1t, int n2t>
__device__ __forceinline__ int judge_ticket(const PersistArgs &a, long long total, unsigned &held, unsigned &t_out,
                                            bool stop_on_error, unsigned ready_t = ~0u)
{
    const unsigned t = held;
    t_out = t;
    if ((long long)t >= total || (stop_on_error && *(volatile int *)a.err))
        return -1;
    held = atomicAdd(a.ticket, 1u);
    const unsigned *cnt;
    unsigned target;
    if (!ticket_dependence<n1t, n2t>(a, total, t, cnt, target))
        return 0;
    if (t == ready_t)
        return 1;
    return wait_count(cnt, target, a.err, a.timeout_ns) ? 1 : 0;
}

// THREADS x 2 CTAs per SM; BIG: radix-16/32 register stages (32 values per thread at
// 256 threads), else radix-8 stages (16 values per thread at 512 threads).
template <int N1, int N2, int MODE, int THREADS, bool BIG>
__global__ void __launch_bounds__(THREADS, 2) inv_persistent_kernel(PersistArgs a)
{
    using C1 = PCfg<N2>; // pass 1: columns of length N2
    using C2 = PCfg<N1>; // pass 2: rows of length N1
    constexpr int DATA = (C1::SMEM_DATA > C2::SMEM_DATA) ? C1::SMEM_DATA : C2::SMEM_DATA;
    constexpr int n1t = N1 / C1::COLS; // P1 items per transform
    constexpr int n2t = N2 / C2::COLS; // P2 items per transform
    constexpr int per_block = n1t + n2t;
    constexpr int F = N1 * N2;
    constexpr int M = F / 2;
    constexpr int NSL = LastNs<N2, 1, BIG>::value;     // pass 1, last stage: Ns
    constexpr int R2F = StageRadix<N1, 1, BIG>::value; // pass 2, first stage: radix
    // two-stage pass 1 (radix R1F then the last stage): its only stage twiddles are
    // the last stage's, so the [r][k] table replaces the W_{N2} table
    constexpr bool P1_TWO = NSL == StageRadix<N2, 1, BIG>::value;
    constexpr bool FOLD = (MODE & OUT_FOLD) != 0;
    // fold-only bins hold unscaled |x|^2: 1/F^2 at the flush (exact, F a power of two)
    constexpr double FLUSH_SCALE2 = (MODE == OUT_FOLD) ? 1.0 / ((double)F * (double)F) : 1.0;
    static_assert(C2::COLS * (N1 / 2) <= 2 * DATA, "fold staging fits in the data tile");
    extern __shared__ float2 smem[];
    float2 *sm = smem;
    float2 *tw2 = smem + DATA;                // W_{N1}: pass-2 stages
    float2 *tw1L = tw2 + N1;                  // pass-1 last stage, [r][k] = W_{N2}^(r*k)
    float2 *tw1 = P1_TWO ? tw1L : tw1L + N2;  // W_{N2}: pass-1 middle stages
    // fold staging tile (C2::COLS * N1/2 floats) in the data tile: pass 2's last stage
    // reads all its inputs before the epilogue writes it
    float *s_p = reinterpret_cast<float *>(sm);
    BinAcc *s_bins = reinterpret_cast<BinAcc *>(tw1L + (P1_TWO ? N2 : 2 * N2)); // K bins
    // (ticket, verdict) published by thread 0; double-buffered by iteration parity
    // so a skipped item (no barrier inside) cannot overwrite what slow threads read
    __shared__ unsigned s_ticket[2];
    __shared__ int s_verdict[2];

    for (int i = threadIdx.x; i < N2; i += THREADS)
    {
        const int r = i / NSL, k = i % NSL; // r*k < N2
        tw1L[i] = __ldg(a.tw.twN2 + r * k);
        if constexpr (!P1_TWO)
            tw1[i] = __ldg(a.tw.twN2 + i);
    }
    for (int i = threadIdx.x; i < N1; i += THREADS)
        tw2[i] = __ldg(a.tw.twN1 + i);
    if constexpr (FOLD)
    {
        for (unsigned i = threadIdx.x; i < a.fold.K; i += THREADS)
            s_bins[i] = BinAcc{0.0f, 0u};
    }
    int fold_d = -1; // the DM trial s_bins holds (uniform over the CTA)

    const long long total = (a.G + a.lag) * (long long)per_block;
    const int B = a.B;
    unsigned held = 0;    // thread 0: the ticket of the next item, fetched one item ahead
    unsigned ready = ~0u; // thread 0: that ticket if its dependence was seen met during the item
    if (threadIdx.x == 0)
        held = atomicAdd(a.ticket, 1u);
    // thread 0, once an item's first-stage loads are issued (the next ticket's atomic
    // has returned by then): precheck the next item's dependence
    auto precheck = [&]() {
        if (threadIdx.x == 0)
            ready = ticket_precheck<n1t, n2t>(a, total, held);
    };
    for (unsigned it = 0;; it++)
    {
        const int par = it & 1;
        if (threadIdx.x == 0)
        {
            unsigned t;
            s_verdict[par] = judge_ticket<n1t, n2t>(a, total, held, t, false, ready);
            s_ticket[par] = t;
            ready = ~0u;
        }
        __syncthreads(); // also fences the previous item's shared-memory use
        const int verdict = s_verdict[par];
        if (verdict < 0)
            break;
        if (verdict == 0)
            continue;
        const long long t = s_ticket[par];
        const long long q = t / per_block;
        const int w = (int)(t % per_block);
        const bool is_p1 = w < n1t;
        const long long f = is_p1 ? q : q - a.lag;
        const int slot = (int)((unsigned)f % (unsigned)a.S);
        float2 *Ts = a.T + (size_t)slot * F;
        const long long gi = a.g0 + f;
        int d, b;
        transform_dm_window((unsigned)gi, (unsigned)B, (unsigned)a.D, (unsigned)a.dm_group, d, b);
        if (is_p1)
        {
            const int c0 = w * C1::COLS;
            PInvLoader<decltype(precheck)> ld{a.ring, a.H + (size_t)d * F, a.delays + (size_t)d * F, c0, N1, F, a.fbs,
                                              a.rbi + b, precheck};
            PStoreT st{Ts, a.tw.lo, a.tw.hi, c0, N2, (unsigned)(N2 - 1), __builtin_ctz((unsigned)N2)};
            fft_stages<N2, C1::COLS, THREADS, +1, 1, true, BIG>(sm, tw1, ld, st, tw1L);
            // publish: the barrier orders every thread's stores before one thread's
            // gpu-scope release reduction (release is cumulative) on the count.  Warp 1
            // publishes, so that its wait for the stores does not delay thread 0's
            // next ticket.
            __syncthreads();
            if (threadIdx.x == 32)
                asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.p1_done + slot) : "memory");
        }
        else
        {
            const int r0 = (w - n1t) * C2::COLS;
            if constexpr (FOLD)
            {
                if (d != fold_d)
                {
                    if (fold_d >= 0)
                        fold_flush<THREADS>(s_bins, a.fold, fold_d, FLUSH_SCALE2);
                    fold_d = d;
                }
            }
            // first stage straight from the slot; its closing barrier means every
            // thread holds its inputs, so the slot may be refilled
            SmemIO<N1, C2::COLS> io{sm};
            fft_stage<N1, C2::COLS, THREADS, +1, 1, false, true, BIG>(
                PTLoader<decltype(precheck)>{Ts, r0, N2, precheck}, io, tw2);
            if (threadIdx.x == 32) // release: every thread's reads of the slot precede the count
                asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.p2_done + slot) : "memory");
            const size_t row = ((size_t)d * B + b) * M;
            PEpilogue<MODE, C2::COLS> ep{a.out_c64 ? a.out_c64 + row : nullptr,
                                         a.out_u16 ? a.out_u16 + row : nullptr,
                                         a.out_pow ? a.out_pow + row : nullptr,
                                         a.pair_pow ? a.pair_pow + row : nullptr,
                                         s_p,
                                         r0,
                                         N1,
                                         N2,
                                         1.0f / (float)F};
            fft_stages<N1, C2::COLS, THREADS, +1, R2F, false, BIG, FOLD>(sm, tw2, PNoLoad{}, ep);
            if constexpr (FOLD)
            {
                fold_tile<C2::COLS, N1 / 2, THREADS>(s_p, s_bins,
                                            fold_phase0(a.fold) + (uint64_t)((uint64_t)b * (uint64_t)M) * a.fold.dphase,
                                            a.fold.dphase, a.fold.K, r0, N2);
                // s_p and the bins are next touched after the next ticket barrier
            }
        }
    }
    if constexpr (FOLD)
    {
        if (fold_d >= 0)
            fold_flush<THREADS>(s_bins, a.fold, fold_d, FLUSH_SCALE2);
    }
}

// ---- split-precision transform on the tensor cores --------------------------------
// F = 2^18 (N1 = N2 = 512).  Each 512-point DFT of a pass is split as n = 32a + b,
// k = ka + 16*kb:
//   step 1 (registers): y[b][ka] = sum_a x[32a + b] W_16^(a*ka), z = y * W_512^(b*ka)
//   step 2 (tensor cores): X[ka + 16*kb] = sum_b z[b][ka] W_32^(b*kb)
// Step 2 is a real GEMM per item of 16 vectors: A rows m = 16*ka + v (two 128-row
// tiles), K = (b, re/im) = 64, B = the real 64 x 64 form of W_32, D = 64 (pass 1)
// or the 32 kept columns kb >= 16 (pass 2: only outputs k1 >= 256 survive the
// discard).  FP32 values are split into 16-bit hi + lo parts (BF16 or FP16) and
// D = Ahi*Bhi + Alo*Bhi + Ahi*Blo accumulates in FP32 in tensor memory: 24 MMAs of
// 128 x N x 16 per item.  FP16 operands are scaled by powers of two chosen from a
// running bound on the spectra so that no value exceeds the FP16 range; the scale is
// taken back out in FP32 afterwards (exact).
//
// The pass-1 -> pass-2 slot is row-major here: element (k2, n1) at k2*512 + n1.
// Shared memory (1024-byte aligned base): A hi tiles (2 x 16 KB), A lo tiles, B hi
// (8 KB), B lo, the step-1 twiddle tables of both passes W[ka][i][bp] =
// W_512^((2bp+i)*ka) * scale (4 KB each), fold bins.  Fold staging reuses the A tiles
// once an item's MMAs are done.
constexpr int TC_N = 512;                  // sub-transform length of both passes
constexpr int TC_COLS = 16;                // vectors per item
constexpr uint32_t TC_A_HI = 0;            // two 128-row tiles, 16 KB each
constexpr uint32_t TC_A_LO = 32768;
constexpr uint32_t TC_B_HI = 65536;        // 64 rows x 128 B
constexpr uint32_t TC_B_LO = 73728;
constexpr uint32_t TC_W1 = 81920;          // 512 float2
constexpr uint32_t TC_W2 = 86016;
constexpr uint32_t TC_BINS = 90112;
constexpr uint32_t TC_TMEM_COLS = 128;     // two 64-column FP32 accumulator tiles

template <bool BF16>
__device__ __forceinline__ void split_hi_lo(float2 z, uint32_t &hi, uint32_t &lo)
{
    if constexpr (BF16)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(z.x, z.y);
        const float2 hf = __bfloat1622float2(h);
        const __nv_bfloat162 l = __floats2bfloat162_rn(z.x - hf.x, z.y - hf.y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    }
    else
    {
        const __half2 h = __floats2half2_rn(z.x, z.y);
        const float2 hf = __half22float2(h);
        const __half2 l = __floats2half2_rn(z.x - hf.x, z.y - hf.y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    }
}

// Step 1 of either pass for this thread's two vectors' columns b = 2bp, 2bp+1:
// 16-point DFTs over a, twiddles from W[ka][i][bp], hi/lo split, stored as A rows
// m = 16*ka + v at K = 4bp .. 4bp+3 (row_off: this thread's byte offset in row v of
// tile 0; row m lands at tile ka/8, 2048*(ka%8) bytes further).
template <bool BF16>
__device__ __forceinline__ void tc_step1(float2 (&x)[2][16], const float2 *__restrict__ W, int bp, uint32_t row_off,
                                         unsigned char *sA_hi, unsigned char *sA_lo)
{
    dftR<16, +1>(x[0]);
    dftR<16, +1>(x[1]);
#pragma unroll
    for (int ka = 0; ka < 16; ka++)
    {
        const float2 z0 = cmul(x[0][ka], W[ka * 32 + bp]);
        const float2 z1 = cmul(x[1][ka], W[ka * 32 + 16 + bp]);
        uint32_t h0, l0, h1, l1;
        split_hi_lo<BF16>(z0, h0, l0);
        split_hi_lo<BF16>(z1, h1, l1);
        const uint32_t off = (uint32_t)(ka >> 3) * 16384u + (uint32_t)(ka & 7) * 2048u + row_off;
        *reinterpret_cast<uint2 *>(sA_hi + off) = make_uint2(h0, h1);
        *reinterpret_cast<uint2 *>(sA_lo + off) = make_uint2(l0, l1);
    }
}

// Thread 0: the 24 MMAs of one item (two A tiles x three products x four K-steps).
// Each tile's 12 MMAs end with a commit to that tile's mbarrier, so the warps that
// read tile 0's accumulator start while tile 1's MMAs still run.
__device__ __forceinline__ void tc_issue(uint32_t tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi, uint32_t b_lo,
                                         uint32_t idesc, uint64_t *mbar)
{
    umma::fence_after_sync();
#pragma unroll
    for (int t = 0; t < 2; t++)
    {
        const uint32_t d = tmem + 64u * t;
        const uint32_t ah = a_hi + 16384u * t, al = a_lo + 16384u * t;
#pragma unroll
        for (int ks = 0; ks < 4; ks++)
            umma::mma_f16(d, umma::desc_sw128(ah + 32u * ks), umma::desc_sw128(b_hi + 32u * ks), idesc, ks > 0);
#pragma unroll
        for (int ks = 0; ks < 4; ks++)
            umma::mma_f16(d, umma::desc_sw128(al + 32u * ks), umma::desc_sw128(b_hi + 32u * ks), idesc, 1u);
#pragma unroll
        for (int ks = 0; ks < 4; ks++)
            umma::mma_f16(d, umma::desc_sw128(ah + 32u * ks), umma::desc_sw128(b_lo + 32u * ks), idesc, 1u);
        umma::commit(mbar + t);
    }
}

template <int MODE, bool BF16>
__global__ void __launch_bounds__(P_THREADS, 2) inv_tc_kernel(PersistArgs a, TcArgs tc)
{
    constexpr int N1 = TC_N, N2 = TC_N, F = N1 * N2, M = F / 2;
    constexpr int n1t = N1 / TC_COLS, n2t = N2 / TC_COLS, per_block = n1t + n2t;
    constexpr bool FOLD = (MODE & OUT_FOLD) != 0;
    constexpr uint32_t IDESC_P1 = umma::idesc_f16(128, 64, BF16);
    constexpr uint32_t IDESC_P2 = umma::idesc_f16(128, 32, BF16);
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t mbar[2]; // MMAs of accumulator tile 0 / tile 1 done
    __shared__ uint32_t tmem_slot;
    __shared__ unsigned s_ticket[2];
    __shared__ int s_verdict[2];
    const uint32_t pad = (1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u;
    unsigned char *base = smem_raw + pad;
    unsigned char *sA_hi = base + TC_A_HI, *sA_lo = base + TC_A_LO;
    float2 *W1 = reinterpret_cast<float2 *>(base + TC_W1);
    float2 *W2 = reinterpret_cast<float2 *>(base + TC_W2);
    BinAcc *s_bins = reinterpret_cast<BinAcc *>(base + TC_BINS);
    float *s_p = reinterpret_cast<float *>(base + TC_A_HI); // fold staging, 16 KB
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // operand scales (powers of two): FP16 keeps every operand below 2^15
    float s1 = 1.0f, s2 = 1.0f;
    if constexpr (!BF16)
    {
        const float mx = __uint_as_float(__ldcg(tc.absmax)) * tc.hmax * 1.41421357f; // max |X*H|
        if (mx > 0.0f && mx < 1e30f)
        {
            // step-1 outputs are at most 16*mx (pass 1) and 16*512*mx (pass 2)
            s1 = ldexpf(1.0f, min(100, max(-100, 14 - ilogbf(16.0f * mx))));
            s2 = ldexpf(1.0f, min(100, max(-100, 14 - ilogbf(8192.0f * mx))));
        }
    }
    // the W_32 operand image (hi then lo, already in the swizzled layout)
    for (int i = tid; i < 1024; i += P_THREADS)
        reinterpret_cast<uint4 *>(base + TC_B_HI)[i] = __ldg(tc.bop + i);
    for (int e = tid; e < 512; e += P_THREADS)
    {
        const int ka = e >> 5, i = (e >> 4) & 1, bp = e & 15;
        const float2 w = __ldg(a.tw.twN1 + (2 * bp + i) * ka); // (2bp+i)*ka < 512
        W1[e] = make_float2(w.x * s1, w.y * s1);
        W2[e] = make_float2(w.x * s2, w.y * s2);
    }
    if constexpr (FOLD)
    {
        for (unsigned i = tid; i < a.fold.K; i += P_THREADS)
            s_bins[i] = BinAcc{0.0f, 0u};
    }
    if (warp == 0)
        umma::tmem_alloc(&tmem_slot, TC_TMEM_COLS);
    if (tid == 0)
    {
        umma::mbar_init(&mbar[0], 1);
        umma::mbar_init(&mbar[1], 1);
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t a_hi = umma::smem_addr(sA_hi), a_lo = umma::smem_addr(sA_lo);
    const uint32_t b_hi = umma::smem_addr(base + TC_B_HI), b_lo = umma::smem_addr(base + TC_B_LO);
    // this thread's accumulator row: tile t = warp/4, TMEM lanes of quarter warp%4
    const int acc_t = warp >> 2, acc_m = 32 * (warp & 3) + lane;
    const int acc_ka = 8 * acc_t + (acc_m >> 4), acc_v = acc_m & 15;
    const uint32_t acc_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 64u * acc_t;
    const float inv_s1 = 1.0f / s1;
    const float out_scale = 1.0f / (s2 * (float)F);
    const double flush_scale2 = (MODE == OUT_FOLD) ? 1.0 / ((double)F * F * (double)s2 * s2) : 1.0;
    int fold_d = -1;
    uint32_t phase = 0;
    bool mma_pending = false;

    const long long total = (a.G + a.lag) * (long long)per_block;
    const int B = a.B;
    unsigned held = 0;
    if (tid == 0)
        held = atomicAdd(a.ticket, 1u);
    for (unsigned it = 0;; it++)
    {
        const int par = it & 1;
        if (tid == 0)
        {
            unsigned t;
            s_verdict[par] = judge_ticket<n1t, n2t>(a, total, held, t, true);
            s_ticket[par] = t;
        }
        __syncthreads(); // also orders the previous item's shared-memory and TMEM use
        const int verdict = s_verdict[par];
        if (verdict < 0)
            break;
        if (verdict == 0)
            continue;
        const long long t = s_ticket[par];
        const long long q = t / per_block;
        const int w = (int)(t % per_block);
        const bool is_p1 = w < n1t;
        const long long f = is_p1 ? q : q - a.lag;
        const int slot = (int)((unsigned)f % (unsigned)a.S);
        float2 *Ts = a.T + (size_t)slot * F;
        const long long gi = a.g0 + f;
        int d, b;
        transform_dm_window((unsigned)gi, (unsigned)B, (unsigned)a.D, (unsigned)a.dm_group, d, b);
        float2 x[2][16];
        if (is_p1)
        {
            // columns n1 = c0 + v; lanes take consecutive columns (128-byte runs)
            const int c0 = w * TC_COLS;
            const int v = lane & 15, bp = 2 * warp + (lane >> 4);
            const int n0 = c0 + v + N1 * 2 * bp;
            const float2 *Hd = a.H + (size_t)d * F;
            const uint16_t *dl = a.delays + (size_t)d * F;
            const int rb = a.rbi + b;
            int sl[2][16];
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int k = 0; k < 16; k++)
                    sl[i][k] = ld_na(dl + n0 + N1 * (32 * k + i));
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int k = 0; k < 16; k++)
                {
                    const int n = n0 + N1 * (32 * k + i);
                    int s = rb - sl[i][k];
                    if (s < 0)
                        s += a.fbs;
                    // 32-bit element offset: fbs * F < 2^32 (host check)
                    x[i][k] = cmul(ld_na(a.ring + ((unsigned)s * (unsigned)F + (unsigned)n)), ld_na(Hd + n));
                }
            const uint32_t row_off = 128u * v + ((uint32_t)(((bp >> 1) ^ v) & 7) << 4) + 8u * (bp & 1);
            tc_step1<BF16>(x, W1, bp, row_off, sA_hi, sA_lo);
        }
        else
        {
            // rows k2 = r0 + v of the row-major slot; lanes take consecutive columns
            const int r0 = (w - n1t) * TC_COLS;
            const int bp = lane & 15, v = 2 * warp + (lane >> 4);
            if constexpr (FOLD)
            {
                if (d != fold_d)
                {
                    if (fold_d >= 0)
                        fold_flush(s_bins, a.fold, fold_d, flush_scale2);
                    fold_d = d;
                }
            }
            const float2 *row = Ts + (size_t)(r0 + v) * N1 + 2 * bp;
#pragma unroll
            for (int k = 0; k < 16; k++)
            {
                const float4 q4 = __ldcg(reinterpret_cast<const float4 *>(row + 32 * k));
                x[0][k] = make_float2(q4.x, q4.y);
                x[1][k] = make_float2(q4.z, q4.w);
            }
            const uint32_t row_off = 128u * v + ((uint32_t)(((bp >> 1) ^ v) & 7) << 4) + 8u * (bp & 1);
            tc_step1<BF16>(x, W2, bp, row_off, sA_hi, sA_lo);
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads(); // A tiles complete; pass 2: every thread holds its slot inputs
        if (tid == 0)
        {
            if (!is_p1) // release: every thread's reads of the slot precede the count
                asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.p2_done + slot) : "memory");
            tc_issue(tmem, a_hi, a_lo, b_hi + (is_p1 ? 0u : 4096u), b_lo + (is_p1 ? 0u : 4096u),
                     is_p1 ? IDESC_P1 : IDESC_P2, mbar);
        }
        // this warp's accumulator tile (and, for tile 1, every MMA of the item) is done
        if (!umma::mbar_wait(&mbar[acc_t], phase, a.timeout_ns))
        {
            atomicExch(a.err, 1); // the next ticket's verdict stops this CTA
            mma_pending = true;
        }
        phase ^= 1u;
        umma::fence_after_sync();
        if (is_p1)
        {
            // D row (ka, v): X1[n1 = c0 + v][k2 = ka + 16 kb], kb = 0..31, times
            // W_F^(n1*k2) (and 1/s1) into the row-major slot
            const int c0 = w * TC_COLS;
            const int n1 = c0 + acc_v;
            float c[2][32];
            umma::tmem_ld32(acc_addr, c[0]);
            umma::tmem_ld32(acc_addr + 32u, c[1]);
            float2 tw = twiddle_F(a.tw.lo, a.tw.hi, (unsigned)(n1 * acc_ka), N2 - 1, 9);
            tw = make_float2(tw.x * inv_s1, tw.y * inv_s1);
            const float2 step = twiddle_F(a.tw.lo, a.tw.hi, (unsigned)(16 * n1), N2 - 1, 9);
            float2 *dst = Ts + (size_t)acc_ka * N1 + n1;
#pragma unroll
            for (int kb = 0; kb < 32; kb++)
            {
                dst[(size_t)kb * 16 * N1] = cmul(make_float2(c[kb >> 4][(2 * kb) & 31], c[kb >> 4][(2 * kb + 1) & 31]), tw);
                tw = cmul(tw, step);
            }
            umma::fence_before_sync();
            __syncthreads();
            if (tid == 0)
                asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.p1_done + slot) : "memory");
        }
        else
        {
            // D row (ka, v): row k2 = r0 + v, outputs k1 = ka + 16 kb for kb = 16..31,
            // i.e. window samples k2 + N2 * (k1 - 256)
            const int r0 = (w - n1t) * TC_COLS;
            float c[32];
            umma::tmem_ld32(acc_addr, c);
            umma::fence_before_sync();
            const size_t rowbase = ((size_t)d * B + b) * M;
#pragma unroll
            for (int j = 0; j < 16; j++)
            {
                const int k1h = acc_ka + 16 * j;
                float2 xv = make_float2(c[2 * j], c[2 * j + 1]);
                if constexpr (MODE != OUT_FOLD)
                {
                    xv.x *= out_scale;
                    xv.y *= out_scale;
                }
                const size_t o = rowbase + r0 + acc_v + (size_t)N2 * k1h;
                if constexpr ((MODE & OUT_C64) != 0)
                    a.out_c64[o] = xv;
                if constexpr ((MODE & OUT_U16) != 0)
                    a.out_u16[o] = encode_u16(xv);
                if constexpr ((MODE & OUT_POW) != 0)
                    a.out_pow[o] = xv.x * xv.x + xv.y * xv.y;
                if constexpr ((MODE & OUT_PAIR) != 0)
                    s_p[k1h * TC_COLS + acc_v] = sqrtf(__ldcs(a.pair_pow + o) + (xv.x * xv.x + xv.y * xv.y));
                else if constexpr (FOLD)
                    s_p[k1h * TC_COLS + acc_v] = xv.x * xv.x + xv.y * xv.y;
            }
            if constexpr (FOLD)
            {
                __syncthreads();
                fold_tile<TC_COLS, N1 / 2>(s_p, s_bins,
                                          fold_phase0(a.fold) + (uint64_t)((uint64_t)b * (uint64_t)M) * a.fold.dphase,
                                          a.fold.dphase, a.fold.K, r0, N2);
            }
        }
    }
    if constexpr (FOLD)
    {
        if (fold_d >= 0)
            fold_flush(s_bins, a.fold, fold_d, flush_scale2);
    }
    // a timed-out item's MMAs may still be running: wait for them once more (bounded)
    // before the accumulator is released
    if (mma_pending && tid == 0)
        (void)umma::mbar_wait(&mbar[1], phase ^ 1u, a.timeout_ns);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0)
        umma::tmem_dealloc(tmem, TC_TMEM_COLS);
}

// This device's persisting-L2 set-aside for the slot ring of the launch at hand: set
// to `bytes` (capped at the device maximum) whenever a launch needs another size, so a
// large ring (e.g. a simulator's filter) does not keep L2 set aside for later work.  A
// failure only costs the hint.
size_t g_l2_set[kMaxDevices] = {};

void ensure_l2_persisting(size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices || g_l2_set[dev] == bytes)
        return;
    int maxp = 0;
    if (cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev) == cudaSuccess)
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::min((size_t)maxp, bytes));
    cudaGetLastError();
    g_l2_set[dev] = bytes;
}

// Launch (or, with `plan`, only size) a persistent transform kernel `k` taking
// (PersistArgs, EXTRA...): grid = resident CTAs per SM (at most max_per_sm) x SMs.
// carveout_blocks > 0: ask for a shared-memory carveout that holds that many CTAs
// (the occupancy query and the launch otherwise assume a smaller default split).
template <class KERNEL, class... EXTRA>
cudaError_t launch_persistent_kernel(KERNEL k, int threads, size_t smem, size_t (&granted)[kMaxDevices],
                                     int per_block, int max_per_sm, int carveout_blocks, int F, const PersistArgs &a,
                                     int sms, cudaStream_t st, PersistPlan *plan, EXTRA... extra)
{
    cudaError_t e = ensure_smem(k, smem, granted);
    if (e != cudaSuccess)
    {
        set_launch_failure_detail("persistent inverse transform", "shared-memory attribute", 0, 0, threads, smem);
        return e;
    }
    if (carveout_blocks > 0 && (e = prefer_carveout(k, smem, carveout_blocks)) != cudaSuccess)
    {
        (void)cudaGetLastError();
        set_launch_failure_detail("persistent inverse transform", "carveout attribute", 0, 0, threads, smem);
        return e;
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
    if (e != cudaSuccess)
        return e;
    const int occupancy = per_sm;
    // the occupancy query does not see the carveout preference: a kernel that asked
    // for room for carveout_blocks CTAs is launched with that many per SM (the
    // ticket order is deadlock-free whatever the residency)
    per_sm = std::min(std::max(per_sm, carveout_blocks), max_per_sm);
    if (a.max_ctas_per_sm > 0)
        per_sm = std::min(per_sm, a.max_ctas_per_sm);
    if (per_sm < 1)
        return cudaErrorInvalidConfiguration;
    const int grid = per_sm * sms;
    if (plan)
    {
        // Enough look-behind that items in flight rarely wait: every CTA holds its
        // current ticket and the next one, 2*grid items = 2*grid/per_block blocks in
        // flight.  P2(f) sits LAG blocks after P1(f); a slot is reused S blocks later,
        // so P1(f) waits on P2(f-S), S-LAG blocks back: S = 2*LAG keeps both distances
        // at LAG.  No more slack than that: at F = 2^20 a slot is 8 MB of L2.
        plan->lag = (2 * grid + per_block - 1) / per_block + 1;
        plan->slots = 2 * plan->lag;
        // A ring of such slots beyond 48 MB loses its lines from L2 before pass 2 reads
        // them; there, LAG sized to 1.5 x grid items is faster despite more waits
        // (F = 2^20: 6 slots of 8 MB, +4 % over 8; 4 or 5 slots are 13 % slower).
        if ((size_t)plan->slots * (size_t)F * sizeof(float2) > ((size_t)48 << 20))
        {
            plan->lag = (3 * grid + 2 * per_block - 1) / (2 * per_block) + 1;
            plan->slots = 2 * plan->lag;
        }
        plan->grid = grid;
        plan->occupancy = occupancy;
        return cudaSuccess;
    }
    // the kernel indexes transforms and tickets in 32 bits; its (d, b) map covers D * B
    if (a.dm_group < 1 || a.D < 1 || a.g0 + a.G > (long long)a.D * a.B)
        return cudaErrorInvalidValue;
    if (a.S <= a.lag || a.g0 < 0 || a.G < 0 || a.g0 + a.G + a.lag >= (1ll << 31) ||
        (a.G + a.lag) * (long long)per_block >= (1ll << 32))
        return cudaErrorInvalidValue;
    // the pass-1 -> pass-2 slots are re-read within a few items: ask L2 to keep them
    // (persisting window over the slot ring; the streamed spectra and responses miss it)
    const size_t slot_bytes = (size_t)a.S * (size_t)F * sizeof(float2);
    ensure_l2_persisting(slot_bytes);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    // the window cannot exceed the device's maximum access-policy window (the largest
    // transforms' slot rings do): it then covers the first part of the ring
    static int max_window[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        dev = 0;
    if (max_window[dev] == 0 &&
        cudaDeviceGetAttribute(&max_window[dev], cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess)
    {
        (void)cudaGetLastError();
        max_window[dev] = -1;
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = (void *)a.T;
    attr[0].val.accessPolicyWindow.num_bytes = std::min(slot_bytes, (size_t)std::max(max_window[dev], 0));
    attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cfg.attrs = attr;
    cfg.numAttrs = max_window[dev] > 0 ? 1 : 0;
    e = cudaLaunchKernelEx(&cfg, k, a, extra...);
    if (e == cudaSuccess)
        e = cudaGetLastError();
    if (e != cudaSuccess)
        set_launch_failure_detail("persistent inverse transform", "launch", grid, 1, threads, smem);
    return e;
}

// Register plan of the FP32 persistent transform for F = N1 x N2: 256 threads with
// radix-16/32 stages, or 512 threads with radix-8 stages.
template <int N1, int N2>
struct PersistPlanOf
{
    static constexpr int THREADS = P_THREADS;
    static constexpr bool BIG = true;
};

template <int N1, int N2, int MODE>
cudaError_t persist_launch(const PersistArgs &a, int sms, cudaStream_t st, PersistPlan *plan)
{
    using C1 = PCfg<N2>;
    using C2 = PCfg<N1>;
    constexpr int THREADS = PersistPlanOf<N1, N2>::THREADS;
    constexpr bool BIG = PersistPlanOf<N1, N2>::BIG;
    constexpr int DATA = (C1::SMEM_DATA > C2::SMEM_DATA) ? C1::SMEM_DATA : C2::SMEM_DATA;
    constexpr bool P1_TWO = LastNs<N2, 1, BIG>::value == StageRadix<N2, 1, BIG>::value;
    const size_t smem = (size_t)(DATA + N1 + (P1_TWO ? N2 : 2 * N2)) * sizeof(float2) +
                        (((MODE & OUT_FOLD) != 0) ? (size_t)a.fold.K * 8 : 0);
    static size_t granted[kMaxDevices] = {};
    constexpr int per_block = N1 / C1::COLS + N2 / C2::COLS;
    return launch_persistent_kernel(inv_persistent_kernel<N1, N2, MODE, THREADS, BIG>, THREADS, smem, granted,
                                    per_block, 1 << 20, 0, N1 * N2, a, sms, st, plan);
}

template <int MODE, bool BF16>
cudaError_t tc_launch(const PersistArgs &a, const TcArgs &tc, int sms, cudaStream_t st, PersistPlan *plan)
{
    const size_t smem = 1024 + TC_BINS + (((MODE & OUT_FOLD) != 0) ? (size_t)a.fold.K * 8 : 0);
    static size_t granted[kMaxDevices] = {};
    // at most 512 / 128 CTAs per SM can hold their tensor-memory columns at once
    return launch_persistent_kernel(inv_tc_kernel<MODE, BF16>, P_THREADS, smem, granted, 2 * (TC_N / TC_COLS),
                                    512 / (int)TC_TMEM_COLS, 2, TC_N * TC_N, a, sms, st, plan, tc);
}

template <bool BF16>
cudaError_t tc_mode(const PersistArgs &a, const TcArgs &tc, int sms, cudaStream_t st, PersistPlan *plan)
{
    switch (a.out_mode)
    {
    case OUT_C64: return tc_launch<OUT_C64, BF16>(a, tc, sms, st, plan);
    case OUT_U16: return tc_launch<OUT_U16, BF16>(a, tc, sms, st, plan);
    case OUT_FOLD: return tc_launch<OUT_FOLD, BF16>(a, tc, sms, st, plan);
    case OUT_C64 | OUT_FOLD: return tc_launch<OUT_C64 | OUT_FOLD, BF16>(a, tc, sms, st, plan);
    case OUT_U16 | OUT_FOLD: return tc_launch<OUT_U16 | OUT_FOLD, BF16>(a, tc, sms, st, plan);
    case OUT_C64 | OUT_U16: return tc_launch<OUT_C64 | OUT_U16, BF16>(a, tc, sms, st, plan);
    case OUT_POW: return tc_launch<OUT_POW, BF16>(a, tc, sms, st, plan);
    case OUT_FOLD | OUT_PAIR: return tc_launch<OUT_FOLD | OUT_PAIR, BF16>(a, tc, sms, st, plan);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t tc_dispatch(int L, int prec, const PersistArgs &a, const TcArgs &tc, int sms, cudaStream_t st,
                        PersistPlan *plan)
{
    // spectra-ring element offsets are 32-bit in the kernel
    if (L != 18 || (unsigned long long)a.fbs * (1ull << L) >= (1ull << 32))
        return cudaErrorInvalidValue;
    switch (prec)
    {
    case PREC_BF16X3: return tc_mode<true>(a, tc, sms, st, plan);
    case PREC_FP16X3: return tc_mode<false>(a, tc, sms, st, plan);
    default: return cudaErrorInvalidValue;
    }
}

template <int N1, int N2>
cudaError_t persist_mode(const PersistArgs &a, int sms, cudaStream_t st, PersistPlan *plan)
{
    switch (a.out_mode)
    {
    case OUT_C64: return persist_launch<N1, N2, OUT_C64>(a, sms, st, plan);
    case OUT_U16: return persist_launch<N1, N2, OUT_U16>(a, sms, st, plan);
    case OUT_FOLD: return persist_launch<N1, N2, OUT_FOLD>(a, sms, st, plan);
    case OUT_C64 | OUT_FOLD: return persist_launch<N1, N2, OUT_C64 | OUT_FOLD>(a, sms, st, plan);
    case OUT_U16 | OUT_FOLD: return persist_launch<N1, N2, OUT_U16 | OUT_FOLD>(a, sms, st, plan);
    case OUT_C64 | OUT_U16: return persist_launch<N1, N2, OUT_C64 | OUT_U16>(a, sms, st, plan);
    case OUT_POW: return persist_launch<N1, N2, OUT_POW>(a, sms, st, plan);
    case OUT_FOLD | OUT_PAIR: return persist_launch<N1, N2, OUT_FOLD | OUT_PAIR>(a, sms, st, plan);
    default: return cudaErrorInvalidValue;
    }
}

// The largest transforms (F = 2^23, 2^24: the plain overlap-save processor at long
// smears) only with the series / fold outputs a single-DM processor uses.
template <int N1, int N2>
cudaError_t persist_mode_large(const PersistArgs &a, int sms, cudaStream_t st, PersistPlan *plan)
{
    switch (a.out_mode)
    {
    case OUT_C64: return persist_launch<N1, N2, OUT_C64>(a, sms, st, plan);
    case OUT_U16: return persist_launch<N1, N2, OUT_U16>(a, sms, st, plan);
    case OUT_FOLD: return persist_launch<N1, N2, OUT_FOLD>(a, sms, st, plan);
    case OUT_C64 | OUT_FOLD: return persist_launch<N1, N2, OUT_C64 | OUT_FOLD>(a, sms, st, plan);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t persist_dispatch(int L, const PersistArgs &a, int sms, cudaStream_t st, PersistPlan *plan)
{
    switch (L)
    {
    case 23: return persist_mode_large<2048, 4096>(a, sms, st, plan);
    case 24: return persist_mode_large<4096, 4096>(a, sms, st, plan);
    case 16: return persist_mode<256, 256>(a, sms, st, plan);
    case 17: return persist_mode<256, 512>(a, sms, st, plan);
    case 18: return persist_mode<512, 512>(a, sms, st, plan);
    case 19: return persist_mode<512, 1024>(a, sms, st, plan);
    case 20: return persist_mode<1024, 1024>(a, sms, st, plan);
    case 21: return persist_mode<1024, 2048>(a, sms, st, plan);
    case 22: return persist_mode<2048, 2048>(a, sms, st, plan);
    default: return cudaErrorInvalidValue;
    }
}

// One thread runs wait_count() on a counter: `preset` is written first, the wait asks
// for `target`.  Nothing else writes the counter, so a preset below the target makes
// the wait run out; the flag and the elapsed %globaltimer time come back.
__global__ void selftest_wait_kernel(unsigned *cnt, unsigned preset, unsigned target, int *err,
                                     unsigned long long timeout_ns, unsigned long long *elapsed_ns)
{
    *cnt = preset;
    __threadfence();
    const uint64_t t0 = global_ns();
    (void)wait_count(cnt, target, err, timeout_ns); // a timeout sets *err
    *elapsed_ns = global_ns() - t0;
}

} // namespace

cudaError_t persist_selftest_wait(unsigned preset, unsigned target, unsigned long long timeout_ns, int *timed_out,
                                  unsigned long long *elapsed_ns)
{
    struct Buf
    {
        unsigned cnt;
        int err;
        unsigned long long elapsed;
    };
    Buf *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(Buf));
    if (e != cudaSuccess)
        return e;
    e = cudaMemset(d, 0, sizeof(Buf));
    if (e == cudaSuccess)
    {
        selftest_wait_kernel<<<1, 1>>>(&d->cnt, preset, target, &d->err, timeout_ns, &d->elapsed);
        e = cudaGetLastError();
    }
    Buf h{};
    if (e == cudaSuccess)
        e = cudaMemcpy(&h, d, sizeof(Buf), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e == cudaSuccess)
    {
        *timed_out = h.err;
        *elapsed_ns = h.elapsed;
    }
    return e;
}

bool persist_supported(int L) { return L >= 16 && L <= 24; }

cudaError_t persist_l2_reset()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaCtxResetPersistingL2Cache()) != cudaSuccess ||
        (e = cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0)) != cudaSuccess)
    {
        (void)cudaGetLastError();
        return e;
    }
    if (dev >= 0 && dev < kMaxDevices)
        g_l2_set[dev] = 0;
    return cudaSuccess;
}

cudaError_t persist_plan(int L, const PersistArgs &a, int sms, PersistPlan *plan)
{
    return persist_dispatch(L, a, sms, nullptr, plan);
}

cudaError_t launch_inverse_persistent(int L, const PersistArgs &a, int sms, cudaStream_t st)
{
    return persist_dispatch(L, a, sms, st, nullptr);
}

bool tc_supported(int L) { return L == 18; }

cudaError_t tc_plan(int L, int prec, const PersistArgs &a, const TcArgs &tc, int sms, PersistPlan *plan)
{
    return tc_dispatch(L, prec, a, tc, sms, nullptr, plan);
}

cudaError_t launch_inverse_tc(int L, int prec, const PersistArgs &a, const TcArgs &tc, int sms, cudaStream_t st)
{
    return tc_dispatch(L, prec, a, tc, sms, st, nullptr);
}

} // namespace msosm
