/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A CPU restatement of the reference's MS-OSM coherent-dedispersion hot path
 * (joezhouchenye/AcceleratedMS-OSM).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm may load it, and only as the checker
 * or the timed CPU baseline.  The product library never links or calls it.
 *
 * Contents (each function cites the reference lines it restates):
 *   planning   : Nd, filter order M, delaycount, per-bin delay map, segments,
 *                dedispersion response H (FP64 throughout)
 *   streaming  : orc64_* (FP64 oracle) and orc32_* (FP32 port), see
 *                orc_msosm_impl.h
 *   codecs     : uint16 offset-binary decode/encode, int8 decode
 *   folding    : intensity + FP64 phase fold exactly as the reference computes it
 *
 * Float/double expression types in the planning code follow the reference
 * operand by operand, because they decide bin boundaries.  Build with
 * -ffp-contract=off (no FMA contraction) so float products round as on x86.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846 /* utils/include/globals.h:30 uses M_PI */

/* ------------------------------------------------------------------------ */
/* tiny thread pool                                                          */
/* ------------------------------------------------------------------------ */
typedef void (*orc_task_fn)(void *ctx, long i, int tid);
typedef struct
{
    long n;
    long next;
    orc_task_fn fn;
    void *ctx;
    int tid;
} orc_pf_arg;

typedef struct
{
    orc_pf_arg *shared;
    int tid;
} orc_pf_thread;

static void *orc_pf_worker(void *p)
{
    orc_pf_thread *t = (orc_pf_thread *)p;
    orc_pf_arg *a = t->shared;
    for (;;)
    {
        long i = __atomic_fetch_add(&a->next, 1, __ATOMIC_RELAXED);
        if (i >= a->n)
            break;
        a->fn(a->ctx, i, t->tid);
    }
    return NULL;
}

static void orc_parallel_for(long n, int nthreads, orc_task_fn fn, void *ctx)
{
    if (nthreads <= 1 || n <= 1)
    {
        for (long i = 0; i < n; i++)
            fn(ctx, i, 0);
        return;
    }
    if (nthreads > n)
        nthreads = (int)n;
    orc_pf_arg a = {n, 0, fn, ctx, 0};
    pthread_t th[256];
    orc_pf_thread targ[256];
    if (nthreads > 256)
        nthreads = 256;
    for (int t = 1; t < nthreads; t++)
    {
        targ[t].shared = &a;
        targ[t].tid = t;
        pthread_create(&th[t], NULL, orc_pf_worker, &targ[t]);
    }
    targ[0].shared = &a;
    targ[0].tid = 0;
    orc_pf_worker(&targ[0]);
    for (int t = 1; t < nthreads; t++)
        pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* FFT + streaming engine, instantiated for double and float                 */
/* ------------------------------------------------------------------------ */
#define ORC_REAL double
#define ORC_SUFFIX _d
#define ORC_PREFIX orc64_
#include "orc_fft_impl.h"
#include "orc_msosm_impl.h"
#undef ORC_REAL
#undef ORC_SUFFIX
#undef ORC_PREFIX

#define ORC_REAL float
#define ORC_SUFFIX _f
#define ORC_PREFIX orc32_
#include "orc_fft_impl.h"
#include "orc_msosm_impl.h"
#undef ORC_REAL
#undef ORC_SUFFIX
#undef ORC_PREFIX

/* ------------------------------------------------------------------------ */
/* planning                                                                  */
/* ------------------------------------------------------------------------ */

/* kdm = 4.15 * 1e15 stored as float (msosm_prepare.cpp:6, msosm_prepare.h:54) */
static float orc_kdm_f(void) { return (float)(4.15 * 1e15); }

/* Dispersion smear in samples, msosm_prepare.cpp:33 / :12:
 *   floor(kdm*dm * (1/pow(f0,2) - 1/pow(f0+bw,2)) / (1/fs)), fs = bw.
 * kdm*dm is a float product; f0+bw a float sum; 1/fs a float quotient. */
static double orc_nd_value(float bw, float dm, float f0)
{
    const float fs = bw;
    const float kd = orc_kdm_f() * dm;
    const float f1 = f0 + bw;
    const double a = 1.0 / ((double)f0 * (double)f0);
    const double b = 1.0 / ((double)f1 * (double)f1);
    const float inv_fs = 1.0f / fs;
    return floor((double)kd * (a - b) / (double)inv_fs);
}

int orc_nd(float bw, float dm, float f0) { return (int)orc_nd_value(bw, dm, f0); }

/* Prepare_OSM keeps Nd as unsigned long (dedispersion/overlap_save/osm_prepare.cpp:8) */
unsigned long orc_osm_nd(float bw, float dm, float f0) { return (unsigned long)orc_nd_value(bw, dm, f0); }

/* calculate_min_order, msosm_prepare.cpp:48-69: per DM 2^ceil(log2(sqrt(512)*sqrt(Nd))),
 * the filter order is the maximum over DMs. */
int orc_min_order_one(int nd)
{
    double order = sqrt(1024 / 2.0) * sqrt((double)nd);
    return (int)pow(2.0, ceil(log2(order)));
}

int orc_min_order(const int *nd, int n)
{
    int m = orc_min_order_one(nd[0]);
    for (int i = 1; i < n; i++)
    {
        int v = orc_min_order_one(nd[i]);
        if (v > m)
            m = v;
    }
    return m;
}

/* initialize_uint16's choice of M, msosm_gpu_batch.cpp:32-41 */
int orc_choose_M(int M_min, int fftpoint)
{
    int M = M_min;
    if (fftpoint != 0)
    {
        M = fftpoint / 2;
        if (M < M_min)
            M = M_min;
    }
    return M;
}

/* msosm_prepare.cpp:217: ceil(Nd / (float)M) -- Nd converts to float first */
int orc_delaycount(int nd, int M) { return (int)ceilf((float)nd / (float)M); }

/* segmentation(i), msosm_prepare.cpp:215-284.
 * The reference computes poscount from the processor-wide running maximum of
 * delaycount (msosm_prepare.cpp:239).  Nd, and so delaycount, is monotone in DM,
 * so for the ascending DM lists the reference requires the running maximum is
 * this DM's own delaycount, which is what is used here.
 * Writes delay[0..2M).  Returns this DM's delaycount.
 * DM lists where dc==0 (DM 0) leave the reference's map uninitialised; the
 * oracle defines delay 0 for every bin there (identity gather). */
int orc_segmentation(float bw, float f0, float dm, int nd, int M, int *delay)
{
    const int F = 2 * M;
    const float fs = bw;
    const float kdm = orc_kdm_f();
    const float w0 = (float)(2 * ORC_PI * (double)f0); /* msosm_prepare.cpp:7 */
    const int dc = orc_delaycount(nd, M);
    for (int k = 0; k < F; k++)
        delay[k] = 0;
    if (dc <= 0)
        return dc;
    float *w = (float *)malloc(sizeof(float) * (size_t)(dc + 1));
    w[0] = -1;
    w[dc] = 1;
    int pos_index = 1;
    const double w0sq_inv = 1.0 / ((double)w0 * (double)w0);
    const double den = 4 * ORC_PI * ORC_PI * (double)kdm * (double)dm;
    for (int j = 1; j < dc; j++)
    {
        /* w[j] = (sqrt(1/(1/w0^2 - j*M/fs/(4 pi^2 kdm dm))) - w0 - pi*fs)/pi/fs */
        const float jm_fs = (float)(j * M) / fs;
        const double inner = w0sq_inv - (double)jm_fs / den;
        const double v = ((sqrt(1.0 / inner) - (double)w0) - ORC_PI * (double)fs) / ORC_PI / (double)fs;
        w[j] = (float)v;
        if (w[j] < 0)
            pos_index = j + 1;
    }
    const int negcount = pos_index;
    const int poscount = dc - pos_index + 1;
    int *segneg = (int *)malloc(sizeof(int) * (size_t)(negcount + 1));
    int *segpos = (int *)malloc(sizeof(int) * (size_t)(poscount + 1));
    for (int j = 0; j < negcount; j++)
        segneg[j] = (int)floorf((w[j] + 2.0f) * (float)M);
    segneg[negcount] = 2 * M;
    segpos[0] = 0;
    for (int j = 0; j < poscount; j++)
        segpos[j + 1] = (int)floorf(w[j + negcount] * (float)M);
    for (int j = 0; j < negcount; j++)
        for (int k = segneg[j]; k < segneg[j + 1]; k++)
            delay[k] = j;
    for (int j = 0; j < poscount; j++)
        for (int k = segpos[j]; k < segpos[j + 1]; k++)
            delay[k] = negcount - 1 + j;
    free(segneg);
    free(segpos);
    free(w);
    return dc;
}

/* build_segments, msosm_gpu_batch.cpp:262-295: runs of equal delay, each at
 * most maxlen (BLOCK_SIZE = 256, gpu/include/gpu_kernel.cuh:6) bins long. */
int orc_build_segments(const int *delay, int F, int maxlen, int *start, int *len, int *group)
{
    if (F <= 0)
        return 0;
    int count = 0;
    int cur_group = delay[0], cur_start = 0;
    for (int k = 1; k < F; k++)
    {
        if (delay[k] != cur_group || k - cur_start == maxlen)
        {
            start[count] = cur_start;
            len[count] = k - cur_start;
            group[count] = cur_group;
            count++;
            cur_start = k;
            cur_group = delay[k];
        }
    }
    start[count] = cur_start;
    len[count] = F - cur_start;
    group[count] = cur_group;
    return count + 1;
}

/* Dedispersion response, generate_dedisp_params, msosm_prepare.cpp:107-164
 * (and osm_prepare.cpp:68-125, identical): FFT-order-shifted chirp
 *   h[M/2+j] = exp(-i phi_j) (j<M/2), h[j-M/2] = exp(-i phi_j) (j>=M/2),
 *   phi_j = 4 pi^2 kdm DM w^2 / ((w+w0) w0^2), w = 2 pi fs j / M   (FP64, kdm=4.15e15)
 * then h = IFFT_M(h)/M, zero-padded to 2M, H = FFT_2M(h).  FP64 throughout
 * here; H is written as 2*F doubles (re, im). */
void orc_response(float bw, float f0, float dm, int M, double *H)
{
    const double pi_d = ORC_PI;
    const double kdm_d = 4.15e15;
    const double fs_d = (double)bw;
    const double dm_d = (double)dm;
    const double f0_d = (double)f0;
    const double w0_d = 2.0 * pi_d * f0_d;
    const double step = 2.0 * pi_d * fs_d / (double)M;
    const int F = 2 * M;
    double *h = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    for (int j = 0; j < M; j++)
    {
        double w = step * (double)j;
        double phase = 4.0 * pi_d * pi_d * kdm_d * dm_d * w * w / ((w + w0_d) * w0_d * w0_d);
        int dst = (j < M / 2) ? (M / 2 + j) : (j - M / 2);
        h[2 * dst] = cos(phase);
        h[2 * dst + 1] = -sin(phase);
    }
    orc64_fft(h, M, +1, 1);
    memset(H, 0, sizeof(double) * 2 * (size_t)F);
    for (int j = 0; j < M; j++)
    {
        H[2 * j] = h[2 * j] / (double)M;
        H[2 * j + 1] = h[2 * j + 1] / (double)M;
    }
    free(h);
    orc64_fft(H, F, -1, 1);
}

/* dH/dDM of the response above (no counterpart in the reference): the chirp
 * phase is linear in DM, so d/dDM exp(-i phi) = -i (phi/DM) exp(-i phi); the
 * IFFT_M / zero-pad / FFT_2M construction is linear and is applied unchanged. */
void orc_response_derivative(float bw, float f0, float dm, int M, double *H)
{
    const double pi_d = ORC_PI;
    const double kdm_d = 4.15e15;
    const double fs_d = (double)bw;
    const double dm_d = (double)dm;
    const double w0_d = 2.0 * pi_d * (double)f0;
    const double step = 2.0 * pi_d * fs_d / (double)M;
    const int F = 2 * M;
    double *h = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    for (int j = 0; j < M; j++)
    {
        double w = step * (double)j;
        double per_dm = 4.0 * pi_d * pi_d * kdm_d * w * w / ((w + w0_d) * w0_d * w0_d);
        double phase = per_dm * dm_d;
        int dst = (j < M / 2) ? (M / 2 + j) : (j - M / 2);
        /* -i * per_dm * (cos - i sin) = -per_dm * sin - i per_dm * cos */
        h[2 * dst] = -per_dm * sin(phase);
        h[2 * dst + 1] = -per_dm * cos(phase);
    }
    orc64_fft(h, M, +1, 1);
    memset(H, 0, sizeof(double) * 2 * (size_t)F);
    for (int j = 0; j < M; j++)
    {
        H[2 * j] = h[2 * j] / (double)M;
        H[2 * j + 1] = h[2 * j + 1] / (double)M;
    }
    free(h);
    orc64_fft(H, F, -1, 1);
}

/* Prepare_OSM::calculate_min_order, osm_prepare.cpp:15-28: M = 2*next_pow2((int)Nd) */
unsigned long orc_osm_min_order(unsigned long nd)
{
    int n = (int)nd;
    int p;
    if (n <= 0)
        p = 1;
    else
    {
        --n;
        n |= n >> 1;
        n |= n >> 2;
        n |= n >> 4;
        n |= n >> 8;
        n |= n >> 16;
        p = n + 1;
    }
    return 2UL * (unsigned long)p;
}

/* ------------------------------------------------------------------------ */
/* codecs                                                                    */
/* ------------------------------------------------------------------------ */

/* uint16ToComplex_kernel, gpu/gpu_kernel.cu:16-30: value = x - 32768*(x!=0), in float.
 * in: n packed uint32 (low 16 bits = real, high 16 = imag); out: n complex (float). */
void orc_decode_u16(const uint32_t *in, size_t n, float *out)
{
    for (size_t i = 0; i < n; i++)
    {
        uint32_t v = in[i];
        uint16_t x = (uint16_t)(v & 0xFFFFu), y = (uint16_t)(v >> 16);
        out[2 * i] = (float)x - 32768.0f * (float)(x != 0);
        out[2 * i + 1] = (float)y - 32768.0f * (float)(y != 0);
    }
}

/* int8 interleaved I/Q (new input type; exact in float). */
void orc_decode_i8(const int8_t *in, size_t n, float *out)
{
    for (size_t i = 0; i < n; i++)
    {
        out[2 * i] = (float)in[2 * i];
        out[2 * i + 1] = (float)in[2 * i + 1];
    }
}

/* __float2uint_rn: round half to even, saturate to [0, 2^32-1], NaN -> 0 */
static uint32_t orc_f2u_rn(float s)
{
    if (!(s > 0.0f))
        return 0u;
    if (s >= 4294967296.0f)
        return 0xFFFFFFFFu;
    return (uint32_t)rintf(s);
}

/* discardSamplesToUint16_kernel epilogue, gpu/gpu_kernel.cu:398-413, applied to
 * already-scaled float values: u = rn(v + 32768*(v!=0)), packed (y<<16)|x. */
void orc_encode_u16(const float *in, size_t n, uint32_t *out)
{
    for (size_t i = 0; i < n; i++)
    {
        float xf = in[2 * i], yf = in[2 * i + 1];
        uint32_t x = orc_f2u_rn(xf + (xf != 0 ? 32768.0f : 0.0f));
        uint32_t y = orc_f2u_rn(yf + (yf != 0 ? 32768.0f : 0.0f));
        out[i] = (y << 16) | x;
    }
}

/* ------------------------------------------------------------------------ */
/* folding                                                                   */
/* ------------------------------------------------------------------------ */

/* calculateIntensity_single_kernel (gpu_kernel.cu:438-444): |a|^2, no sqrt */
void orc_intensity1(const float *a, size_t n, float *out)
{
    for (size_t i = 0; i < n; i++)
        out[i] = a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1];
}

/* calculateIntensity_kernel (gpu_kernel.cu:430-436): sqrt(|a|^2+|b|^2) */
void orc_intensity2(const float *a, const float *b, size_t n, float *out)
{
    for (size_t i = 0; i < n; i++)
        out[i] = sqrtf(a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1] + b[2 * i] * b[2 * i] +
                       b[2 * i + 1] * b[2 * i + 1]);
}

/* foldDataPhase_kernel (gpu_kernel.cu:462-485) on the host. */
void orc_fold(const float *inten, size_t n, unsigned long K, double t_start, double dt, double period,
              double *sum, unsigned long long *cnt)
{
    for (size_t i = 0; i < n; i++)
    {
        float val = inten[i];
        if (val == 0.0f)
            continue;
        double t = t_start + (double)i * dt;
        double phase = fmod(t / period, 1.0);
        unsigned long bin = (unsigned long)floor(phase * (double)K);
        if (bin >= K)
            bin = K - 1;
        sum[bin] += (double)val;
        cnt[bin] += 1ULL;
    }
}

/* The phase bin alone, for index-level checks. */
unsigned long orc_fold_bin(double t_start, double dt, double period, unsigned long K, size_t i)
{
    double t = t_start + (double)i * dt;
    double phase = fmod(t / period, 1.0);
    unsigned long bin = (unsigned long)floor(phase * (double)K);
    return bin >= K ? K - 1 : bin;
}

/* computeFoldedData_kernel (gpu_kernel.cu:498-508) */
void orc_fold_finalize(const double *sum, const unsigned long long *cnt, unsigned long K, float *out)
{
    for (unsigned long b = 0; b < K; b++)
        out[b] = cnt[b] > 0 ? (float)(sum[b] / (double)cnt[b]) : 0.0f;
}
