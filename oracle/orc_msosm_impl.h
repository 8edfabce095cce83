/*
 * ORACLE (test infrastructure only) -- streaming MS-OSM restated on the CPU.
 *
 * Included twice by msosm_oracle.c (ORC_REAL=double -> orc64_*, ORC_REAL=float
 * -> orc32_*).  The FP64 instance is the parity oracle; the FP32 instance is the
 * "port" timed as the CPU baseline.  Nothing in the product links this file.
 *
 * Semantics restated from the reference's GPU processor:
 *   ring / overlap bookkeeping  dedispersion/msosm/msosm_gpu_batch.cpp:153-176
 *     - complex input buffer of (B+1)*M samples, first M = previous call's tail,
 *       zero before the first call (msosm_gpu_batch.cpp:50-52, 153-165)
 *     - forward spectra ring of fbs slots; call s writes slots
 *       rbi..rbi+B-1 with rbi = (s*B) mod fbs (msosm_gpu_batch.cpp:167-176)
 *   forward FFT: B windows of F=2M samples, hop M (msosm_gpu_batch.cpp:100-107, 189-191)
 *   gather x multiply: gpu/gpu_kernel.cu:106-192
 *       x[n] = ring[((rbi + b - delay[n]) mod fbs)][n] * H[n]   (no 1/F here)
 *   inverse FFT (unnormalised): msosm_gpu_batch.cpp:135,196-199
 *   discard: gpu/gpu_kernel.cu:346-368  out[(d*B+b)*M+o] = y[M+o] * (1/(2M))
 *   fold: gpu/gpu_kernel.cu:430-496 and folding/fold_gpu.cpp:48-54
 * The ring is zeroed here (the reference leaves it uninitialised,
 * msosm_gpu_batch.cpp:122), so warm-up outputs are deterministic.
 */
#ifndef ORC_REAL
#error "define ORC_REAL before including orc_msosm_impl.h"
#endif

#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC_FN(name) ORC_CAT(name, ORC_SUFFIX)
#define ORC_API(name) ORC_CAT(ORC_PREFIX, name)

typedef struct
{
    int M, F, B, D, fbs;
    long step;
    int nthreads;
    int *delays;     /* D*F */
    ORC_REAL *H;     /* D*F complex */
    ORC_REAL *ring;  /* fbs*F complex */
    ORC_REAL *buf;   /* (B+1)*M complex : [tail | new] */
    ORC_FN(orc_plan) * pf;
    ORC_FN(orc_plan) * pb;
    ORC_REAL *scratch; /* nthreads * 2F complex */
    /* fold */
    unsigned long K;
    double period, dt, t_start;
    double *fsum;              /* nthreads * D*K */
    unsigned long long *fcnt;  /* nthreads * D*K */
    /* per-call job context */
    ORC_REAL *out;
    int rbi;
} ORC_FN(orc_msosm);

ORC_FN(orc_msosm) * ORC_API(msosm_create)(int M, int B, int D, const int *delays, const ORC_REAL *H, int fbs, int nthreads)
{
    ORC_FN(orc_msosm) *h = (ORC_FN(orc_msosm) *)calloc(1, sizeof(*h));
    const int F = 2 * M;
    h->M = M;
    h->F = F;
    h->B = B;
    h->D = D;
    h->fbs = fbs;
    h->nthreads = nthreads > 0 ? nthreads : 1;
    h->delays = (int *)malloc(sizeof(int) * (size_t)D * F);
    memcpy(h->delays, delays, sizeof(int) * (size_t)D * F);
    h->H = (ORC_REAL *)malloc(sizeof(ORC_REAL) * 2 * (size_t)D * F);
    memcpy(h->H, H, sizeof(ORC_REAL) * 2 * (size_t)D * F);
    h->ring = (ORC_REAL *)calloc((size_t)fbs * F * 2, sizeof(ORC_REAL));
    h->buf = (ORC_REAL *)calloc((size_t)(B + 1) * M * 2, sizeof(ORC_REAL));
    h->pf = ORC_FN(orc_plan_create)(F, -1);
    h->pb = ORC_FN(orc_plan_create)(F, +1);
    h->scratch = (ORC_REAL *)malloc(sizeof(ORC_REAL) * 2 * 2 * (size_t)F * h->nthreads);
    return h;
}

void ORC_API(msosm_destroy)(ORC_FN(orc_msosm) * h)
{
    if (!h)
        return;
    free(h->delays);
    free(h->H);
    free(h->ring);
    free(h->buf);
    ORC_FN(orc_plan_destroy)(h->pf);
    ORC_FN(orc_plan_destroy)(h->pb);
    free(h->scratch);
    free(h->fsum);
    free(h->fcnt);
    free(h);
}

/* Enable folding of the 1-pol intensity |x|^2 of every DM's output into K
 * phase bins.  Mirrors Fold_GPU(period, fs, size, .., time_bin)
 * (folding/fold_gpu.cpp:4-25): period and fs arrive as float, dt = 1/fs in double. */
void ORC_API(msosm_set_fold)(ORC_FN(orc_msosm) * h, unsigned long K, float period, float fs)
{
    h->K = K;
    h->period = (double)period;
    h->dt = 1.0 / (double)fs;
    h->t_start = 0.0;
    free(h->fsum);
    free(h->fcnt);
    h->fsum = (double *)calloc((size_t)h->nthreads * h->D * K, sizeof(double));
    h->fcnt = (unsigned long long *)calloc((size_t)h->nthreads * h->D * K, sizeof(unsigned long long));
}

static void ORC_FN(fwd_task)(void *ctx, long b, int tid)
{
    ORC_FN(orc_msosm) *h = (ORC_FN(orc_msosm) *)ctx;
    const int F = h->F, M = h->M;
    ORC_REAL *slot = h->ring + 2 * (size_t)(h->rbi + b) * F;
    memcpy(slot, h->buf + 2 * (size_t)b * M, sizeof(ORC_REAL) * 2 * F);
    ORC_FN(orc_fft_exec)(h->pf, slot, h->scratch + 2 * (size_t)tid * 2 * F);
}

static void ORC_FN(inv_task)(void *ctx, long job, int tid)
{
    ORC_FN(orc_msosm) *h = (ORC_FN(orc_msosm) *)ctx;
    const int F = h->F, M = h->M, B = h->B, fbs = h->fbs;
    const int d = (int)(job / B), b = (int)(job % B);
    ORC_REAL *x = h->scratch + 2 * (size_t)tid * 2 * F;
    ORC_REAL *sc = x + 2 * (size_t)F;
    const int *dl = h->delays + (size_t)d * F;
    const ORC_REAL *Hd = h->H + 2 * (size_t)d * F;
    for (int n = 0; n < F; n++)
    {
        int slot = h->rbi + b - dl[n];
        slot = ((slot % fbs) + fbs) % fbs; /* gpu_kernel.cu:141-142 */
        const ORC_REAL *sp = h->ring + 2 * ((size_t)slot * F + n);
        ORC_REAL vr = sp[0], vi = sp[1];
        ORC_REAL pr = Hd[2 * n], pi_ = Hd[2 * n + 1];
        x[2 * n] = vr * pr - vi * pi_; /* gpu_kernel.cu:183-184 */
        x[2 * n + 1] = vr * pi_ + vi * pr;
    }
    ORC_FN(orc_fft_exec)(h->pb, x, sc);
    const ORC_REAL scale = (ORC_REAL)1 / (ORC_REAL)(2 * M); /* gpu_kernel.cu:358 */
    ORC_REAL *o = h->out ? h->out + 2 * ((size_t)(d * B + b) * M) : NULL;
    double *fs = h->fsum ? h->fsum + ((size_t)tid * h->D + d) * h->K : NULL;
    unsigned long long *fc = h->fcnt ? h->fcnt + ((size_t)tid * h->D + d) * h->K : NULL;
    for (int i = 0; i < M; i++)
    {
        ORC_REAL yr = x[2 * (M + i)] * scale, yi = x[2 * (M + i) + 1] * scale;
        if (o)
        {
            o[2 * i] = yr;
            o[2 * i + 1] = yi;
        }
        if (fs)
        {
            /* calculateIntensity_single_kernel: |a|^2 in float (gpu_kernel.cu:438-444) */
            float fx = (float)yr, fy = (float)yi;
            float val = fx * fx + fy * fy;
            if (val == 0.0f) /* gpu_kernel.cu:474-476 */
                continue;
            double t = h->t_start + (double)((size_t)b * M + i) * h->dt;
            double phase = fmod(t / h->period, 1.0);
            unsigned long bin = (unsigned long)floor(phase * (double)h->K);
            if (bin >= h->K)
                bin = h->K - 1;
            fs[bin] += (double)val;
            fc[bin] += 1ULL;
        }
    }
}

/* One filter_block call: B*M new complex samples in, D*B*M complex samples out
 * (out may be NULL when only folding). */
void ORC_API(msosm_process)(ORC_FN(orc_msosm) * h, const ORC_REAL *in, ORC_REAL *out)
{
    const int M = h->M, B = h->B;
    /* overlap: previous tail is buf[B*M..(B+1)*M) -> buf[0..M) (msosm_gpu_batch.cpp:155-162) */
    if (h->step > 0)
        memmove(h->buf, h->buf + 2 * (size_t)B * M, sizeof(ORC_REAL) * 2 * M);
    memcpy(h->buf + 2 * (size_t)M, in, sizeof(ORC_REAL) * 2 * (size_t)B * M);
    h->rbi = (int)((h->step * B) % h->fbs);
    orc_parallel_for(B, h->nthreads, ORC_FN(fwd_task), h);
    h->out = out;
    orc_parallel_for((long)h->D * B, h->nthreads, ORC_FN(inv_task), h);
    h->out = NULL;
    if (h->fsum)
        h->t_start += (double)((size_t)B * M) * h->dt; /* fold_gpu.cpp:53 */
    h->step++;
}

/* Sum the per-thread fold partials into sum[D*K], cnt[D*K]. */
void ORC_API(msosm_fold_read)(ORC_FN(orc_msosm) * h, double *sum, unsigned long long *cnt)
{
    const size_t DK = (size_t)h->D * h->K;
    for (size_t i = 0; i < DK; i++)
    {
        double s = 0;
        unsigned long long c = 0;
        for (int t = 0; t < h->nthreads; t++)
        {
            s += h->fsum[t * DK + i];
            c += h->fcnt[t * DK + i];
        }
        sum[i] = s;
        cnt[i] = c;
    }
}

long ORC_API(msosm_step)(ORC_FN(orc_msosm) * h) { return h->step; }

/* Plain batched FFT through the same engine (used to cross-check against numpy). */
void ORC_API(fft)(ORC_REAL *x, int n, int sign, int count)
{
    ORC_FN(orc_plan) *p = ORC_FN(orc_plan_create)(n, sign);
    ORC_REAL *sc = (ORC_REAL *)malloc(sizeof(ORC_REAL) * 2 * (size_t)n);
    for (int c = 0; c < count; c++)
        ORC_FN(orc_fft_exec)(p, x + 2 * (size_t)c * n, sc);
    free(sc);
    ORC_FN(orc_plan_destroy)(p);
}

#undef ORC_FN
#undef ORC_API
#undef ORC_CAT
#undef ORC_CAT2
