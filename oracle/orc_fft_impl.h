/*
 * ORACLE (test infrastructure only) -- radix-4/radix-2 Stockham FFT on the CPU.
 *
 * Included twice by msosm_oracle.c, once with ORC_REAL=double (the FP64 oracle)
 * and once with ORC_REAL=float (the FP32 CPU port used as the timed CPU baseline).
 * It stands in for the FFTW / cuFFT transforms the reference calls:
 *   - FFTW_BACKWARD/FFTW_FORWARD in dedispersion/msosm/msosm_prepare.cpp:200-221
 *   - cufftExecC2C forward/inverse in dedispersion/msosm/msosm_gpu_batch.cpp:191,196-199
 * Sign convention follows FFTW/cuFFT: sign=-1 forward, sign=+1 inverse,
 * both unnormalised.  Twiddles are always computed in double and rounded.
 */
#ifndef ORC_REAL
#error "define ORC_REAL before including orc_fft_impl.h"
#endif

#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC_FN(name) ORC_CAT(name, ORC_SUFFIX)

typedef struct
{
    int n;
    int sign;
    ORC_REAL *tw;  /* n complex entries: exp(sign*2*pi*i*k/n) */
    ORC_REAL *buf; /* scratch, n complex */
} ORC_FN(orc_plan);

static ORC_FN(orc_plan) * ORC_FN(orc_plan_create)(int n, int sign)
{
    ORC_FN(orc_plan) *p = (ORC_FN(orc_plan) *)calloc(1, sizeof(*p));
    p->n = n;
    p->sign = sign;
    p->tw = (ORC_REAL *)malloc(sizeof(ORC_REAL) * 2 * (size_t)n);
    p->buf = (ORC_REAL *)malloc(sizeof(ORC_REAL) * 2 * (size_t)n);
    for (int k = 0; k < n; k++)
    {
        /* exact angle reduction: k/n is a dyadic rational */
        double a = 2.0 * ORC_PI * (double)k / (double)n;
        p->tw[2 * k] = (ORC_REAL)cos(a);
        p->tw[2 * k + 1] = (ORC_REAL)(sign * sin(a));
    }
    return p;
}

static void ORC_FN(orc_plan_destroy)(ORC_FN(orc_plan) * p)
{
    if (!p)
        return;
    free(p->tw);
    free(p->buf);
    free(p);
}

/* In-place transform of x (n interleaved complex values). scratch: n complex. */
static void ORC_FN(orc_fft_exec)(const ORC_FN(orc_plan) * p, ORC_REAL *x, ORC_REAL *scratch)
{
    const int n = p->n;
    const ORC_REAL s = (ORC_REAL)p->sign;
    const ORC_REAL *tw = p->tw;
    ORC_REAL *src = x, *dst = scratch;
    if (n <= 1)
        return;
    int Ns = 1;
    while (Ns < n)
    {
        int R = (n / Ns >= 4) ? 4 : 2;
        int q = n / R; /* stride between butterfly inputs */
        int step = n / (Ns * R);
        for (int j = 0; j < q; j++)
        {
            int k = j & (Ns - 1);
            int base = (j / Ns) * Ns * R + k;
            if (R == 4)
            {
                ORC_REAL v0r = src[2 * j], v0i = src[2 * j + 1];
                ORC_REAL v1r = src[2 * (j + q)], v1i = src[2 * (j + q) + 1];
                ORC_REAL v2r = src[2 * (j + 2 * q)], v2i = src[2 * (j + 2 * q) + 1];
                ORC_REAL v3r = src[2 * (j + 3 * q)], v3i = src[2 * (j + 3 * q) + 1];
                if (Ns > 1)
                {
                    int t1 = k * step, t2 = 2 * k * step, t3 = 3 * k * step;
                    ORC_REAL wr, wi, tr;
                    wr = tw[2 * t1]; wi = tw[2 * t1 + 1];
                    tr = v1r * wr - v1i * wi; v1i = v1r * wi + v1i * wr; v1r = tr;
                    wr = tw[2 * t2]; wi = tw[2 * t2 + 1];
                    tr = v2r * wr - v2i * wi; v2i = v2r * wi + v2i * wr; v2r = tr;
                    wr = tw[2 * t3]; wi = tw[2 * t3 + 1];
                    tr = v3r * wr - v3i * wi; v3i = v3r * wi + v3i * wr; v3r = tr;
                }
                ORC_REAL ar = v0r + v2r, ai = v0i + v2i; /* v0+v2 */
                ORC_REAL br = v0r - v2r, bi = v0i - v2i; /* v0-v2 */
                ORC_REAL cr = v1r + v3r, ci = v1i + v3i; /* v1+v3 */
                ORC_REAL dr = v1r - v3r, di = v1i - v3i; /* v1-v3 */
                /* W = s*i ; W*d = s*(-di + i dr) */
                ORC_REAL wdr = -s * di, wdi = s * dr;
                dst[2 * base] = ar + cr;
                dst[2 * base + 1] = ai + ci;
                dst[2 * (base + Ns)] = br + wdr;
                dst[2 * (base + Ns) + 1] = bi + wdi;
                dst[2 * (base + 2 * Ns)] = ar - cr;
                dst[2 * (base + 2 * Ns) + 1] = ai - ci;
                dst[2 * (base + 3 * Ns)] = br - wdr;
                dst[2 * (base + 3 * Ns) + 1] = bi - wdi;
            }
            else
            {
                ORC_REAL v0r = src[2 * j], v0i = src[2 * j + 1];
                ORC_REAL v1r = src[2 * (j + q)], v1i = src[2 * (j + q) + 1];
                if (Ns > 1)
                {
                    int t1 = k * step;
                    ORC_REAL wr = tw[2 * t1], wi = tw[2 * t1 + 1];
                    ORC_REAL tr = v1r * wr - v1i * wi;
                    v1i = v1r * wi + v1i * wr;
                    v1r = tr;
                }
                dst[2 * base] = v0r + v1r;
                dst[2 * base + 1] = v0i + v1i;
                dst[2 * (base + Ns)] = v0r - v1r;
                dst[2 * (base + Ns) + 1] = v0i - v1i;
            }
        }
        ORC_REAL *t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    if (src != x)
        memcpy(x, src, sizeof(ORC_REAL) * 2 * (size_t)n);
}

#undef ORC_FN
#undef ORC_CAT
#undef ORC_CAT2
