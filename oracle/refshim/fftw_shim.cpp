/*
 * ORACLE build shim -- FFTW3f-API transforms for the reference planning build.
 * Iterative radix-2 in double precision, output rounded to float.  Sign and
 * scaling follow FFTW: FFTW_FORWARD = exp(-2 pi i nk/N), unnormalised both ways.
 */
#include "fftw3.h"
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

struct orc_fftwf_plan_s
{
    int n;
    int sign;
    fftwf_complex *in;
    fftwf_complex *out;
};

extern "C" void *fftwf_malloc(size_t n) { return std::malloc(n); }
extern "C" void fftwf_free(void *p) { std::free(p); }

extern "C" fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned)
{
    fftwf_plan p = new orc_fftwf_plan_s;
    p->n = n;
    p->sign = sign;
    p->in = in;
    p->out = out;
    return p;
}

static void dft_double(int n, int sign, const fftwf_complex *in, fftwf_complex *out)
{
    std::vector<double> re(n), im(n);
    int bits = 0;
    while ((1 << bits) < n)
        bits++;
    for (int i = 0; i < n; i++)
    {
        int r = 0;
        for (int b = 0; b < bits; b++)
            if (i & (1 << b))
                r |= 1 << (bits - 1 - b);
        re[r] = in[i][0];
        im[r] = in[i][1];
    }
    const double PI = 3.14159265358979323846;
    for (int len = 2; len <= n; len <<= 1)
    {
        int half = len / 2;
        for (int k = 0; k < half; k++)
        {
            double a = 2.0 * PI * (double)k / (double)len;
            double wr = std::cos(a), wi = sign * std::sin(a);
            for (int s = 0; s < n; s += len)
            {
                int i0 = s + k, i1 = s + k + half;
                double xr = re[i1] * wr - im[i1] * wi;
                double xi = re[i1] * wi + im[i1] * wr;
                re[i1] = re[i0] - xr;
                im[i1] = im[i0] - xi;
                re[i0] += xr;
                im[i0] += xi;
            }
        }
    }
    for (int i = 0; i < n; i++)
    {
        out[i][0] = (float)re[i];
        out[i][1] = (float)im[i];
    }
}

extern "C" void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out)
{
    dft_double(p->n, p->sign, in, out);
}

extern "C" void fftwf_execute(const fftwf_plan p) { dft_double(p->n, p->sign, p->in, p->out); }

extern "C" void fftwf_destroy_plan(fftwf_plan p) { delete p; }
