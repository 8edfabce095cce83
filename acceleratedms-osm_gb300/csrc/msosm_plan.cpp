// Host-side planning of the MS-OSM engine (see msosm_plan.h).
#include "msosm_plan.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>

namespace msosm {

namespace {
constexpr double kPi = 3.14159265358979323846; // M_PI, as utils/include/globals.h:30

// kdm = 4.15 * 1e15 kept as float by Prepare_MSOSM (msosm_prepare.h:54)
inline float kdm_float() { return (float)(4.15 * 1e15); }

double nd_value(float bw, float dm, float f0)
{
    const float fs = bw;
    const float kd = kdm_float() * dm;     // float product
    const float f1 = f0 + bw;               // float sum
    const double a = 1.0 / ((double)f0 * (double)f0); // pow(f0,2): square of a float is exact in double
    const double b = 1.0 / ((double)f1 * (double)f1);
    const float inv_fs = 1.0f / fs;         // float quotient
    return std::floor((double)kd * (a - b) / (double)inv_fs);
}
} // namespace

int plan_nd(float bw, float dm, float f0) { return (int)nd_value(bw, dm, f0); }

unsigned long plan_osm_nd(float bw, float dm, float f0) { return (unsigned long)nd_value(bw, dm, f0); }

int plan_min_order(int nd)
{
    const double order = std::sqrt(1024 / 2.0) * std::sqrt((double)nd); // MIN_SEGMENT_POINTS = 1024
    return (int)std::pow(2.0, std::ceil(std::log2(order)));
}

unsigned long plan_osm_min_order(unsigned long nd)
{
    int n = (int)nd; // Prepare_OSM::next_power_of_2 takes an int
    int p = 1;
    if (n > 0)
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

int plan_delaycount(int nd, int M) { return (int)std::ceil((float)nd / (float)M); }

int plan_segmentation(float bw, float f0, float dm, int nd, int M, uint16_t *delay)
{
    const int F = 2 * M;
    const float fs = bw;
    const float kdm = kdm_float();
    const float w0 = (float)(2 * kPi * (double)f0);
    const int dc = plan_delaycount(nd, M);
    std::fill(delay, delay + F, (uint16_t)0);
    if (dc <= 0)
        return dc;
    // boundary frequencies in units of pi*fs, stored as float like the reference's w[]
    std::vector<float> w(dc + 1);
    w[0] = -1.0f;
    w[dc] = 1.0f;
    int pos_index = 1;
    const double w0sq_inv = 1.0 / ((double)w0 * (double)w0);
    const double den = 4 * kPi * kPi * (double)kdm * (double)dm;
    for (int j = 1; j < dc; j++)
    {
        const float jm_fs = (float)(j * M) / fs;
        const double inner = w0sq_inv - (double)jm_fs / den;
        w[j] = (float)(((std::sqrt(1.0 / inner) - (double)w0) - kPi * (double)fs) / kPi / (double)fs);
        if (w[j] < 0)
            pos_index = j + 1;
    }
    // Negative-frequency bins [M, 2M) carry delays 0..negcount-1 from the band
    // bottom upward; positive bins [0, M) continue from negcount-1.  Written in the
    // reference's loop order so overlapping ranges resolve identically.
    const int negcount = pos_index;
    const int poscount = dc - pos_index + 1;
    std::vector<int> segneg(negcount + 1), segpos(poscount + 1);
    for (int j = 0; j < negcount; j++)
        segneg[j] = (int)std::floor((w[j] + 2.0f) * (float)M);
    segneg[negcount] = 2 * M;
    segpos[0] = 0;
    for (int j = 0; j < poscount; j++)
        segpos[j + 1] = (int)std::floor(w[j + negcount] * (float)M);
    for (int j = 0; j < negcount; j++)
        for (int k = std::max(segneg[j], 0); k < std::min(segneg[j + 1], F); k++)
            delay[k] = (uint16_t)j;
    for (int j = 0; j < poscount; j++)
        for (int k = std::max(segpos[j], 0); k < std::min(segpos[j + 1], F); k++)
            delay[k] = (uint16_t)(negcount - 1 + j);
    return dc;
}

namespace {

using cd = std::complex<double>;

// In-place iterative radix-2 FFT of length n (power of two) with a shared table
// tw[k] = exp(-2 pi i k / n), k < n/2.  sign -1 forward, +1 inverse (unnormalised).
void fft_inplace(cd *x, int n, int sign, const cd *tw)
{
    for (int i = 1, j = 0; i < n; i++)
    {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1)
            j ^= bit;
        j ^= bit;
        if (i < j)
            std::swap(x[i], x[j]);
    }
    for (int len = 2; len <= n; len <<= 1)
    {
        const int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len)
        {
            for (int k = 0; k < half; k++)
            {
                cd w = tw[k * step];
                if (sign > 0)
                    w = std::conj(w);
                const cd u = x[s + k], v = x[s + k + half] * w;
                x[s + k] = u + v;
                x[s + k + half] = u - v;
            }
        }
    }
}

std::vector<cd> make_table(int n)
{
    std::vector<cd> tw(n / 2 > 0 ? n / 2 : 1);
    for (int k = 0; k < n / 2; k++)
    {
        const double a = 2.0 * kPi * (double)k / (double)n;
        tw[k] = cd(std::cos(a), -std::sin(a));
    }
    return tw;
}

// H = FFT_2M(zero-pad(IFFT_M(c)/M)) evaluated as
//   H[2k]   = c[k]                                (FFT_M undoes IFFT_M)
//   H[2k+1] = FFT_M(h[j] * exp(-i pi j / M))[k],  h = IFFT_M(c)/M
// which needs two M-point transforms instead of an M- and a 2M-point one.
// derivative == true gives dH/dDM: the chirp's phase is linear in DM, so
// d/dDM exp(-i phi) = -i (phi/DM) exp(-i phi), and the construction is linear.
void response_into(float bw, float f0, float dm, int M, float *Hout, const cd *tw, const cd *twist, cd *c, cd *h,
                   bool derivative)
{
    const double kdm_d = 4.15e15;
    const double fs_d = (double)bw, dm_d = (double)dm, f0_d = (double)f0;
    const double w0_d = 2.0 * kPi * f0_d;
    const double step = 2.0 * kPi * fs_d / (double)M;
    for (int j = 0; j < M; j++)
    {
        const double w = step * (double)j;
        const double phase = 4.0 * kPi * kPi * kdm_d * dm_d * w * w / ((w + w0_d) * w0_d * w0_d);
        const int dst = (j < M / 2) ? (M / 2 + j) : (j - M / 2);
        c[dst] = cd(std::cos(phase), -std::sin(phase));
        if (derivative)
        {
            const double per_dm = 4.0 * kPi * kPi * kdm_d * w * w / ((w + w0_d) * w0_d * w0_d);
            c[dst] *= cd(0.0, -per_dm);
        }
    }
    std::memcpy((void *)h, (const void *)c, sizeof(cd) * (size_t)M);
    fft_inplace(h, M, +1, tw);
    const double invM = 1.0 / (double)M;
    for (int j = 0; j < M; j++)
        h[j] *= invM * twist[j];
    fft_inplace(h, M, -1, tw);
    for (int k = 0; k < M; k++)
    {
        Hout[4 * (size_t)k] = (float)c[k].real();
        Hout[4 * (size_t)k + 1] = (float)c[k].imag();
        Hout[4 * (size_t)k + 2] = (float)h[k].real();
        Hout[4 * (size_t)k + 3] = (float)h[k].imag();
    }
}

std::vector<cd> make_twist(int M)
{
    std::vector<cd> t(M);
    for (int j = 0; j < M; j++)
    {
        const double a = kPi * (double)j / (double)M;
        t[j] = cd(std::cos(a), -std::sin(a));
    }
    return t;
}

} // namespace

void plan_response(float bw, float f0, float dm, int M, float *Hout)
{
    plan_responses(bw, f0, &dm, 1, M, Hout, 1);
}

void plan_responses(float bw, float f0, const float *dms, int n, int M, float *Hout, int threads, bool derivative)
{
    if (n <= 0)
        return;
    const std::vector<cd> tw = make_table(M);
    const std::vector<cd> twist = make_twist(M);
    int nt = std::max(1, std::min(threads, n));
    auto work = [&](int t) {
        std::vector<cd> c(M), h(M);
        for (int i = t; i < n; i += nt)
            response_into(bw, f0, dms[i], M, Hout + (size_t)i * 4 * M, tw.data(), twist.data(), c.data(), h.data(),
                          derivative);
    };
    if (nt == 1)
    {
        work(0);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
        pool.emplace_back(work, t);
    for (auto &th : pool)
        th.join();
}

void plan_dispersion_response(float bw, float f0, float dm, unsigned long nd, int F, float *Hout)
{
    const double kdm_d = 4.15e15;
    const double fs_d = (double)bw, dm_d = (double)dm, f0_d = (double)f0;
    const double w0_d = 2.0 * kPi * f0_d;
    size_t fp = 1;
    while (fp < nd + 1)
        fp <<= 1;
    // chirp at fp bins: bin k < fp/2 sits fs/2 + k*fs/fp above the band's lower edge,
    // bin k >= fp/2 at k*fs/fp - fs/2
    std::vector<cd> h(fp);
    const double step = fs_d / (double)fp;
    for (size_t k = 0; k < fp; k++)
    {
        const double f = (k < fp / 2) ? fs_d / 2.0 + (double)k * step : (double)k * step - fs_d / 2.0;
        const double w = 2.0 * kPi * f;
        const double phase = 4.0 * kPi * kPi * kdm_d * dm_d * w * w / ((w + w0_d) * w0_d * w0_d);
        h[k] = cd(std::cos(phase), std::sin(phase));
    }
    if (fp > 1)
    {
        const std::vector<cd> tw = make_table((int)fp);
        fft_inplace(h.data(), (int)fp, +1, tw.data());
    }
    const double inv = 1.0 / (double)fp;
    // the response occupies indices fp-nd .. fp-1 and 0 (negative times): make it causal
    std::vector<cd> H((size_t)F, cd(0.0, 0.0));
    for (unsigned long j = 0; j < nd; j++)
        H[j] = h[fp - nd + j] * inv;
    H[nd] = h[0] * inv;
    const std::vector<cd> twF = make_table(F);
    fft_inplace(H.data(), F, -1, twF.data());
    for (int k = 0; k < F; k++)
    {
        Hout[2 * (size_t)k] = (float)H[k].real();
        Hout[2 * (size_t)k + 1] = (float)H[k].imag();
    }
}

} // namespace msosm
