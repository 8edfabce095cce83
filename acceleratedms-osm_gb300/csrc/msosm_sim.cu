// Simulated dispersed-pulsar baseband on the GPU: the simulated_pulsar front end
// (simulated_pulsar/simulated_complex_signal.cpp, simulated_pulsar/AWGN.cpp).
//
// Signal model, per output sample e (sample rate fs = bw):
//   emission x[i]:  pulse kinds
//     TEST_PULSE  three Gaussian components at phases 0.455 / 0.500 / 0.555
//                 (generate_test_pulse, simulated_complex_signal.cpp:44-72), peak
//                 amplitude 10000, times complex unit-variance Gaussian noise: every
//                 period is an independent realisation
//     GAUSSIAN    one Gaussian component of FWHM duty*period at phase 0.5, same
//                 amplitude convention
//     IMPULSES    two real impulses of 32767 at samples Np/2 and Np/2 + 2 of every
//                 period (generate_pulsar_signal, :563-571), deterministic
//   dispersion:     y = h * x with h the causal dispersion impulse response
//                 (:347-395; plan_dispersion_response in msosm_plan.cpp), applied by
//                 the engine's own overlap-save transform; the output skips the
//                 response's Nd-sample delay (:438-442), so dedispersion puts the pulse
//                 back at its emitted phase
//   noise:          optional complex AWGN at a per-sample SNR against the emission's
//                 mean power (AWGN.cpp:20-58 with sigma = sqrt(10^(-SNR'/10)),
//                 SNR' = SNR - signal power in dB, simulated_complex_signal.cpp:599-604)
//   output formats: complex64; uint16 offset-binary pairs (0 kept for "no data",
//                 :657-658, otherwise trunc(v + 32768) clamped to [0, 65535]); int8
//                 interleaved I/Q (round, clipped to [-127, 127]); all after a scale.
// Random numbers come from a counter-based generator (Philox-4x32-10, Salmon et al.,
// SC'11) keyed by the seed and indexed by the sample, so every sample is independent
// of how the stream is cut into calls; Gaussian pairs from the Box-Muller transform.
#include "msosm_gb300.h"
#include "msosm_internal.h"
#include "msosm_plan.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

namespace {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

// Philox-4x32-10: ten rounds of two 32x32->64 multiplies with a Weyl key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; r++)
    {
        const uint32_t hi0 = __umulhi(kPhiloxM0, c.x), lo0 = kPhiloxM0 * c.x;
        const uint32_t hi1 = __umulhi(kPhiloxM1, c.z), lo1 = kPhiloxM1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += kPhiloxW0;
        k.y += kPhiloxW1;
    }
    return c;
}

// Two independent N(0,1) values for sample i of stream `stream` (0 emission,
// 1 additive noise, 2 stand-alone AWGN): Box-Muller on the top 24 bits of two words.
__device__ __forceinline__ float2 normal_pair(unsigned long long seed, uint32_t stream, unsigned long long i)
{
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), stream, 0u),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const float u1 = ((float)(r.x >> 8) + 0.5f) * 5.9604644775390625e-8f; // (0, 1]
    const float u2 = (float)(r.y >> 8) * 5.9604644775390625e-8f;          // [0, 1)
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    return make_float2(rad * c, rad * s);
}

struct PulseArgs
{
    int kind;
    unsigned long long Np;
    float amp;       // profile -> amplitude of each quadrature (peak 10000 / sqrt 2)
    float inv_sigma; // GAUSSIAN: 1 / (component width in turns)
    unsigned long long seed;
};

__device__ __forceinline__ float gauss_bump(float x, float mu, float inv_w)
{
    const float z = (x - mu) * inv_w;
    return expf(-0.5f * z * z);
}

// Emission samples i0 .. i0+n-1 of the pulse train.
__global__ void sim_pulse_kernel(float2 *__restrict__ x, unsigned long long i0, unsigned long long n, PulseArgs p)
{
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x)
    {
        const unsigned long long i = i0 + k;
        const unsigned long long j = i % p.Np;
        float2 v;
        if (p.kind == MSOSM_SIM_IMPULSES)
        {
            const bool hit = j == p.Np / 2 || j == p.Np / 2 + 2;
            v = make_float2(hit ? 32767.0f : 0.0f, 0.0f);
        }
        else
        {
            const float ph = (float)j / (float)p.Np;
            float prof;
            if (p.kind == MSOSM_SIM_TEST_PULSE)
                prof = 0.45f * gauss_bump(ph, 0.455f, 125.0f) + gauss_bump(ph, 0.5f, 1.0f / 0.012f) +
                       0.28f * gauss_bump(ph, 0.555f, 1.0f / 0.006f);
            else
                prof = gauss_bump(ph, 0.5f, p.inv_sigma);
            const float a = prof * p.amp;
            const float2 g = normal_pair(p.seed, 0u, i);
            v = make_float2(a * g.x, a * g.y);
        }
        x[k] = v;
    }
}

struct EmitArgs
{
    int fmt;
    float scale;
    float noise_sigma; // per quadrature; 0 = no noise
    unsigned long long seed;
};

__device__ __forceinline__ uint32_t enc_u16(float c)
{
    if (c == 0.0f)
        return 0u;
    return __float2uint_rz(fminf(fmaxf(c + 32768.0f, 0.0f), 65535.0f));
}

__device__ __forceinline__ signed char enc_i8(float c) { return (signed char)(int)fminf(fmaxf(rintf(c), -127.0f), 127.0f); }

// Output samples e0 .. e0+n-1 from the dispersed series y (y[k] is sample e0 + k):
// add noise, scale, encode.
__global__ void sim_emit_kernel(const float2 *__restrict__ y, unsigned long long e0, unsigned long long n,
                                void *__restrict__ out, EmitArgs a)
{
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x)
    {
        float2 v = y[k];
        if (a.noise_sigma > 0.0f)
        {
            const float2 g = normal_pair(a.seed, 1u, e0 + k);
            v.x += a.noise_sigma * g.x;
            v.y += a.noise_sigma * g.y;
        }
        v.x *= a.scale;
        v.y *= a.scale;
        if (a.fmt == MSOSM_IN_C64)
            static_cast<float2 *>(out)[k] = v;
        else if (a.fmt == MSOSM_IN_U16)
            static_cast<uint32_t *>(out)[k] = enc_u16(v.x) | (enc_u16(v.y) << 16);
        else
        {
            char2 o;
            o.x = enc_i8(v.x);
            o.y = enc_i8(v.y);
            static_cast<char2 *>(out)[k] = o;
        }
    }
}

__global__ void awgn_kernel(float2 *__restrict__ out, unsigned long long i0, unsigned long long n, float mean,
                            float stddev, unsigned long long seed)
{
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x)
    {
        const float2 g = normal_pair(seed, 2u, i0 + k);
        out[k] = make_float2(mean + stddev * g.x, mean + stddev * g.y);
    }
}

size_t fmt_bytes(int fmt)
{
    switch (fmt)
    {
    case MSOSM_IN_C64: return 8;
    case MSOSM_IN_U16: return 4;
    case MSOSM_IN_I8: return 2;
    default: return 0;
    }
}

int launch_grid(unsigned long long n)
{
    const unsigned long long blocks = (n + 255) / 256;
    return (int)std::max<unsigned long long>(1, std::min<unsigned long long>(blocks, 152ull * 16));
}

bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

constexpr unsigned long long kChunkTarget = 1ull << 23; // emission samples per filter call

double profile_value(int kind, double x, double duty)
{
    if (kind == MSOSM_SIM_TEST_PULSE)
        return 0.45 * std::exp(-0.5 * std::pow((x - 0.455) / 0.008, 2.0)) +
               std::exp(-0.5 * std::pow((x - 0.5) / 0.012, 2.0)) +
               0.28 * std::exp(-0.5 * std::pow((x - 0.555) / 0.006, 2.0));
    const double sig = duty / (2.0 * std::sqrt(2.0 * std::log(2.0)));
    return std::exp(-0.5 * std::pow((x - 0.5) / sig, 2.0));
}

} // namespace

struct msosm_sim_s
{
    float bw = 0, f0 = 0, dm = 0, period = 0;
    unsigned long long Np = 0, nd = 0;
    int kind = MSOSM_SIM_TEST_PULSE;
    float duty = 0.05f;
    bool noise = false;
    float snr_db = 0.0f;
    unsigned long long seed = 1;
    // dispersion filter: an overlap-save handle of order M, B windows per call
    msosm_t *filt = nullptr;
    int M = 0, B = 0;
    unsigned long long chunk = 0; // B * M samples per filter call
    float2 *d_x = nullptr;        // one chunk of emission
    void *d_stage = nullptr;      // one chunk of encoded output for host destinations
    double p_sig = 0, peak = 1;   // mean emission power per sample, profile maximum
    long long cur_chunk = -1;     // the filter's output holds y of this chunk
    unsigned long long pos = 0;   // next output sample
    bool started = false;
    std::string err;

    int fail(int code, const std::string &m)
    {
        err = m;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return MSOSM_ERR_CUDA;
    }
    // profile maximum over one period and mean |x|^2 per sample (both quadratures:
    // amplitude^2 of each times 2 = (profile * 10000 / peak)^2)
    void measure()
    {
        if (kind == MSOSM_SIM_IMPULSES)
        {
            peak = 1.0;
            p_sig = 2.0 * 32767.0 * 32767.0 / (double)Np;
            return;
        }
        std::vector<double> prof(Np);
        double mx = 0;
        for (unsigned long long j = 0; j < Np; j++)
        {
            prof[j] = profile_value(kind, (double)j / (double)Np, (double)duty);
            mx = std::max(mx, prof[j]);
        }
        double sum = 0;
        const double scale = 10000.0 / mx;
        for (unsigned long long j = 0; j < Np; j++)
            sum += (prof[j] * scale) * (prof[j] * scale);
        peak = mx;
        p_sig = sum / (double)Np;
    }
    double noise_sigma() const { return noise ? std::sqrt(p_sig / std::pow(10.0, snr_db / 10.0) / 2.0) : 0.0; }
    void release()
    {
        if (filt)
            msosm_destroy(filt);
        filt = nullptr;
        if (d_x)
            cudaFree(d_x);
        if (d_stage)
            cudaFree(d_stage);
        d_x = nullptr;
        d_stage = nullptr;
    }
    ~msosm_sim_s() { release(); }
};

extern "C" int msosm_sim_create(float bw, float f0, float dm, float period, msosm_sim_t **out)
{
    if (!out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (!(bw > 0) || !(f0 > 0) || !(dm >= 0) || !(period > 0))
        return MSOSM_ERR_ARG;
    const float fs = bw;
    const unsigned long long Np = (unsigned long long)(period * fs); // float product, truncated (:27)
    if (Np < 8)
        return MSOSM_ERR_ARG;
    msosm_sim_t *s = new (std::nothrow) msosm_sim_s();
    if (!s)
        return MSOSM_ERR_NOMEM;
    s->bw = bw;
    s->f0 = f0;
    s->dm = dm;
    s->period = period;
    s->Np = Np;
    s->nd = msosm::plan_osm_nd(bw, dm, f0); // the simulator's Nd expression (:28) is Prepare_OSM's
    s->measure();
    *out = s;
    return MSOSM_OK;
}

extern "C" int msosm_sim_set_pulse(msosm_sim_t *s, int kind, float duty)
{
    if (!s)
        return MSOSM_ERR_ARG;
    if (s->started)
        return s->fail(MSOSM_ERR_STATE, "set_pulse after the first generate");
    if (kind != MSOSM_SIM_TEST_PULSE && kind != MSOSM_SIM_GAUSSIAN && kind != MSOSM_SIM_IMPULSES)
        return s->fail(MSOSM_ERR_ARG, "unknown pulse kind");
    if (kind == MSOSM_SIM_GAUSSIAN && !(duty > 0 && duty < 1))
        return s->fail(MSOSM_ERR_ARG, "duty must be in (0, 1)");
    s->kind = kind;
    s->duty = duty;
    s->measure();
    return MSOSM_OK;
}

extern "C" int msosm_sim_set_noise(msosm_sim_t *s, int enable, float snr_db)
{
    if (!s)
        return MSOSM_ERR_ARG;
    if (s->started)
        return s->fail(MSOSM_ERR_STATE, "set_noise after the first generate");
    s->noise = enable != 0;
    s->snr_db = snr_db;
    return MSOSM_OK;
}

extern "C" int msosm_sim_set_seed(msosm_sim_t *s, unsigned long long seed)
{
    if (!s)
        return MSOSM_ERR_ARG;
    if (s->started)
        return s->fail(MSOSM_ERR_STATE, "set_seed after the first generate");
    s->seed = seed;
    return MSOSM_OK;
}

extern "C" int msosm_sim_info(const msosm_sim_t *s, unsigned long long *period_samples, unsigned long long *nd,
                              double *signal_power, double *noise_sigma)
{
    if (!s)
        return MSOSM_ERR_ARG;
    if (period_samples)
        *period_samples = s->Np;
    if (nd)
        *nd = s->nd;
    if (signal_power)
        *signal_power = s->p_sig;
    if (noise_sigma)
        *noise_sigma = s->noise_sigma();
    return MSOSM_OK;
}

// Set-up on the first generate: the dispersion filter (order M = next_pow2(Nd + 1),
// at least 2^15, so the response's Nd + 1 taps fit one overlap) and the buffers.
static int sim_setup(msosm_sim_t *s)
{
    int M = 1 << 15;
    while ((unsigned long long)M < s->nd + 1)
        M <<= 1;
    if (2ll * M > (1ll << 24))
        return s->fail(MSOSM_ERR_UNSUPPORTED, "dispersion smear of 2^23 samples or more (Nd = " + std::to_string(s->nd) +
                                                  "): the filter transform would exceed 2^24 points");
    const int B = (int)std::max<unsigned long long>(1, kChunkTarget / (unsigned long long)M);
    int rc = msosm_filter_create(s->bw, s->f0, M, &s->filt);
    if (rc != MSOSM_OK)
        return s->fail(rc, "filter create");
    if ((rc = msosm_init(s->filt, 2 * M, B, MSOSM_IN_C64, MSOSM_OUT_C64)) != MSOSM_OK)
        return s->fail(rc, std::string("filter init: ") + msosm_last_error(s->filt));
    std::vector<float> H(4 * (size_t)M);
    msosm::plan_dispersion_response(s->bw, s->f0, s->dm, s->nd, 2 * M, H.data());
    if ((rc = msosm_set_response(s->filt, 0, H.data())) != MSOSM_OK)
        return s->fail(rc, std::string("filter response: ") + msosm_last_error(s->filt));
    s->M = M;
    s->B = B;
    s->chunk = (unsigned long long)B * M;
    cudaError_t e;
    if ((e = cudaMalloc(&s->d_x, s->chunk * sizeof(float2))) != cudaSuccess)
        return s->cuda_fail(e, "cudaMalloc(emission)");
    if ((e = cudaMalloc(&s->d_stage, s->chunk * sizeof(float2))) != cudaSuccess)
        return s->cuda_fail(e, "cudaMalloc(stage)");
    s->started = true;
    return MSOSM_OK;
}

extern "C" int msosm_sim_generate(msosm_sim_t *s, unsigned long long n, int out_format, float scale, void *out,
                                  void *stream)
{
    if (!s)
        return MSOSM_ERR_ARG;
    if (!out && n)
        return s->fail(MSOSM_ERR_ARG, "null output");
    const size_t eb = fmt_bytes(out_format);
    if (!eb)
        return s->fail(MSOSM_ERR_ARG, "unknown output format");
    if (!s->started)
    {
        int rc = sim_setup(s);
        if (rc != MSOSM_OK)
            return rc;
    }
    if (n == 0)
        return MSOSM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = on_device(out);
    const EmitArgs ea{out_format, scale, (float)s->noise_sigma(), s->seed};
    const PulseArgs pa{s->kind, s->Np, (float)(10000.0 / s->peak / std::sqrt(2.0)),
                       (float)((2.0 * std::sqrt(2.0 * std::log(2.0))) / (double)s->duty), s->seed};
    // output sample e is y[e + Nd]; call c of the filter yields y[c*chunk .. (c+1)*chunk)
    const unsigned long long y_begin = s->pos + s->nd, y_end = y_begin + n;
    cudaError_t e;
    for (unsigned long long y = y_begin; y < y_end;)
    {
        const long long c = (long long)(y / s->chunk);
        while (s->cur_chunk < c)
        {
            // the filter sees every emission chunk in order (its overlap state)
            const long long next = s->cur_chunk + 1;
            sim_pulse_kernel<<<launch_grid(s->chunk), 256, 0, st>>>(s->d_x, (unsigned long long)next * s->chunk,
                                                                  s->chunk, pa);
            if ((e = cudaGetLastError()) != cudaSuccess)
                return s->cuda_fail(e, "pulse kernel launch");
            const int rc = msosm_process(s->filt, s->d_x, st);
            if (rc != MSOSM_OK)
                return s->fail(rc, std::string("filter: ") + msosm_last_error(s->filt));
            s->cur_chunk = next;
        }
        const unsigned long long c_end = (unsigned long long)(c + 1) * s->chunk;
        const unsigned long long take = std::min(y_end, c_end) - y;
        const float2 *ysrc =
            static_cast<const float2 *>(msosm_device_output(s->filt)) + (y - (unsigned long long)c * s->chunk);
        const unsigned long long e0 = y - s->nd; // output sample index of ysrc[0]
        unsigned char *dst = static_cast<unsigned char *>(out) + (size_t)(e0 - s->pos) * eb;
        sim_emit_kernel<<<launch_grid(take), 256, 0, st>>>(ysrc, e0, take, dev ? (void *)dst : s->d_stage, ea);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return s->cuda_fail(e, "emit kernel launch");
        if (!dev)
        {
            if ((e = cudaMemcpyAsync(dst, s->d_stage, (size_t)take * eb, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return s->cuda_fail(e, "copy to host");
        }
        y += take;
    }
    s->pos += n;
    return MSOSM_OK;
}

extern "C" unsigned long long msosm_sim_position(const msosm_sim_t *s) { return s ? s->pos : 0; }

extern "C" const char *msosm_sim_last_error(const msosm_sim_t *s) { return s ? s->err.c_str() : "null handle"; }

extern "C" int msosm_sim_destroy(msosm_sim_t *s)
{
    if (!s)
        return MSOSM_ERR_ARG;
    delete s;
    return MSOSM_OK;
}

extern "C" int msosm_awgn(unsigned long long seed, unsigned long long first, unsigned long long n, float mean,
                          float stddev, float *out, void *stream)
{
    if (!out && n)
        return MSOSM_ERR_ARG;
    if (n == 0)
        return MSOSM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (on_device(out))
    {
        awgn_kernel<<<launch_grid(n), 256, 0, st>>>(reinterpret_cast<float2 *>(out), first, n, mean, stddev, seed);
        return cudaGetLastError() == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
    }
    const unsigned long long chunk = std::min<unsigned long long>(n, 1ull << 24);
    float2 *d = nullptr;
    if (cudaMalloc(&d, chunk * sizeof(float2)) != cudaSuccess)
        return MSOSM_ERR_CUDA;
    int rc = MSOSM_OK;
    for (unsigned long long k = 0; k < n; k += chunk)
    {
        const unsigned long long m = std::min(chunk, n - k);
        awgn_kernel<<<launch_grid(m), 256, 0, st>>>(d, first + k, m, mean, stddev, seed);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(out + 2 * k, d, m * sizeof(float2), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
        {
            rc = MSOSM_ERR_CUDA;
            break;
        }
    }
    cudaFree(d);
    return rc;
}
