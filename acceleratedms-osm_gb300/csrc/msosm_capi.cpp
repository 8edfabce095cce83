// C ABI of the MS-OSM engine (declared in include/msosm_gb300.h).
//
// Host orchestration of one streaming step, mirroring
// MSOSM_GPU_BATCH::filter_block_uint16 (dedispersion/msosm/msosm_gpu_batch.cpp:178-236):
//   1. new samples reach the device: host inputs are copied on the handle's copy
//      stream into one of two staging buffers (overlapping the previous step's
//      transforms), device inputs are read in place;
//   2. forward transforms of the B overlapping windows into ring slots
//      rbi..rbi+B-1, rbi = (step*B) mod fbs (increment_fft_output, :167-176); the
//      decode and the tail hand-over (increment_fft_input, :153-165) are fused in;
//   3. every (DM, window): gather x response -> inverse -> discard/scale -> outputs
//      and/or fold, as one persistent launch (F >= 2^16, msosm_persist.cu) or as
//      pass-1/pass-2 launch pairs over chunks sized for L2 (msosm_inverse.cu).
// The work is ordered on the caller's stream (the copy stream joins it through
// events); nothing synchronises the device.
#include "msosm_gb300.h"
#include "msosm_internal.h"

#include "msosm_kernels.cuh"
#include "msosm_persist.cuh"
#include "msosm_plan.h"
#include "msosm_tc.cuh"
#include "msosm_writer.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

using msosm::Geom;
using msosm::Twiddles;

namespace {

constexpr int kMinLog2F = 8;
constexpr int kMaxLog2F = 24;
constexpr size_t kIntermediateBudget = 64ull << 20; // bytes of pass-1 output kept per launch pair
constexpr unsigned kMaxFusedBins = 8192;
constexpr int kMaxSlots = 256;                            // intermediate slots of the persistent transform
constexpr unsigned long long kWaitTimeoutNs = 2000000000; // device-side wait limit (2 s)

size_t in_elem_bytes(int fmt)
{
    switch (fmt)
    {
    case MSOSM_IN_U16: return 4;
    case MSOSM_IN_C64: return 8;
    case MSOSM_IN_I8: return 2;
    default: return 0;
    }
}

bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

int ilog2(long long v)
{
    int l = 0;
    while ((1ll << l) < v)
        l++;
    return l;
}

// Fraction of a turn in Q0.64 fixed point.
uint64_t turns_q64(long double turns)
{
    long double f = turns - floorl(turns);
    long double v = ldexpl(f, 64);
    if (!(v < 18446744073709551616.0L))
        return 0;
    if (v < 0)
        return 0;
    return (uint64_t)v;
}

template <class T>
cudaError_t dalloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0)
        return cudaSuccess;
    return cudaMalloc((void **)p, count * sizeof(T));
}

void dfree(void *p)
{
    if (p)
        cudaFree(p);
}

// Kernel timing: with timing on, each launch is bracketed by a pair of CUDA
// events recorded on its stream; elapsed times are summed when read (after a
// stream sync), so timing never blocks the launch path.  Launches and
// transforms are counted whether or not timing is on.
struct Profiler
{
    static constexpr int KINDS = 5;
    bool on = false;
    long long launches[KINDS] = {};
    long long transforms[KINDS] = {};
    double ms[KINDS] = {};
    long long timed[KINDS] = {};
    struct Pending
    {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t cur = nullptr;

    cudaEvent_t get()
    {
        if (!pool.empty())
        {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        return e;
    }
    void begin(int, cudaStream_t st)
    {
        if (!on)
            return;
        cur = get();
        if (cur)
            cudaEventRecord(cur, st);
    }
    void end(int kind, cudaStream_t st, long long ntrans)
    {
        launches[kind]++;
        transforms[kind] += ntrans;
        if (!on || !cur)
            return;
        cudaEvent_t b = get();
        if (!b)
            return;
        cudaEventRecord(b, st);
        pending.push_back({kind, cur, b});
        cur = nullptr;
    }
    // Resolve recorded pairs; call after the stream(s) completed.
    cudaError_t collect()
    {
        for (auto &p : pending)
        {
            float t = 0.f;
            cudaError_t e = cudaEventElapsedTime(&t, p.a, p.b);
            if (e != cudaSuccess)
                return e;
            ms[p.kind] += t;
            timed[p.kind]++;
            pool.push_back(p.a);
            pool.push_back(p.b);
        }
        pending.clear();
        return cudaSuccess;
    }
    void reset()
    {
        collect();
        for (int k = 0; k < KINDS; k++)
        {
            launches[k] = transforms[k] = timed[k] = 0;
            ms[k] = 0;
        }
    }
    ~Profiler()
    {
        for (auto &p : pending)
        {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        for (auto e : pool)
            cudaEventDestroy(e);
    }
};

} // namespace

struct msosm_fold_s
{
    float period = 0, fs = 0;
    double P = 0, dt = 0, t_start = 0;
    unsigned long size = 0, K = 0;
    int S = 0;
    double *d_sum = nullptr;
    unsigned long long *d_cnt = nullptr;
    float *d_folded = nullptr;
    float *d_pair = nullptr; // 2-pol fused fold: the first polarisation's |a|^2, num_series*size
    std::string err;

    msosm::FoldArgs args() const
    {
        msosm::FoldArgs a;
        a.sum = d_sum;
        a.cnt = d_cnt;
        a.phase0 = turns_q64((long double)t_start / (long double)P);
        a.dphase = turns_q64((long double)dt / (long double)P);
        a.K = (unsigned)K;
        return a;
    }
    ~msosm_fold_s()
    {
        dfree(d_sum);
        dfree(d_cnt);
        dfree(d_folded);
        dfree(d_pair);
    }
};

struct msosm_s
{
    bool osm = false;
    float bw = 0, f0 = 0;
    std::vector<float> dms;
    int D = 0;
    std::vector<int> nd, dc;
    int M_min = 0, M = 0, F = 0, B = 0, fbs = 0, delaycount = 0;
    int in_format = 0, out_mode = 0;
    bool inited = false;
    Geom g{};
    // device state
    float2 *d_ring = nullptr;
    float2 *d_H = nullptr;
    uint16_t *d_delays = nullptr;
    float2 *d_T = nullptr;
    int T_cap = 0;
    float2 *d_tail[2] = {nullptr, nullptr};
    int tail_cur = 0;
    void *d_in = nullptr;  // host-input staging, two buffers: the copy of call s+1
    void *d_in2 = nullptr; // overlaps the transforms of call s (the reference's stream mode)
    cudaStream_t copy_st = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_consumed[2] = {nullptr, nullptr};
    int in_buf = 0;
    float2 *d_out_c64 = nullptr;
    uint32_t *d_out_u16 = nullptr;
    float2 *d_tw = nullptr;
    Twiddles tw_fwd{}, tw_inv{};
    // persistent inverse transform (F >= 2^16): ticket + per-slot counters, error flag
    bool persist = false;
    int sms = 0;
    int T_slots = 0;
    unsigned *d_sync = nullptr; // [1 + 2*kMaxSlots]
    int *d_err = nullptr;
    long long step = 0;
    msosm_fold_t *fold = nullptr;
    msosm_writer_s *writer = nullptr;
    // split-precision transform (tensor cores): precision, W_32 operand image, FP16
    // operand-scale bound (running max |component| of the ring) and max |H|
    int precision = msosm::PREC_FP32;
    msosm::PersistPlan last_plan{}; // geometry of the last persistent launch
    void *d_tc_op = nullptr;
    unsigned *d_absmax = nullptr;
    float hmax = 1.0f;
    uint64_t *graph_phase = nullptr; // while capturing a graph: the fold's device-resident phase
    int ctas_per_sm = 0;              // launch shape of the persistent transform (0 = as many as fit)
    int dm_group = 0;                 // transform order: DM trials per window-major group (0: by size)
    float *pair_out = nullptr;      // first polarisation of a 2-pol fused fold: |a|^2 goes here
    const float *pair_in = nullptr; // second polarisation: folds sqrt(pair_in + |b|^2)
    Profiler prof;
    std::string err;

    int fail(int code, const std::string &msg)
    {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        const char *detail = msosm::launch_failure_detail();
        if (detail && *detail)
            err += std::string(" [") + detail + "]";
        msosm::set_launch_failure_detail("", "", 0, 0, 0, 0);
        (void)cudaGetLastError(); // a non-sticky error must not surface in a later call
        return MSOSM_ERR_CUDA;
    }
    void release()
    {
        dfree(d_ring);
        dfree(d_H);
        dfree(d_delays);
        dfree(d_T);
        dfree(d_tail[0]);
        dfree(d_tail[1]);
        if (copy_st)
            cudaStreamSynchronize(copy_st);
        dfree(d_in);
        dfree(d_in2);
        for (int i = 0; i < 2; i++)
        {
            if (ev_copied[i])
                cudaEventDestroy(ev_copied[i]);
            if (ev_consumed[i])
                cudaEventDestroy(ev_consumed[i]);
            ev_copied[i] = ev_consumed[i] = nullptr;
        }
        if (copy_st)
            cudaStreamDestroy(copy_st);
        copy_st = nullptr;
        in_buf = 0;
        dfree(d_out_c64);
        dfree(d_out_u16);
        dfree(d_tw);
        dfree(d_sync);
        dfree(d_err);
        dfree(d_tc_op);
        dfree(d_absmax);
        d_tc_op = nullptr;
        d_absmax = nullptr;
        precision = msosm::PREC_FP32;
        d_sync = nullptr;
        d_err = nullptr;
        d_ring = d_H = d_T = d_out_c64 = d_tw = nullptr;
        d_tail[0] = d_tail[1] = nullptr;
        d_delays = nullptr;
        d_in = d_in2 = nullptr;
        d_out_u16 = nullptr;
        inited = false;
    }
    ~msosm_s() { release(); }
};

// -----------------------------------------------------------------------------
extern "C" const char *msosm_version(void) { return "msosm_gb300 0.1 (sm_103a)"; }

extern "C" const char *msosm_status_string(int s)
{
    switch (s)
    {
    case MSOSM_OK: return "ok";
    case MSOSM_ERR_ARG: return "invalid argument";
    case MSOSM_ERR_STATE: return "call out of order";
    case MSOSM_ERR_CUDA: return "CUDA error";
    case MSOSM_ERR_NOMEM: return "out of memory";
    case MSOSM_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown status";
    }
}

// ---- host-only planning ------------------------------------------------------
extern "C" int msosm_plan_nd(float bw, float f0, const float *dms, int num_dms, int *nd_out)
{
    if (!dms || !nd_out || num_dms <= 0)
        return MSOSM_ERR_ARG;
    for (int i = 0; i < num_dms; i++)
        nd_out[i] = msosm::plan_nd(bw, dms[i], f0);
    return MSOSM_OK;
}

extern "C" int msosm_plan_min_order(const int *nd, int num_dms, int *M_min_out)
{
    if (!nd || !M_min_out || num_dms <= 0)
        return MSOSM_ERR_ARG;
    int m = 0;
    for (int i = 0; i < num_dms; i++)
        m = std::max(m, msosm::plan_min_order(nd[i]));
    *M_min_out = m;
    return MSOSM_OK;
}

extern "C" int msosm_plan_segmentation(float bw, float f0, float dm, int nd, int M, int *delay_out, int *dc_out)
{
    if (M <= 0 || !delay_out)
        return MSOSM_ERR_ARG;
    if (msosm::plan_delaycount(nd, M) > 65535)
        return MSOSM_ERR_UNSUPPORTED;
    std::vector<uint16_t> d((size_t)2 * M);
    const int dc = msosm::plan_segmentation(bw, f0, dm, nd, M, d.data());
    for (size_t i = 0; i < d.size(); i++)
        delay_out[i] = d[i];
    if (dc_out)
        *dc_out = dc;
    return MSOSM_OK;
}

extern "C" int msosm_plan_response(float bw, float f0, float dm, int M, float *H_out)
{
    if (M <= 0 || !is_pow2(M) || !H_out)
        return MSOSM_ERR_ARG;
    msosm::plan_response(bw, f0, dm, M, H_out);
    return MSOSM_OK;
}

extern "C" int osm_plan(float bw, float dm, float f0, unsigned long *nd_out, unsigned long *M_min_out)
{
    const unsigned long nd = msosm::plan_osm_nd(bw, dm, f0);
    if (nd_out)
        *nd_out = nd;
    if (M_min_out)
        *M_min_out = msosm::plan_osm_min_order(nd);
    return MSOSM_OK;
}

extern "C" int msosm_create(float bw, float f0, const float *dms, int num_dms, msosm_t **out)
{
    if (!out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (num_dms <= 0 || !dms || !(bw > 0) || !(f0 > 0))
        return MSOSM_ERR_ARG;
    for (int i = 0; i < num_dms; i++)
        if (!(dms[i] >= 0) || (i > 0 && dms[i] < dms[i - 1]))
            return MSOSM_ERR_ARG; // DMs must be non-negative and ascending
    msosm_t *h = new (std::nothrow) msosm_s();
    if (!h)
        return MSOSM_ERR_NOMEM;
    h->bw = bw;
    h->f0 = f0;
    h->dms.assign(dms, dms + num_dms);
    h->D = num_dms;
    h->nd.resize(num_dms);
    h->M_min = 0;
    for (int i = 0; i < num_dms; i++)
    {
        h->nd[i] = msosm::plan_nd(bw, dms[i], f0);
        h->M_min = std::max(h->M_min, msosm::plan_min_order(h->nd[i]));
    }
    *out = h;
    return MSOSM_OK;
}

extern "C" int osm_create(float bw, float dm, float f0, msosm_t **out)
{
    if (!out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (!(bw > 0) || !(f0 > 0) || !(dm >= 0))
        return MSOSM_ERR_ARG;
    msosm_t *h = new (std::nothrow) msosm_s();
    if (!h)
        return MSOSM_ERR_NOMEM;
    h->osm = true;
    h->bw = bw;
    h->f0 = f0;
    h->dms.assign(1, dm);
    h->D = 1;
    const unsigned long nd = msosm::plan_osm_nd(bw, dm, f0);
    h->nd.assign(1, (int)nd);
    const unsigned long mmin = msosm::plan_osm_min_order(nd);
    h->M_min = (int)std::min<unsigned long>(mmin, 1ul << 30);
    *out = h;
    return MSOSM_OK;
}

int msosm_filter_create(float bw, float f0, int M, msosm_t **out)
{
    if (!out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (!(bw > 0) || !(f0 > 0) || M < 1 || !is_pow2(M))
        return MSOSM_ERR_ARG;
    msosm_t *h = new (std::nothrow) msosm_s();
    if (!h)
        return MSOSM_ERR_NOMEM;
    h->osm = true;
    h->bw = bw;
    h->f0 = f0;
    h->dms.assign(1, 0.0f);
    h->D = 1;
    h->nd.assign(1, 0);
    h->M_min = M;
    *out = h;
    return MSOSM_OK;
}

// Largest |H| over interleaved (re, im) floats.
static float max_abs_complex(const std::vector<float> &H)
{
    double m = 0;
    for (size_t i = 0; i + 1 < H.size(); i += 2)
        m = std::max(m, std::hypot((double)H[i], (double)H[i + 1]));
    return (float)m;
}

static int build_twiddles(msosm_t *h)
{
    const int N1 = h->g.N1, N2 = h->g.N2, F = h->g.F;
    // per direction: twN1 (N1), twN2 (N2), lo (N2), hi (N1)
    const size_t per = (size_t)2 * N1 + 2 * N2;
    std::vector<float2> host(2 * per);
    const double PI = 3.14159265358979323846;
    for (int dir = 0; dir < 2; dir++)
    {
        const double sgn = dir == 0 ? -1.0 : 1.0;
        float2 *base = host.data() + dir * per;
        auto w = [&](long long m, long long n) {
            // exp(sgn*2*pi*i*m/n) with m reduced exactly
            const double a = 2.0 * PI * (double)(m % n) / (double)n;
            return make_float2((float)std::cos(a), (float)(sgn * std::sin(a)));
        };
        for (int m = 0; m < N1; m++)
            base[m] = w(m, N1);
        for (int m = 0; m < N2; m++)
            base[N1 + m] = w(m, N2);
        for (int m = 0; m < N2; m++)
            base[N1 + N2 + m] = w(m, F);
        for (int m = 0; m < N1; m++)
            base[N1 + 2 * N2 + m] = w((long long)m * N2, F);
    }
    cudaError_t e = dalloc(&h->d_tw, host.size());
    if (e != cudaSuccess)
        return h->cuda_fail(e, "cudaMalloc(twiddles)");
    e = cudaMemcpy(h->d_tw, host.data(), host.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "cudaMemcpy(twiddles)");
    for (int dir = 0; dir < 2; dir++)
    {
        float2 *base = h->d_tw + dir * per;
        Twiddles t{base, base + N1, base + N1 + N2, base + N1 + 2 * N2};
        (dir == 0 ? h->tw_fwd : h->tw_inv) = t;
    }
    return MSOSM_OK;
}

extern "C" int msosm_init(msosm_t *h, int fftpoint, int batch, int in_format, int out_mode)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (h->inited)
        return h->fail(MSOSM_ERR_STATE, "msosm_init called twice");
    if (batch <= 0)
        return h->fail(MSOSM_ERR_ARG, "batch must be positive");
    if (in_elem_bytes(in_format) == 0)
        return h->fail(MSOSM_ERR_ARG, "unknown input format");
    if (out_mode & ~(MSOSM_OUT_C64 | MSOSM_OUT_U16))
        return h->fail(MSOSM_ERR_ARG, "unknown output mode bits");
    if (fftpoint < 0)
        return h->fail(MSOSM_ERR_ARG, "fftpoint must be >= 0");
    // initialize_uint16's rule (msosm_gpu_batch.cpp:32-41 / osm_gpu_batch.cpp:27-37)
    int M = h->M_min;
    if (fftpoint != 0)
    {
        M = fftpoint / 2;
        if (M < h->M_min)
        {
            std::fprintf(stderr,
                         "Warning: The filter order is too small for the given FFT point. The minimum FFT point %d "
                         "is used.\n",
                         2 * h->M_min);
            M = h->M_min;
        }
    }
    const long long F = 2ll * M;
    if (!is_pow2(F) || ilog2(F) < kMinLog2F || ilog2(F) > kMaxLog2F)
        return h->fail(MSOSM_ERR_UNSUPPORTED, "FFT size " + std::to_string(F) + " outside [2^8, 2^24]");
    h->M = M;
    h->F = (int)F;
    h->B = batch;
    h->in_format = in_format;
    h->out_mode = out_mode;
    const int L = ilog2(F);
    h->g = Geom{L, (int)F, M, 1 << (L / 2), 1 << (L - L / 2)};

    // segmentation of every DM (msosm_gpu_batch.cpp:54-61)
    const size_t DF = (size_t)h->D * F;
    std::vector<uint16_t> delays(DF, 0);
    h->dc.assign(h->D, 0);
    h->delaycount = 0;
    if (!h->osm)
    {
        for (int i = 0; i < h->D; i++)
        {
            const int dc = msosm::plan_delaycount(h->nd[i], M);
            if (dc > 65535)
                return h->fail(MSOSM_ERR_UNSUPPORTED, "delaycount above 65535");
            h->dc[i] = msosm::plan_segmentation(h->bw, h->f0, h->dms[i], h->nd[i], M, delays.data() + (size_t)i * F);
            h->delaycount = std::max(h->delaycount, h->dc[i]);
        }
    }
    else
    {
        h->dc[0] = 1;
        h->delaycount = 1;
    }
    // ring of past spectra (msosm_gpu_batch.cpp:113-122), at least one batch
    int fbs = h->delaycount + batch - 1;
    if (fbs % batch)
        fbs += batch - fbs % batch;
    h->fbs = std::max(fbs, batch);

    // responses (msosm_gpu_batch.cpp:86-93) on host threads, FP64 inside
    std::vector<float> H(2 * DF);
    const int threads = (int)std::max(1u, std::thread::hardware_concurrency());
    msosm::plan_responses(h->bw, h->f0, h->dms.data(), h->D, M, H.data(), threads);
    h->hmax = max_abs_complex(H);

    cudaError_t e;
    const size_t ring_elems = (size_t)h->fbs * F;
    if ((e = dalloc(&h->d_ring, ring_elems)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMalloc(ring)");
    if ((e = cudaMemset(h->d_ring, 0, ring_elems * sizeof(float2))) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMemset(ring)");
    if ((e = dalloc(&h->d_H, DF)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMalloc(H)");
    if ((e = cudaMemcpy(h->d_H, H.data(), DF * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMemcpy(H)");
    if ((e = dalloc(&h->d_delays, DF)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMalloc(delays)");
    if ((e = cudaMemcpy(h->d_delays, delays.data(), DF * sizeof(uint16_t), cudaMemcpyHostToDevice)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMemcpy(delays)");
    const long long per_launch = (long long)(kIntermediateBudget / ((size_t)F * sizeof(float2)));
    h->T_cap = (int)std::max<long long>(batch, std::min<long long>((long long)h->D * batch, std::max(1ll, per_launch)));
    // persistent inverse transform: a few slots, enough for 2 CTAs per SM in flight
    h->persist = msosm::persist_supported(L);
    h->T_slots = h->T_cap;
    if (h->persist)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if ((e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaDeviceGetAttribute");
        // an upper bound of the kernel's plan (lag = ceil(2*grid/items per transform)
        // + 1, 2*lag slots) for any grid up to 4 CTAs per SM
        const int per_block = (int)(2 * F / 8192);
        const int lag_max = (2 * 4 * h->sms + per_block - 1) / per_block + 1;
        const int slots = std::min(kMaxSlots, 2 * lag_max);
        h->T_slots = std::max(batch, slots);
        if ((e = dalloc(&h->d_sync, (size_t)1 + 2 * kMaxSlots)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMalloc(sync)");
        if ((e = dalloc(&h->d_err, 1)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMalloc(err)");
        if ((e = cudaMemset(h->d_err, 0, sizeof(int))) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMemset(err)");
    }
    if ((e = dalloc(&h->d_T, (size_t)h->T_slots * F)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMalloc(intermediate)");
    for (int i = 0; i < 2; i++)
    {
        if ((e = dalloc(&h->d_tail[i], (size_t)M)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMalloc(tail)");
        if ((e = cudaMemset(h->d_tail[i], 0, (size_t)M * sizeof(float2))) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMemset(tail)");
    }
    const size_t in_bytes = (size_t)batch * M * in_elem_bytes(in_format);
    if ((e = cudaMalloc(&h->d_in, in_bytes)) != cudaSuccess || (e = cudaMalloc(&h->d_in2, in_bytes)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaMalloc(input)");
    if ((e = cudaStreamCreateWithFlags(&h->copy_st, cudaStreamNonBlocking)) != cudaSuccess)
        return h->release(), h->cuda_fail(e, "cudaStreamCreate(copy)");
    for (int i = 0; i < 2; i++)
        if ((e = cudaEventCreateWithFlags(&h->ev_copied[i], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&h->ev_consumed[i], cudaEventDisableTiming)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaEventCreate(copy)");
    const size_t out_elems = (size_t)h->D * batch * M;
    if (out_mode & MSOSM_OUT_C64)
        if ((e = dalloc(&h->d_out_c64, out_elems)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMalloc(output)");
    if (out_mode & MSOSM_OUT_U16)
        if ((e = dalloc(&h->d_out_u16, out_elems)) != cudaSuccess)
            return h->release(), h->cuda_fail(e, "cudaMalloc(output u16)");
    int rc = build_twiddles(h);
    if (rc != MSOSM_OK)
        return h->release(), rc;
    h->step = 0;
    h->tail_cur = 0;
    h->inited = true;
    return MSOSM_OK;
}

extern "C" int msosm_set_precision(msosm_t *h, int precision)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "set_precision before init");
    if (precision != MSOSM_PREC_FP32 && precision != MSOSM_PREC_BF16X3 && precision != MSOSM_PREC_FP16X3)
        return h->fail(MSOSM_ERR_ARG, "unknown precision");
    if (precision == MSOSM_PREC_FP32)
    {
        h->precision = msosm::PREC_FP32;
        return MSOSM_OK;
    }
    if (!h->persist || !msosm::tc_supported(h->g.L))
        return h->fail(MSOSM_ERR_UNSUPPORTED, "the split-precision transform is built for fftpoint 2^18 only");
    if ((unsigned long long)h->fbs * (unsigned long long)h->F >= (1ull << 32))
        return h->fail(MSOSM_ERR_UNSUPPORTED, "spectra ring too long for the split-precision transform");
    cudaError_t e;
    if (!h->d_tc_op && (e = cudaMalloc(&h->d_tc_op, 16384)) != cudaSuccess)
        return h->cuda_fail(e, "cudaMalloc(tensor-core operand)");
    if (!h->d_absmax && (e = dalloc(&h->d_absmax, 1)) != cudaSuccess)
        return h->cuda_fail(e, "cudaMalloc(spectra bound)");
    // the operand image and a bound covering every spectrum already in the ring
    if ((e = msosm::tc_build_operand(h->d_tc_op, precision == MSOSM_PREC_BF16X3, nullptr)) != cudaSuccess ||
        (e = cudaMemset(h->d_absmax, 0, sizeof(unsigned))) != cudaSuccess ||
        (e = msosm::tc_absmax(h->d_ring, (size_t)h->fbs * h->F, h->d_absmax, nullptr)) != cudaSuccess ||
        (e = cudaDeviceSynchronize()) != cudaSuccess)
        return h->cuda_fail(e, "set_precision");
    h->precision = precision == MSOSM_PREC_BF16X3 ? msosm::PREC_BF16X3 : msosm::PREC_FP16X3;
    return MSOSM_OK;
}

extern "C" int msosm_get_precision(const msosm_t *h)
{
    return h ? h->precision : -1;
}

extern "C" int msosm_reset_l2_persisting(void)
{
    return msosm::persist_l2_reset() == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
}

extern "C" int msosm_set_launch_shape(msosm_t *h, int ctas_per_sm, int dm_group)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (ctas_per_sm < 0 || ctas_per_sm > 4)
        return h->fail(MSOSM_ERR_ARG, "ctas_per_sm must be 0 (as many as fit) .. 4");
    if (dm_group < 0)
        return h->fail(MSOSM_ERR_ARG, "dm_group must be >= 0");
    h->ctas_per_sm = ctas_per_sm;
    if (dm_group > 0)
        h->dm_group = dm_group;
    return MSOSM_OK;
}

extern "C" int msosm_get_launch_info(const msosm_t *h, int *grid, int *occupancy, int *lag, int *slots)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (grid)
        *grid = h->last_plan.grid;
    if (occupancy)
        *occupancy = h->last_plan.occupancy;
    if (lag)
        *lag = h->last_plan.lag;
    if (slots)
        *slots = h->last_plan.slots;
    return MSOSM_OK;
}

extern "C" int msosm_get_dims(const msosm_t *h, int *M, int *M_min, int *fftpoint, int *batch, int *num_dms,
                              int *delaycount, int *ring_blocks)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (M)
        *M = h->M;
    if (M_min)
        *M_min = h->M_min;
    if (fftpoint)
        *fftpoint = h->F;
    if (batch)
        *batch = h->B;
    if (num_dms)
        *num_dms = h->D;
    if (delaycount)
        *delaycount = h->delaycount;
    if (ring_blocks)
        *ring_blocks = h->fbs;
    return MSOSM_OK;
}

extern "C" int msosm_get_nd(const msosm_t *h, int *nd_out)
{
    if (!h || !nd_out)
        return MSOSM_ERR_ARG;
    std::copy(h->nd.begin(), h->nd.end(), nd_out);
    return MSOSM_OK;
}

extern "C" int msosm_get_delaycounts(const msosm_t *h, int *dc_out)
{
    if (!h || !dc_out)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return MSOSM_ERR_STATE;
    std::copy(h->dc.begin(), h->dc.end(), dc_out);
    return MSOSM_OK;
}

extern "C" int msosm_get_delay_points(const msosm_t *h, int dm_index, int *out)
{
    if (!h || !out || dm_index < 0 || dm_index >= h->D)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return MSOSM_ERR_STATE;
    std::vector<uint16_t> tmp(h->F);
    cudaError_t e = cudaMemcpy(tmp.data(), h->d_delays + (size_t)dm_index * h->F, h->F * sizeof(uint16_t),
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return const_cast<msosm_t *>(h)->cuda_fail(e, "cudaMemcpy(delays)");
    for (int i = 0; i < h->F; i++)
        out[i] = tmp[i];
    return MSOSM_OK;
}

extern "C" int msosm_get_response(const msosm_t *h, int dm_index, float *out)
{
    if (!h || !out || dm_index < 0 || dm_index >= h->D)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return MSOSM_ERR_STATE;
    cudaError_t e =
        cudaMemcpy(out, h->d_H + (size_t)dm_index * h->F, (size_t)h->F * sizeof(float2), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return const_cast<msosm_t *>(h)->cuda_fail(e, "cudaMemcpy(H)");
    return MSOSM_OK;
}

static bool is_device_pointer(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static int process_one(msosm_t *h, const void *in, bool in_on_device, cudaStream_t st)
{
    const size_t in_bytes = (size_t)h->B * h->M * in_elem_bytes(h->in_format);
    const void *src = in;
    cudaError_t e;
    const int k = h->in_buf;
    if (!in_on_device)
    {
        // host input: copied on the handle's copy stream into the staging buffer that the
        // call two back has finished reading, so it overlaps the previous call's transforms
        void *buf = k ? h->d_in2 : h->d_in;
        h->in_buf ^= 1;
        if ((e = cudaStreamWaitEvent(h->copy_st, h->ev_consumed[k], 0)) != cudaSuccess ||
            (e = cudaMemcpyAsync(buf, in, in_bytes, cudaMemcpyDefault, h->copy_st)) != cudaSuccess ||
            (e = cudaEventRecord(h->ev_copied[k], h->copy_st)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(st, h->ev_copied[k], 0)) != cudaSuccess)
            return h->cuda_fail(e, "cudaMemcpyAsync(input)");
        src = buf;
    }
    const int rbi = (int)((h->step * h->B) % h->fbs);
    const float2 *tail = h->d_tail[h->tail_cur];
    float2 *tail_next = h->d_tail[h->tail_cur ^ 1];
    Profiler &pr = h->prof;
    pr.begin(MSOSM_KERNEL_FWD_PASS1, st);
    e = msosm::launch_forward_p1(h->g, h->tw_fwd, h->in_format, src, tail, tail_next, h->d_T, h->B, st);
    pr.end(MSOSM_KERNEL_FWD_PASS1, st, h->B);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "forward transform launch (pass 1)");
    if (!in_on_device && (e = cudaEventRecord(h->ev_consumed[k], st)) != cudaSuccess) // pass 1 read the input
        return h->cuda_fail(e, "cudaEventRecord(input)");
    pr.begin(MSOSM_KERNEL_FWD_PASS2, st);
    e = msosm::launch_forward_p2(h->g, h->tw_fwd, h->d_T, h->d_ring, rbi, h->B, st);
    pr.end(MSOSM_KERNEL_FWD_PASS2, st, h->B);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "forward transform launch (pass 2)");
    if (h->precision == msosm::PREC_FP16X3 &&
        (e = msosm::tc_absmax(h->d_ring + (size_t)rbi * h->F, (size_t)h->B * h->F, h->d_absmax, st)) != cudaSuccess)
        return h->cuda_fail(e, "spectra bound launch");

    // a step with nothing to produce (no series output, no fold) only advances the
    // stream: the tail and the ring of spectra, e.g. to skip the ring's warm-up
    if (h->out_mode == MSOSM_OUT_NONE && !h->fold && !h->pair_out)
    {
        h->tail_cur ^= 1;
        h->step++;
        return MSOSM_OK;
    }
    msosm::InvArgs a{};
    a.ring = h->d_ring;
    a.H = h->d_H;
    a.delays = h->d_delays;
    a.T = h->d_T;
    a.rbi = rbi;
    a.fbs = h->fbs;
    a.B = h->B;
    a.out_mode = 0;
    if (h->out_mode & MSOSM_OUT_C64)
        a.out_mode |= msosm::OUT_C64;
    if (h->out_mode & MSOSM_OUT_U16)
        a.out_mode |= msosm::OUT_U16;
    a.out_c64 = h->d_out_c64;
    a.out_u16 = h->d_out_u16;
    if (h->fold)
    {
        a.out_mode |= msosm::OUT_FOLD;
        a.fold = h->fold->args();
        a.fold.phase_dev = h->graph_phase;
        if (h->pair_in)
            a.out_mode |= msosm::OUT_PAIR;
    }
    if (h->pair_out)
        a.out_mode |= msosm::OUT_POW;
    const long long total = (long long)h->D * h->B;
    if (h->persist)
    {
        msosm::PersistArgs pa{};
        pa.ring = h->d_ring;
        pa.H = h->d_H;
        pa.delays = h->d_delays;
        pa.T = h->d_T;
        pa.rbi = rbi;
        pa.fbs = h->fbs;
        pa.B = h->B;
        pa.g0 = 0;
        pa.G = total;
        pa.tw = h->tw_inv;
        pa.out_mode = a.out_mode;
        pa.out_c64 = a.out_c64;
        pa.out_u16 = a.out_u16;
        pa.out_pow = h->pair_out;
        pa.pair_pow = h->pair_in;
        pa.fold = a.fold;
        pa.ticket = h->d_sync;
        pa.p1_done = h->d_sync + 1;
        pa.p2_done = h->d_sync + 1 + kMaxSlots;
        pa.err = h->d_err;
        pa.timeout_ns = kWaitTimeoutNs;
        pa.max_ctas_per_sm = h->ctas_per_sm;
        pa.D = h->D;
        // default order: window-major groups of 4 DM trials up to 2^18-point transforms
        // (512-DM, 2^18 workload: groups of 1 / 2 / 3 / 4 / 8 / 16 / 32 measured 9.42 / 9.59 /
        // 9.63 / 9.64 / 9.51 / 9.32 / 9.29e10), DM-major above (groups cost 2.5 % at 2^20)
        const int dm_group = h->dm_group > 0 ? h->dm_group : (h->g.L <= 18 ? 4 : 1);
        pa.dm_group = std::max(1, std::min(dm_group, h->D));
        msosm::TcArgs tc{static_cast<const uint4 *>(h->d_tc_op), h->d_absmax, h->hmax};
        const bool use_tc = h->precision != msosm::PREC_FP32;
        msosm::PersistPlan plan;
        e = use_tc ? msosm::tc_plan(h->g.L, h->precision, pa, tc, h->sms, &plan)
                   : msosm::persist_plan(h->g.L, pa, h->sms, &plan);
        if (e != cudaSuccess)
            return h->cuda_fail(e, "persistent transform plan");
        pa.lag = plan.lag;
        pa.S = std::min(plan.slots, h->T_slots);
        h->last_plan = plan;
        h->last_plan.slots = pa.S;
        if (pa.S <= pa.lag)
            return h->fail(MSOSM_ERR_UNSUPPORTED, "intermediate ring too small for the persistent transform");
        if ((e = cudaMemsetAsync(h->d_sync, 0, sizeof(unsigned) * (1 + 2 * kMaxSlots), st)) != cudaSuccess)
            return h->cuda_fail(e, "cudaMemsetAsync(sync)");
        pr.begin(MSOSM_KERNEL_INV_FUSED, st);
        e = use_tc ? msosm::launch_inverse_tc(h->g.L, h->precision, pa, tc, h->sms, st)
                   : msosm::launch_inverse_persistent(h->g.L, pa, h->sms, st);
        pr.end(MSOSM_KERNEL_INV_FUSED, st, total);
        if (e != cudaSuccess)
            return h->cuda_fail(e, "persistent inverse transform launch");
    }
    for (long long g0 = 0; !h->persist && g0 < total; g0 += h->T_cap)
    {
        const int count = (int)std::min<long long>(h->T_cap, total - g0);
        pr.begin(MSOSM_KERNEL_INV_PASS1, st);
        e = msosm::launch_inverse_p1(h->g, h->tw_inv, a, g0, count, st);
        pr.end(MSOSM_KERNEL_INV_PASS1, st, count);
        if (e != cudaSuccess)
            return h->cuda_fail(e, "inverse transform launch (pass 1)");
        pr.begin(MSOSM_KERNEL_INV_PASS2, st);
        e = msosm::launch_inverse_p2(h->g, h->tw_inv, a, g0, count, st);
        pr.end(MSOSM_KERNEL_INV_PASS2, st, count);
        if (e != cudaSuccess)
            return h->cuda_fail(e, "inverse transform launch (pass 2)");
    }
    if (h->fold && h->graph_phase &&
        (e = msosm::launch_phase_advance(h->graph_phase, (uint64_t)((uint64_t)h->B * (uint64_t)h->M) * a.fold.dphase,
                                         st)) != cudaSuccess)
        return h->cuda_fail(e, "fold phase advance");
    if (h->fold)
        h->fold->t_start += (double)((size_t)h->B * h->M) * h->fold->dt; // fold_gpu.cpp:53
    if (h->writer)
    {
        std::string werr;
        int rc = msosm::writer_submit_device(h->writer, h->d_out_u16, st, werr);
        if (rc != MSOSM_OK)
            return h->fail(rc, werr);
    }
    h->tail_cur ^= 1;
    h->step++;
    return MSOSM_OK;
}

extern "C" int msosm_attach_writer(msosm_t *h, msosm_writer_t *w)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (!w)
    {
        h->writer = nullptr;
        return MSOSM_OK;
    }
    if (!h->inited || !h->d_out_u16)
        return h->fail(MSOSM_ERR_STATE, "attach_writer needs an initialised handle with MSOSM_OUT_U16");
    if (msosm::writer_num_files(w) != h->D ||
        msosm::writer_bytes_per_step(w) != (size_t)h->D * h->B * h->M * sizeof(uint32_t))
        return h->fail(MSOSM_ERR_ARG, "writer must have one file per DM and B*M*4 bytes per DM per step");
    h->writer = w;
    return MSOSM_OK;
}

extern "C" int msosm_writer_copy_output(msosm_writer_t *w, msosm_t *h, void *stream)
{
    if (!h || !w)
        return MSOSM_ERR_ARG;
    if (!h->inited || !h->d_out_u16)
        return h->fail(MSOSM_ERR_STATE, "writer_copy_output needs an initialised handle with MSOSM_OUT_U16");
    if (msosm::writer_num_files(w) != h->D ||
        msosm::writer_bytes_per_step(w) != (size_t)h->D * h->B * h->M * sizeof(uint32_t))
        return h->fail(MSOSM_ERR_ARG, "writer must have one file per DM and B*M*4 bytes per DM per step");
    std::string werr;
    const int rc = msosm::writer_submit_device(w, h->d_out_u16, (cudaStream_t)stream, werr);
    return rc == MSOSM_OK ? rc : h->fail(rc, werr);
}

// ---- CUDA-graph capture of consecutive steps ------------------------------------
struct msosm_graph_s
{
    msosm_t *h = nullptr;
    int nsteps = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t *d_phase = nullptr; // the fold's phase, read and advanced by the graph's calls
    ~msosm_graph_s()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        dfree(d_phase);
    }
};

static long long gcd_ll(long long a, long long b) { return b ? gcd_ll(b, a % b) : a; }

extern "C" int msosm_graph_create(msosm_t *h, const void *in, int nsteps, msosm_graph_t **out)
{
    if (!h || !out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "graph_create before init");
    if (!h->persist)
        return h->fail(MSOSM_ERR_UNSUPPORTED, "graph capture needs the persistent transform (fftpoint >= 65536)");
    if (h->writer || h->prof.on)
        return h->fail(MSOSM_ERR_STATE, "graph capture with a writer attached or timing on");
    if (!in || !is_device_pointer(in) || ((uintptr_t)in % in_elem_bytes(h->in_format)) != 0)
        return h->fail(MSOSM_ERR_ARG, "graph input must be aligned device memory");
    // the ring slots and the tail buffer repeat with this period in steps: a graph of a
    // multiple of it continues the stream exactly on every launch
    const long long ring_period = h->fbs / h->B;
    const long long period = ring_period / gcd_ll(ring_period, 2) * 2;
    if (nsteps <= 0 || nsteps % period != 0)
        return h->fail(MSOSM_ERR_ARG, "nsteps must be a positive multiple of " + std::to_string(period) +
                                          " (the ring's period in steps)");
    msosm_graph_s *g = new (std::nothrow) msosm_graph_s();
    if (!g)
        return MSOSM_ERR_NOMEM;
    g->h = h;
    g->nsteps = nsteps;
    cudaError_t e;
    if (h->fold && (e = dalloc(&g->d_phase, 1)) != cudaSuccess)
    {
        delete g;
        return h->cuda_fail(e, "cudaMalloc(graph phase)");
    }
    cudaStream_t cs = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess)
    {
        delete g;
        return h->cuda_fail(e, "cudaStreamCreate(capture)");
    }
    // host-side state the captured calls advance; restored afterwards (capture runs nothing)
    const long long step0 = h->step;
    const int tail0 = h->tail_cur;
    const double t0 = h->fold ? h->fold->t_start : 0.0;
    h->graph_phase = g->d_phase;
    cudaGraph_t graph = nullptr;
    int rc = MSOSM_OK;
    const size_t step_bytes = (size_t)h->B * h->M * in_elem_bytes(h->in_format);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess)
        rc = h->cuda_fail(e, "cudaStreamBeginCapture");
    for (int s = 0; rc == MSOSM_OK && s < nsteps; s++)
        rc = process_one(h, (const char *)in + (size_t)s * step_bytes, true, cs);
    if (e == cudaSuccess)
    {
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (rc == MSOSM_OK && e2 != cudaSuccess)
            rc = h->cuda_fail(e2, "cudaStreamEndCapture");
    }
    if (rc == MSOSM_OK && (e = cudaGraphInstantiate(&g->exec, graph, 0)) != cudaSuccess)
        rc = h->cuda_fail(e, "cudaGraphInstantiate");
    if (graph)
        cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    h->graph_phase = nullptr;
    h->step = step0;
    h->tail_cur = tail0;
    if (h->fold)
        h->fold->t_start = t0;
    if (rc != MSOSM_OK)
    {
        delete g;
        return rc;
    }
    *out = g;
    return MSOSM_OK;
}

extern "C" int msosm_graph_launch(msosm_graph_t *g, void *stream)
{
    if (!g || !g->h)
        return MSOSM_ERR_ARG;
    msosm_t *h = g->h;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if (h->fold)
    {
        // the phase of this launch's first sample, as msosm_process would pass it
        const msosm::FoldArgs fa = h->fold->args();
        if ((e = msosm::launch_phase_set(g->d_phase, fa.phase0, st)) != cudaSuccess)
            return h->cuda_fail(e, "fold phase set");
    }
    if ((e = cudaGraphLaunch(g->exec, st)) != cudaSuccess)
        return h->cuda_fail(e, "cudaGraphLaunch");
    h->step += g->nsteps;
    h->tail_cur ^= (g->nsteps & 1);
    if (h->fold)
        h->fold->t_start += (double)g->nsteps * (double)((size_t)h->B * h->M) * h->fold->dt;
    return MSOSM_OK;
}

extern "C" int msosm_graph_destroy(msosm_graph_t *g)
{
    if (!g)
        return MSOSM_ERR_ARG;
    delete g;
    return MSOSM_OK;
}

extern "C" int msosm_process(msosm_t *h, const void *in, void *stream)
{
    return msosm_process_many(h, in, 1, stream);
}

extern "C" int msosm_process_many(msosm_t *h, const void *in, int nsteps, void *stream)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "msosm_process before msosm_init");
    if (!in || nsteps < 0)
        return h->fail(MSOSM_ERR_ARG, "null input");
    cudaStream_t st = (cudaStream_t)stream;
    // device input is read in place only when aligned to its element size (the
    // kernels use 8/4/2-byte vector loads); anything else goes through staging
    const bool dev = is_device_pointer(in) && ((uintptr_t)in % in_elem_bytes(h->in_format)) == 0;
    const size_t step_bytes = (size_t)h->B * h->M * in_elem_bytes(h->in_format);
    for (int s = 0; s < nsteps; s++)
    {
        int rc = process_one(h, (const char *)in + (size_t)s * step_bytes, dev, st);
        if (rc != MSOSM_OK)
            return rc;
    }
    return MSOSM_OK;
}

extern "C" int msosm_get_output(msosm_t *h, void *out, void *stream)
{
    if (!h || !out)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "get_output before init");
    const size_t n = (size_t)h->D * h->B * h->M;
    cudaError_t e;
    if (h->d_out_c64)
        e = cudaMemcpyAsync(out, h->d_out_c64, n * sizeof(float2), cudaMemcpyDefault, (cudaStream_t)stream);
    else if (h->d_out_u16)
        e = cudaMemcpyAsync(out, h->d_out_u16, n * sizeof(uint32_t), cudaMemcpyDefault, (cudaStream_t)stream);
    else
        return h->fail(MSOSM_ERR_STATE, "no series output configured");
    if (e != cudaSuccess)
        return h->cuda_fail(e, "cudaMemcpyAsync(output)");
    return MSOSM_OK;
}

extern "C" void *msosm_device_output(msosm_t *h) { return h ? (void *)h->d_out_c64 : nullptr; }
extern "C" void *msosm_device_output_u16(msosm_t *h) { return h ? (void *)h->d_out_u16 : nullptr; }
extern "C" long long msosm_steps(const msosm_t *h) { return h ? h->step : -1; }

extern "C" int msosm_sync(msosm_t *h, void *stream)
{
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return h ? h->cuda_fail(e, "cudaStreamSynchronize") : MSOSM_ERR_CUDA;
    if (h && h->d_err)
    {
        int err = 0;
        e = cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            return h->cuda_fail(e, "cudaMemcpy(err)");
        if (err)
            return h->fail(MSOSM_ERR_CUDA, "a device-side wait of the persistent transform timed out; outputs of "
                                           "this handle are invalid");
    }
    return MSOSM_OK;
}

extern "C" int msosm_destroy(msosm_t *h)
{
    if (!h)
        return MSOSM_ERR_ARG;
    delete h;
    return MSOSM_OK;
}

extern "C" const char *msosm_last_error(const msosm_t *h) { return h ? h->err.c_str() : "null handle"; }

extern "C" int msosm_profile_enable(msosm_t *h, int on)
{
    if (!h)
        return MSOSM_ERR_ARG;
    h->prof.on = on != 0;
    return MSOSM_OK;
}

extern "C" int msosm_profile_reset(msosm_t *h)
{
    if (!h)
        return MSOSM_ERR_ARG;
    h->prof.reset();
    return MSOSM_OK;
}

extern "C" int msosm_profile_read(msosm_t *h, int kind, double *ms_total, long long *launches, long long *timed,
                                  long long *transforms)
{
    if (!h || kind < 0 || kind >= Profiler::KINDS)
        return MSOSM_ERR_ARG;
    cudaError_t e = h->prof.collect();
    if (e != cudaSuccess)
        return h->cuda_fail(e, "cudaEventElapsedTime (kernel timing; sync the stream first)");
    if (ms_total)
        *ms_total = h->prof.ms[kind];
    if (launches)
        *launches = h->prof.launches[kind];
    if (timed)
        *timed = h->prof.timed[kind];
    if (transforms)
        *transforms = h->prof.transforms[kind];
    return MSOSM_OK;
}

// ---- FFT-size autotuning ---------------------------------------------------------
extern "C" int msosm_selftest_umma(int bf16, int n, int b_row0, const uint16_t *A, const uint16_t *B, float *D,
                                   int *timed_out)
{
    if (!A || !B || !D || !timed_out || (n != 32 && n != 64) || b_row0 < 0 || b_row0 + n > 64 || b_row0 % 8)
        return MSOSM_ERR_ARG;
    cudaError_t e = msosm::tc_selftest_umma(bf16, n, b_row0, A, B, D, timed_out);
    return e == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
}

extern "C" int msosm_selftest_wait(unsigned preset, unsigned target, unsigned long long timeout_ns, int *timed_out,
                                   unsigned long long *elapsed_ns)
{
    if (!timed_out || !elapsed_ns || timeout_ns == 0 || timeout_ns > kWaitTimeoutNs)
        return MSOSM_ERR_ARG;
    const cudaError_t e = msosm::persist_selftest_wait(preset, target, timeout_ns, timed_out, elapsed_ns);
    return e == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
}

extern "C" int msosm_autotune(float bw, float f0, const float *dms, int num_dms, int batch, int in_format,
                              int min_fftpoint, int max_fftpoint, int steps, int *best_fftpoint, double *best_rate)
{
    if (!dms || num_dms <= 0 || batch <= 0 || steps <= 0 || !best_fftpoint || in_elem_bytes(in_format) == 0)
        return MSOSM_ERR_ARG;
    // DM subset: up to 16 spread over the list, the largest always included
    std::vector<float> sub;
    const int nsub = std::min(num_dms, 16);
    for (int i = 0; i < nsub; i++)
        sub.push_back(dms[(long long)i * (num_dms - 1) / std::max(1, nsub - 1)]);
    sub.back() = dms[num_dms - 1];
    std::sort(sub.begin(), sub.end());
    int mmin = 0;
    for (float d : sub)
        mmin = std::max(mmin, msosm::plan_min_order(msosm::plan_nd(bw, d, f0)));
    const long long lo = std::max<long long>(std::max(min_fftpoint, 1 << kMinLog2F), 2ll * mmin);
    const long long hi = std::min<long long>(max_fftpoint, 1ll << kMaxLog2F);
    int best = 0;
    double best_r = 0.0;
    for (long long F = 1; F <= hi; F <<= 1)
    {
        if (F < lo)
            continue;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        // ring (>= delaycount + batch slots), responses, delays, intermediate, input
        const int dc = msosm::plan_delaycount(msosm::plan_nd(bw, sub.back(), f0), (int)(F / 2));
        const double need = (double)F * 8 * (dc + 2 * batch + 64) + (double)sub.size() * F * 10 +
                            (double)batch * F / 2 * in_elem_bytes(in_format) * 2;
        if (need > 0.8 * (double)free_b)
            continue;
        msosm_t *h = nullptr;
        if (msosm_create(bw, f0, sub.data(), (int)sub.size(), &h) != MSOSM_OK)
            continue;
        int rc = msosm_init(h, (int)F, batch, in_format, MSOSM_OUT_NONE);
        msosm_fold_t *f = nullptr;
        if (rc == MSOSM_OK)
            rc = msosm_fold_create(1.0f, bw, (unsigned long)batch * (F / 2), 64, (int)sub.size(), &f);
        if (rc == MSOSM_OK)
            rc = msosm_attach_fold(h, f);
        void *in = nullptr;
        const size_t in_bytes = (size_t)batch * (F / 2) * in_elem_bytes(in_format);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (rc == MSOSM_OK && cudaMalloc(&in, in_bytes) == cudaSuccess && cudaMemset(in, 0, in_bytes) == cudaSuccess &&
            cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess)
        {
            rc = msosm_process(h, in, nullptr); // warm-up
            cudaEventRecord(e0, nullptr);
            for (int s = 0; rc == MSOSM_OK && s < steps; s++)
                rc = msosm_process(h, in, nullptr);
            cudaEventRecord(e1, nullptr);
            if (rc == MSOSM_OK)
                rc = msosm_sync(h, nullptr);
            float ms = 0.f;
            if (rc == MSOSM_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f)
            {
                const double rate = (double)steps * batch * (F / 2) * sub.size() / (ms * 1e-3);
                if (rate > best_r)
                {
                    best_r = rate;
                    best = (int)F;
                }
            }
        }
        cudaGetLastError();
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
        if (in)
            cudaFree(in);
        msosm_destroy(h);
        if (f)
            msosm_fold_destroy(f);
    }
    if (!best)
        return MSOSM_ERR_UNSUPPORTED;
    *best_fftpoint = best;
    if (best_rate)
        *best_rate = best_r;
    return MSOSM_OK;
}

extern "C" int msosm_autotune_shape(float bw, float f0, const float *dms, int num_dms, int in_format,
                                    int min_fftpoint, int max_fftpoint, const int *batches, int num_batches,
                                    int steps, int *best_fftpoint, int *best_batch, int *best_ctas_per_sm,
                                    double *best_rate)
{
    if (!dms || num_dms <= 0 || !batches || num_batches <= 0 || steps <= 0 || !best_fftpoint || !best_batch ||
        !best_ctas_per_sm || in_elem_bytes(in_format) == 0)
        return MSOSM_ERR_ARG;
    std::vector<float> sub;
    const int nsub = std::min(num_dms, 16);
    for (int i = 0; i < nsub; i++)
        sub.push_back(dms[(long long)i * (num_dms - 1) / std::max(1, nsub - 1)]);
    sub.back() = dms[num_dms - 1];
    std::sort(sub.begin(), sub.end());
    int mmin = 0;
    for (float d : sub)
        mmin = std::max(mmin, msosm::plan_min_order(msosm::plan_nd(bw, d, f0)));
    const long long lo = std::max<long long>(std::max(min_fftpoint, 1 << kMinLog2F), 2ll * mmin);
    const long long hi = std::min<long long>(max_fftpoint, 1ll << kMaxLog2F);
    double best_r = 0.0;
    *best_fftpoint = *best_batch = *best_ctas_per_sm = 0;
    for (long long F = 1; F <= hi; F <<= 1)
    {
        if (F < lo)
            continue;
        for (int bi = 0; bi < num_batches; bi++)
        {
            const int batch = batches[bi];
            if (batch <= 0)
                continue;
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            const int dc = msosm::plan_delaycount(msosm::plan_nd(bw, sub.back(), f0), (int)(F / 2));
            const double need = (double)F * 8 * (dc + 2 * batch + 64) + (double)sub.size() * F * 10 +
                                (double)batch * F / 2 * in_elem_bytes(in_format) * 2;
            if (need > 0.8 * (double)free_b)
                continue;
            // launch shapes: as many CTAs per SM as fit, then one (persistent sizes only)
            for (int ctas : {0, 1})
            {
                if (ctas == 1 && F < (1 << 16))
                    continue;
                msosm_t *h = nullptr;
                if (msosm_create(bw, f0, sub.data(), (int)sub.size(), &h) != MSOSM_OK)
                    continue;
                int rc = msosm_init(h, (int)F, batch, in_format, MSOSM_OUT_NONE);
                if (rc == MSOSM_OK)
                    rc = msosm_set_launch_shape(h, ctas, 0);
                msosm_fold_t *f = nullptr;
                if (rc == MSOSM_OK)
                    rc = msosm_fold_create(1.0f, bw, (unsigned long)batch * (F / 2), 64, (int)sub.size(), &f);
                if (rc == MSOSM_OK)
                    rc = msosm_attach_fold(h, f);
                void *in = nullptr;
                const size_t in_bytes = (size_t)batch * (F / 2) * in_elem_bytes(in_format);
                cudaEvent_t e0 = nullptr, e1 = nullptr;
                if (rc == MSOSM_OK && cudaMalloc(&in, in_bytes) == cudaSuccess &&
                    cudaMemset(in, 0, in_bytes) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
                    cudaEventCreate(&e1) == cudaSuccess)
                {
                    rc = msosm_process(h, in, nullptr); // warm-up
                    cudaEventRecord(e0, nullptr);
                    for (int s = 0; rc == MSOSM_OK && s < steps; s++)
                        rc = msosm_process(h, in, nullptr);
                    cudaEventRecord(e1, nullptr);
                    if (rc == MSOSM_OK)
                        rc = msosm_sync(h, nullptr);
                    float ms = 0.f;
                    if (rc == MSOSM_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f)
                    {
                        const double rate = (double)steps * batch * (F / 2) * sub.size() / (ms * 1e-3);
                        if (rate > best_r)
                        {
                            best_r = rate;
                            *best_fftpoint = (int)F;
                            *best_batch = batch;
                            *best_ctas_per_sm = ctas;
                        }
                    }
                }
                cudaGetLastError();
                if (e0)
                    cudaEventDestroy(e0);
                if (e1)
                    cudaEventDestroy(e1);
                if (in)
                    cudaFree(in);
                msosm_destroy(h);
                if (f)
                    msosm_fold_destroy(f);
            }
        }
    }
    if (best_rate)
        *best_rate = best_r;
    return *best_fftpoint ? MSOSM_OK : MSOSM_ERR_UNSUPPORTED;
}

// ---- DM derivative ------------------------------------------------------------------
extern "C" int msosm_plan_response_derivative(float bw, float f0, float dm, int M, float *H_out)
{
    if (M <= 0 || !is_pow2(M) || !H_out)
        return MSOSM_ERR_ARG;
    msosm::plan_responses(bw, f0, &dm, 1, M, H_out, 1, true);
    return MSOSM_OK;
}

extern "C" int msosm_set_response(msosm_t *h, int dm_index, const float *H)
{
    if (!h || !H)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "set_response before init");
    if (dm_index < 0 || dm_index >= h->D)
        return h->fail(MSOSM_ERR_ARG, "dm_index out of range");
    const bool dev = is_device_pointer(H);
    std::vector<float> host(2 * (size_t)h->F);
    cudaError_t e = cudaMemcpy(host.data(), H, host.size() * sizeof(float), dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "cudaMemcpy(H)");
    // the FP16 operand scaling needs a bound on |H| over every row
    h->hmax = std::max(h->hmax, max_abs_complex(host));
    e = cudaMemcpy(h->d_H + (size_t)dm_index * h->F, host.data(), (size_t)h->F * sizeof(float2), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? MSOSM_OK : h->cuda_fail(e, "cudaMemcpy(H)");
}

extern "C" int msosm_use_response_derivative(msosm_t *h)
{
    if (!h)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "use_response_derivative before init");
    const size_t DF = (size_t)h->D * h->F;
    std::vector<float> H(2 * DF);
    const int threads = (int)std::max(1u, std::thread::hardware_concurrency());
    msosm::plan_responses(h->bw, h->f0, h->dms.data(), h->D, h->M, H.data(), threads, true);
    h->hmax = max_abs_complex(H);
    cudaError_t e = cudaMemcpy(h->d_H, H.data(), DF * sizeof(float2), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? MSOSM_OK : h->cuda_fail(e, "cudaMemcpy(dH)");
}

extern "C" int msosm_fold_accumulate_cross(msosm_fold_t *f, const void *x, const void *dx, void *stream)
{
    if (!f || !x || !dx)
        return MSOSM_ERR_ARG;
    cudaError_t e = msosm::launch_fold((const float2 *)x, (const float2 *)dx, f->size, f->S, f->args(),
                                       (cudaStream_t)stream, msosm::FOLD_CROSS);
    if (e != cudaSuccess)
    {
        f->err = std::string("fold launch: ") + cudaGetErrorString(e);
        return MSOSM_ERR_CUDA;
    }
    f->t_start += (double)f->size * f->dt;
    return MSOSM_OK;
}

// ---- checkpoint / resume --------------------------------------------------------
namespace {
struct StreamStateHeader
{
    uint32_t magic; // 'MSST'
    uint32_t version;
    int32_t M, F, B, fbs, in_format, tail_cur;
    int64_t step;
};
constexpr uint32_t kStateMagic = 0x5453534Du;
struct FoldStateHeader
{
    uint32_t magic; // 'MSFS'
    uint32_t version;
    uint64_t K, size;
    int32_t S, pad;
    double t_start, P, dt;
};
constexpr uint32_t kFoldMagic = 0x5346534Du;
} // namespace

extern "C" size_t msosm_state_bytes(const msosm_t *h)
{
    if (!h || !h->inited)
        return 0;
    return sizeof(StreamStateHeader) + ((size_t)h->M + (size_t)h->fbs * h->F) * sizeof(float2);
}

extern "C" int msosm_save_state(msosm_t *h, void *buf, size_t bytes, void *stream)
{
    if (!h || !buf)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "save_state before init");
    if (bytes < msosm_state_bytes(h))
        return h->fail(MSOSM_ERR_ARG, "state buffer too small");
    cudaStream_t st = (cudaStream_t)stream;
    StreamStateHeader hd{kStateMagic, 1, h->M, h->F, h->B, h->fbs, h->in_format, h->tail_cur, h->step};
    char *p = static_cast<char *>(buf);
    cudaError_t e = cudaMemcpyAsync(p, &hd, sizeof(hd), cudaMemcpyDefault, st);
    p += sizeof(hd);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p, h->d_tail[h->tail_cur], (size_t)h->M * sizeof(float2), cudaMemcpyDefault, st);
    p += (size_t)h->M * sizeof(float2);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p, h->d_ring, (size_t)h->fbs * h->F * sizeof(float2), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? MSOSM_OK : h->cuda_fail(e, "save_state");
}

extern "C" int msosm_load_state(msosm_t *h, const void *buf, size_t bytes, void *stream)
{
    if (!h || !buf)
        return MSOSM_ERR_ARG;
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "load_state before init");
    if (bytes < msosm_state_bytes(h))
        return h->fail(MSOSM_ERR_ARG, "state buffer too small");
    cudaStream_t st = (cudaStream_t)stream;
    StreamStateHeader hd{};
    cudaError_t e = cudaMemcpyAsync(&hd, buf, sizeof(hd), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "load_state");
    if (hd.magic != kStateMagic || hd.version != 1)
        return h->fail(MSOSM_ERR_ARG, "not a stream state");
    if (hd.M != h->M || hd.F != h->F || hd.B != h->B || hd.fbs != h->fbs)
        return h->fail(MSOSM_ERR_ARG, "state was saved with a different M, batch or ring size");
    const char *p = static_cast<const char *>(buf) + sizeof(hd);
    // the saved tail becomes the current tail buffer
    e = cudaMemcpyAsync(h->d_tail[h->tail_cur], p, (size_t)h->M * sizeof(float2), cudaMemcpyDefault, st);
    p += (size_t)h->M * sizeof(float2);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_ring, p, (size_t)h->fbs * h->F * sizeof(float2), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return h->cuda_fail(e, "load_state");
    h->step = hd.step;
    if (h->precision == msosm::PREC_FP16X3)
    {
        // the operand-scale bound must cover the loaded ring
        if ((e = cudaMemsetAsync(h->d_absmax, 0, sizeof(unsigned), st)) != cudaSuccess ||
            (e = msosm::tc_absmax(h->d_ring, (size_t)h->fbs * h->F, h->d_absmax, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return h->cuda_fail(e, "load_state (spectra bound)");
    }
    return MSOSM_OK;
}

extern "C" size_t msosm_fold_state_bytes(const msosm_fold_t *f)
{
    if (!f)
        return 0;
    return sizeof(FoldStateHeader) + (size_t)f->K * f->S * (sizeof(double) + sizeof(unsigned long long));
}

extern "C" int msosm_fold_save_state(msosm_fold_t *f, void *buf, size_t bytes, void *stream)
{
    if (!f || !buf || bytes < msosm_fold_state_bytes(f))
        return MSOSM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)f->K * f->S;
    FoldStateHeader hd{kFoldMagic, 1, f->K, f->size, f->S, 0, f->t_start, f->P, f->dt};
    char *p = static_cast<char *>(buf);
    cudaError_t e = cudaMemcpyAsync(p, &hd, sizeof(hd), cudaMemcpyDefault, st);
    p += sizeof(hd);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p, f->d_sum, n * sizeof(double), cudaMemcpyDefault, st);
    p += n * sizeof(double);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p, f->d_cnt, n * sizeof(unsigned long long), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
}

extern "C" int msosm_fold_load_state(msosm_fold_t *f, const void *buf, size_t bytes, void *stream)
{
    if (!f || !buf || bytes < msosm_fold_state_bytes(f))
        return MSOSM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    FoldStateHeader hd{};
    cudaError_t e = cudaMemcpyAsync(&hd, buf, sizeof(hd), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return MSOSM_ERR_CUDA;
    if (hd.magic != kFoldMagic || hd.version != 1 || hd.K != f->K || hd.S != f->S || hd.size != f->size ||
        hd.P != f->P || hd.dt != f->dt)
        return MSOSM_ERR_ARG;
    const size_t n = (size_t)f->K * f->S;
    const char *p = static_cast<const char *>(buf) + sizeof(hd);
    e = cudaMemcpyAsync(f->d_sum, p, n * sizeof(double), cudaMemcpyDefault, st);
    p += n * sizeof(double);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(f->d_cnt, p, n * sizeof(unsigned long long), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return MSOSM_ERR_CUDA;
    f->t_start = hd.t_start;
    return MSOSM_OK;
}

// ---- folding ------------------------------------------------------------------
extern "C" int msosm_fold_create(float period, float fs, unsigned long size, unsigned long time_bin, int num_series,
                                 msosm_fold_t **out)
{
    if (!out)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    if (!(period > 0) || !(fs > 0) || num_series <= 0)
        return MSOSM_ERR_ARG;
    msosm_fold_t *f = new (std::nothrow) msosm_fold_s();
    if (!f)
        return MSOSM_ERR_NOMEM;
    f->period = period;
    f->fs = fs;
    f->P = (double)period;      // period_seconds (fold_gpu.cpp:9)
    f->dt = 1.0 / (double)fs;   // fold_data_phase (fold_gpu.cpp:50)
    f->size = size;
    // period_samples = (unsigned long)(float)(period*fs) (fold_gpu.cpp:10-16)
    const float psf = period * fs;
    f->K = time_bin ? time_bin : (unsigned long)psf;
    f->S = num_series;
    // the fold kernels reduce runs of 16 consecutive samples (see fold_accumulate)
    if (f->K == 0 || f->K > (1ul << 30) || (double)period * (double)fs <= 16.0)
    {
        delete f;
        return MSOSM_ERR_ARG;
    }
    const size_t n = (size_t)f->K * num_series;
    if (dalloc(&f->d_sum, n) != cudaSuccess || dalloc(&f->d_cnt, n) != cudaSuccess ||
        dalloc(&f->d_folded, n) != cudaSuccess)
    {
        cudaGetLastError();
        delete f;
        return MSOSM_ERR_NOMEM;
    }
    if (cudaMemset(f->d_sum, 0, n * sizeof(double)) != cudaSuccess ||
        cudaMemset(f->d_cnt, 0, n * sizeof(unsigned long long)) != cudaSuccess)
    {
        delete f;
        return MSOSM_ERR_CUDA;
    }
    *out = f;
    return MSOSM_OK;
}

extern "C" int msosm_fold_accumulate(msosm_fold_t *f, const void *pol1, const void *pol2, void *stream)
{
    if (!f || !pol1)
        return MSOSM_ERR_ARG;
    cudaError_t e = msosm::launch_fold((const float2 *)pol1, (const float2 *)pol2, f->size, f->S, f->args(),
                                       (cudaStream_t)stream);
    if (e != cudaSuccess)
    {
        f->err = std::string("fold launch: ") + cudaGetErrorString(e);
        return MSOSM_ERR_CUDA;
    }
    f->t_start += (double)f->size * f->dt; // fold_gpu.cpp:53
    return MSOSM_OK;
}

extern "C" int msosm_fold_read(msosm_fold_t *f, float *folded, double *sums, unsigned long long *counts,
                               void *stream)
{
    if (!f)
        return MSOSM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)f->K * f->S;
    cudaError_t e = cudaSuccess;
    if (folded)
    {
        e = msosm::launch_fold_finalize(f->d_sum, f->d_cnt, f->d_folded, n, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(folded, f->d_folded, n * sizeof(float), cudaMemcpyDefault, st);
    }
    if (e == cudaSuccess && sums)
        e = cudaMemcpyAsync(sums, f->d_sum, n * sizeof(double), cudaMemcpyDefault, st);
    if (e == cudaSuccess && counts)
        e = cudaMemcpyAsync(counts, f->d_cnt, n * sizeof(unsigned long long), cudaMemcpyDefault, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        f->err = std::string("fold read: ") + cudaGetErrorString(e);
        return MSOSM_ERR_CUDA;
    }
    return MSOSM_OK;
}

extern "C" int msosm_fold_reset(msosm_fold_t *f, void *stream)
{
    if (!f)
        return MSOSM_ERR_ARG;
    const size_t n = (size_t)f->K * f->S;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(f->d_sum, 0, n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(f->d_cnt, 0, n * sizeof(unsigned long long), st) != cudaSuccess)
        return MSOSM_ERR_CUDA;
    f->t_start = 0.0;
    return MSOSM_OK;
}

extern "C" int msosm_fold_dims(const msosm_fold_t *f, unsigned long *time_bin, int *num_series, unsigned long *size)
{
    if (!f)
        return MSOSM_ERR_ARG;
    if (time_bin)
        *time_bin = f->K;
    if (num_series)
        *num_series = f->S;
    if (size)
        *size = f->size;
    return MSOSM_OK;
}

extern "C" int msosm_fold_destroy(msosm_fold_t *f)
{
    if (!f)
        return MSOSM_ERR_ARG;
    delete f;
    return MSOSM_OK;
}

extern "C" int msosm_attach_fold(msosm_t *h, msosm_fold_t *f)
{
    if (!h)
        return MSOSM_ERR_ARG;
    h->pair_in = nullptr;
    h->pair_out = nullptr;
    if (!f)
    {
        h->fold = nullptr;
        return MSOSM_OK;
    }
    if (!h->inited)
        return h->fail(MSOSM_ERR_STATE, "attach_fold before init");
    if (f->S != h->D || f->size != (unsigned long)h->B * h->M)
        return h->fail(MSOSM_ERR_ARG, "fold must have num_series == num_dms and size == B*M");
    if (f->K > kMaxFusedBins)
        return h->fail(MSOSM_ERR_UNSUPPORTED, "fused fold supports at most 8192 bins");
    // The fused epilogue reduces each half-warp's 16 samples when their first and
    // last bins agree, which needs those samples to span less than one period.
    // A half-warp covers 16 consecutive time samples, or 16/cols runs of cols
    // samples N2 apart when a tile holds fewer than 16 rows.
    const int n1 = h->g.N1, n2 = h->g.N2;
    const int cols = h->persist ? 8192 / n1 : (n1 <= 512 ? 16 : (n1 == 1024 ? 8 : 4));
    const double span = cols >= 16 ? 16.0 : (double)(16 / cols - 1) * n2 + cols;
    if ((double)f->P / f->dt <= span)
        return h->fail(MSOSM_ERR_UNSUPPORTED, "fold period shorter than the fused epilogue's sample span");
    h->fold = f;
    return MSOSM_OK;
}

extern "C" int msosm_attach_fold_pol2(msosm_t *first, msosm_t *second, msosm_fold_t *f)
{
    if (!first || !second || first == second)
        return MSOSM_ERR_ARG;
    if (!f)
    {
        msosm_attach_fold(first, nullptr);
        return msosm_attach_fold(second, nullptr);
    }
    if (!first->inited || !second->inited)
        return second->fail(MSOSM_ERR_STATE, "attach_fold_pol2 before init");
    if (first->D != second->D || first->B != second->B || first->M != second->M || first->dms != second->dms)
        return second->fail(MSOSM_ERR_ARG, "attach_fold_pol2: both polarisations need the same DMs, batch and size");
    if (!first->persist || !second->persist)
        return second->fail(MSOSM_ERR_UNSUPPORTED, "the fused 2-pol fold needs fftpoint >= 65536");
    if (first->out_mode != MSOSM_OUT_NONE || second->out_mode != MSOSM_OUT_NONE)
        return second->fail(MSOSM_ERR_UNSUPPORTED, "the fused 2-pol fold needs both handles in MSOSM_OUT_NONE");
    int rc = msosm_attach_fold(second, f); // the fold checks (sizes, bins, period span)
    if (rc != MSOSM_OK)
        return rc;
    const size_t n = (size_t)second->D * second->B * second->M;
    if (!f->d_pair)
    {
        cudaError_t e = dalloc(&f->d_pair, n);
        if (e != cudaSuccess)
        {
            msosm_attach_fold(second, nullptr);
            return second->cuda_fail(e, "cudaMalloc(2-pol power)");
        }
    }
    msosm_attach_fold(first, nullptr);
    first->pair_out = f->d_pair;
    second->pair_in = f->d_pair;
    return MSOSM_OK;
}
