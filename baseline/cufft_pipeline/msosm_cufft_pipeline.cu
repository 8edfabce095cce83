// GPU baseline, not part of the engine: the reference's own MS-OSM GPU design restated on
// cuFFT, so that the engine can be timed against that design on the same GB300.
//
// Per call of B windows (dedispersion/msosm/msosm_gpu_batch.cpp:178-236, fold mode):
//   1. the B*M new samples follow the previous call's last M samples in one window buffer
//      (increment_fft_input, msosm_gpu_batch.cpp:153-165);
//   2. one batched cuFFT forward transform of B overlapping windows (idist = M) into B slots
//      of the spectra ring (msosm_gpu_batch.cpp:100-107, 191);
//   3. per DM chunk: the delayed-bin gather x response (gatherMultiply_kernel,
//      gpu/gpu_kernel.cu:105-210), one batched cuFFT inverse transform of chunk*B windows
//      (msosm_gpu_batch.cpp:196-199), and the overlap discard x 1/F (discardSamples_kernel,
//      gpu/gpu_kernel.cu:346-376) fused here with |x|^2 and the phase fold
//      (calculateIntensity / foldDataPhase_kernel, gpu/gpu_kernel.cu:430-496).
// Differences from the reference, each in the baseline's favour or forced: 64-bit indexing
// and DM chunks instead of one D*B*F buffer (the reference overflows int32 there); the
// inverse runs in place; discard and fold are one kernel; the fold phase is the engine's
// Q0.64 fixed-point phase instead of per-sample FP64 fmod (GB300's FP64 rate would
// otherwise bound this baseline); DM trials are folded together, not one series.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <new>

namespace {

struct Pipe
{
    int L = 0, F = 0, M = 0, B = 0, D = 0, fbs = 0, chunk = 0, K = 0;
    cufftHandle fwd = 0, inv = 0;
    bool fwd_ok = false, inv_ok = false;
    float2 *win = nullptr;  // (B+1)*M: previous tail, then the new samples
    float2 *ring = nullptr; // fbs*F spectra
    float2 *buf = nullptr;  // chunk*B*F inverse-transform buffer
    const float2 *H = nullptr;
    const uint16_t *delays = nullptr;
    double *sum = nullptr;
    unsigned long long *cnt = nullptr;
    int rbi = 0;
    double P = 0, dt = 0, t_start = 0;
    ~Pipe()
    {
        if (fwd_ok)
            cufftDestroy(fwd);
        if (inv_ok)
            cufftDestroy(inv);
        cudaFree(win);
        cudaFree(ring);
        cudaFree(buf);
        cudaFree(sum);
        cudaFree(cnt);
    }
};

uint64_t turns_q64(long double turns)
{
    long double f = turns - floorl(turns);
    long double v = ldexpl(f, 64);
    if (!(v < 18446744073709551616.0L) || v < 0)
        return 0;
    return (uint64_t)v;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// buf[(dl*B + b)*F + n] = ring[((rbi + b - delay[d][n]) mod fbs)*F + n] * H[d][n], d = d0 + dl
__global__ void gather_multiply(const float2 *__restrict__ ring, const float2 *__restrict__ H,
                                const uint16_t *__restrict__ delays, float2 *__restrict__ buf, int d0, int nd,
                                int B, int L, int fbs, int rbi)
{
    const int F = 1 << L;
    const size_t total = (size_t)nd * B * F;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const int n = (int)(i & (size_t)(F - 1));
        const unsigned w = (unsigned)(i >> L);
        const int b = (int)(w % (unsigned)B), dl = (int)(w / (unsigned)B);
        const size_t t = (size_t)(d0 + dl) * F + n;
        int s = rbi + b - (int)delays[t];
        if (s < 0)
            s += fbs;
        buf[i] = cmul(ring[(size_t)s * F + n], H[t]);
    }
}

// Samples M..2M-1 of each inverse transform, x 1/F, |x|^2 folded into D x K bins.
// One block per (window, 4096-sample tile); runs of 16 samples aggregate in shared memory.
__global__ void discard_fold(const float2 *__restrict__ buf, int d0, int B, int F, int M, uint64_t phase0,
                             uint64_t dphase, unsigned K, double *__restrict__ sum, unsigned long long *__restrict__ cnt)
{
    extern __shared__ float s_bins[]; // K sums, then K counts
    unsigned *s_cnt = reinterpret_cast<unsigned *>(s_bins + K);
    for (unsigned i = threadIdx.x; i < 2 * K; i += blockDim.x)
        s_bins[i] = 0.0f;
    __syncthreads();
    const int w = blockIdx.y; // dl*B + b
    const int b = w % B, dl = w / B;
    const float scale = 1.0f / (float)F;
    const float2 *src = buf + (size_t)w * F + M;
    const int base = blockIdx.x * 4096 + threadIdx.x * 16; // 256 threads x 16 samples
    if (base < M)
    {
        const uint64_t ph0 = phase0 + (uint64_t)((uint64_t)b * (uint64_t)M + (uint64_t)base) * dphase;
        const unsigned bf = (unsigned)__umul64hi(ph0, (unsigned long long)K);
        const unsigned bl = (unsigned)__umul64hi(ph0 + 15ull * dphase, (unsigned long long)K);
        float acc = 0.0f;
        unsigned nz = 0;
        for (int i = 0; i < 16; i++)
        {
            float2 v = src[base + i];
            v.x *= scale;
            v.y *= scale;
            const float p = v.x * v.x + v.y * v.y;
            if (bf == bl)
            {
                acc += p;
                nz += (p != 0.0f);
            }
            else if (p != 0.0f)
            {
                const unsigned bi = (unsigned)__umul64hi(ph0 + (uint64_t)i * dphase, (unsigned long long)K);
                atomicAdd(s_bins + bi, p);
                atomicAdd(s_cnt + bi, 1u);
            }
        }
        if (bf == bl && nz)
        {
            atomicAdd(s_bins + bf, acc);
            atomicAdd(s_cnt + bf, nz);
        }
    }
    __syncthreads();
    double *gs = sum + (size_t)(d0 + dl) * K;
    unsigned long long *gc = cnt + (size_t)(d0 + dl) * K;
    for (unsigned i = threadIdx.x; i < K; i += blockDim.x)
        if (s_cnt[i])
        {
            atomicAdd(gs + i, (double)s_bins[i]);
            atomicAdd(gc + i, (unsigned long long)s_cnt[i]);
        }
}

} // namespace

extern "C" {

// fftpoint F = 2^L (F >= 8192), batch B windows per call, D trials processed `chunk` at a
// time, fold of K bins with period (s) and sample rate fs (Hz) as Fold_GPU takes them.
// H and delays: the caller's device tables, D*F each (the engine's plan); fbs: ring slots.
int mcp_create(int L, int B, int D, int fbs, int chunk, int K, float period, float fs, const void *H,
               const void *delays, void **out)
{
    if (!out || L < 13 || L > 24 || B <= 0 || D <= 0 || fbs < B || chunk <= 0 || K <= 0 || !H || !delays)
        return 1;
    *out = nullptr;
    Pipe *p = new (std::nothrow) Pipe();
    if (!p)
        return 2;
    p->L = L;
    p->F = 1 << L;
    p->M = p->F / 2;
    p->B = B;
    p->D = D;
    p->fbs = fbs;
    // the inverse plan's batch is fixed: the largest chunk up to the request dividing D
    p->chunk = chunk < D ? chunk : D;
    while (D % p->chunk)
        p->chunk--;
    p->K = K;
    p->H = (const float2 *)H;
    p->delays = (const uint16_t *)delays;
    p->P = (double)period;
    p->dt = 1.0 / (double)fs;
    const size_t F = p->F, M = p->M;
    bool ok = cudaMalloc(&p->win, (B + 1) * M * sizeof(float2)) == cudaSuccess &&
              cudaMemset(p->win, 0, (B + 1) * M * sizeof(float2)) == cudaSuccess &&
              cudaMalloc(&p->ring, (size_t)fbs * F * sizeof(float2)) == cudaSuccess &&
              cudaMemset(p->ring, 0, (size_t)fbs * F * sizeof(float2)) == cudaSuccess &&
              cudaMalloc(&p->buf, (size_t)p->chunk * B * F * sizeof(float2)) == cudaSuccess &&
              cudaMalloc(&p->sum, (size_t)D * K * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&p->cnt, (size_t)D * K * sizeof(unsigned long long)) == cudaSuccess &&
              cudaMemset(p->sum, 0, (size_t)D * K * sizeof(double)) == cudaSuccess &&
              cudaMemset(p->cnt, 0, (size_t)D * K * sizeof(unsigned long long)) == cudaSuccess;
    int n[1] = {p->F};
    if (ok)
        ok = p->fwd_ok = cufftPlanMany(&p->fwd, 1, n, n, 1, (int)M, n, 1, p->F, CUFFT_C2C, B) == CUFFT_SUCCESS;
    if (ok)
        ok = p->inv_ok = cufftPlanMany(&p->inv, 1, n, n, 1, p->F, n, 1, p->F, CUFFT_C2C, p->chunk * B) == CUFFT_SUCCESS;
    if (!ok)
    {
        delete p;
        return 3;
    }
    *out = p;
    return 0;
}

// One call: B*M complex64 samples (device pointer), all D trials, fold accumulated.
int mcp_process(void *h, const void *in, void *stream)
{
    Pipe *p = (Pipe *)h;
    if (!p || !in)
        return 1;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t M = p->M, F = p->F;
    const int B = p->B;
    if (cudaMemcpyAsync(p->win + M, in, (size_t)B * M * sizeof(float2), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return 2;
    if (cufftSetStream(p->fwd, st) != CUFFT_SUCCESS || cufftSetStream(p->inv, st) != CUFFT_SUCCESS)
        return 3;
    if (cufftExecC2C(p->fwd, (cufftComplex *)p->win, (cufftComplex *)(p->ring + (size_t)p->rbi * F), CUFFT_FORWARD) !=
        CUFFT_SUCCESS)
        return 4;
    const uint64_t phase0 = turns_q64((long double)p->t_start / (long double)p->P);
    const uint64_t dphase = turns_q64((long double)p->dt / (long double)p->P);
    for (int d0 = 0; d0 < p->D; d0 += p->chunk)
    {
        const int nd = (p->D - d0) < p->chunk ? (p->D - d0) : p->chunk;
        gather_multiply<<<4 * 152 * 8, 256, 0, st>>>(p->ring, p->H, p->delays, p->buf, d0, nd, B, p->L, p->fbs, p->rbi);
        if (cudaGetLastError() != cudaSuccess)
            return 5;
        if (cufftExecC2C(p->inv, (cufftComplex *)p->buf, (cufftComplex *)p->buf, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return 7;
        dim3 grid((unsigned)((M + 4095) / 4096), (unsigned)(nd * B));
        discard_fold<<<grid, 256, 2 * p->K * sizeof(float), st>>>(p->buf, d0, B, p->F, p->M, phase0, dphase,
                                                                  (unsigned)p->K, p->sum, p->cnt);
        if (cudaGetLastError() != cudaSuccess)
            return 8;
    }
    // the last M samples are the next call's first window half
    if (cudaMemcpyAsync(p->win, p->win + (size_t)B * M, M * sizeof(float2), cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
        return 9;
    p->rbi = (p->rbi + B) % p->fbs;
    p->t_start += (double)((size_t)B * M) * p->dt;
    return 0;
}

int mcp_read(void *h, double *sum, unsigned long long *cnt)
{
    Pipe *p = (Pipe *)h;
    if (!p)
        return 1;
    if (cudaDeviceSynchronize() != cudaSuccess)
        return 2;
    const size_t n = (size_t)p->D * p->K;
    if (cudaMemcpy(sum, p->sum, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cnt, p->cnt, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess)
        return 3;
    return 0;
}

int mcp_reset_fold(void *h, void *stream)
{
    Pipe *p = (Pipe *)h;
    if (!p)
        return 1;
    const size_t n = (size_t)p->D * p->K;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(p->sum, 0, n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(p->cnt, 0, n * sizeof(unsigned long long), st) != cudaSuccess)
        return 2;
    p->t_start = 0.0;
    return 0;
}

void mcp_destroy(void *h) { delete (Pipe *)h; }

} // extern "C"
