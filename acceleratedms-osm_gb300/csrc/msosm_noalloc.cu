// Overlap-save filtering of a baseband segment without any device allocation.
//
// Some callers cannot allocate device memory when they call the filter:
//  * real-time acquisition loops that allocate everything at start-up, because
//    cudaMalloc/cudaFree synchronise the whole device and can stall the stream
//    past the next buffer's deadline;
//  * plug-ins running inside a host application that owns the GPU's memory
//    budget and does not let its plug-ins allocate memory of their own.
// msosm_osm_filter_noalloc serves them: it runs the engine's transform kernels
// (forward passes, response multiply, inverse passes, overlap discard) on
// buffers the caller passes in, and keeps its intermediates in one file-scope
// __device__ array of fixed size instead of calling cudaMalloc.
//
// The array is part of the library image: every GPU that loads the library
// holds its 18,939,904 bytes (about 18 MiB) until the process exits.  The
// first call on each device looks the array's device address up with
// cudaGetSymbolAddress (a one-time set-up per device), so make that first call
// before any stream capture begins.  The looked-up address is kept for the life
// of the process, so the entry point must not be used on a device after
// cudaDeviceReset (which unloads the module the array lives in).  All calls
// share the array and it keeps the last call's contents, so calls whose work
// overlaps on the GPU (for example the same or different threads issuing on two
// streams without ordering between them) race on it; order such calls on one
// stream.
#include "msosm_gb300.h"
#include "msosm_kernels.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace {

// Largest count * fftpoint (points of one pass) the scratch array holds.
constexpr size_t kNoallocMaxPoints = size_t(1) << 20;
constexpr int kNoallocMaxLog2F = 20;
constexpr int kNoallocMinLog2F = 8;
// twiddles of both directions: twN1, twN2, lo (N2), hi (N1) each, N1, N2 <= 1024
constexpr size_t kTwElems = 2 * (2 * 1024 + 2 * 1024);

constexpr size_t kOffT = 0;                                              // pass-1 intermediate
constexpr size_t kOffSpec = kOffT + kNoallocMaxPoints * sizeof(float2);  // spectra (and the discarded tail)
constexpr size_t kOffDelay = kOffSpec + kNoallocMaxPoints * sizeof(float2); // zero delay map
constexpr size_t kOffTw = kOffDelay + (size_t(1) << kNoallocMaxLog2F) * sizeof(uint16_t);
constexpr size_t kScratchBytes = kOffTw + kTwElems * sizeof(float2);

constexpr int kMaxDev = 64;

} // namespace

// The scratch.  In host code this name is only a host-side stand-in for the
// device array: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_osm_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_setup_mu;
void *g_scratch_dev[kMaxDev] = {};

// Once per device, with that device current: the device address of the array.
int scratch_address(void **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev)
        return MSOSM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_dev[dev])
    {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_osm_noalloc_scratch);
        if (e != cudaSuccess || !p)
        {
            std::fprintf(stderr, "msosm_osm_filter_noalloc: cudaGetSymbolAddress failed: %s\n",
                         cudaGetErrorString(e));
            return MSOSM_ERR_CUDA;
        }
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return MSOSM_OK;
}

// Device memory of the current device (or managed memory): anything else would
// make the kernels reach another GPU's memory or host memory.
bool device_pointer(const void *p)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

// W tables for both directions, laid out as the engine's handles lay them out
// (per direction: W_N1^m, W_N2^m, W_F^m for m < N2, W_F^(m*N2) for m < N1), computed
// on the device from (N1, N2, F) in double precision and rounded once to float;
// the same launch zeroes the delay map, since the array keeps what the last call
// left there.
__global__ void noalloc_setup_kernel(float2 *tw, int N1, int N2, int F, uint32_t *delay_words, int nwords)
{
    const int per = 2 * N1 + 2 * N2;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * per; i += stride)
    {
        const int dir = i / per, j = i % per;
        long long m, n;
        if (j < N1)
            m = j, n = N1;
        else if (j < N1 + N2)
            m = j - N1, n = N2;
        else if (j < N1 + 2 * N2)
            m = j - N1 - N2, n = F;
        else
            m = (long long)(j - N1 - 2 * N2) * N2, n = F;
        double s, c;
        sincospi(2.0 * (double)(m % n) / (double)n, &s, &c); // exp(+-2 pi i m/n)
        tw[i] = make_float2((float)c, (float)(dir == 0 ? -s : s));
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += stride)
        delay_words[i] = 0u;
}

} // namespace

extern "C" int msosm_osm_filter_noalloc(const void *x, const void *H, int fftpoint, int count, void *out,
                                        void *stream)
{
    if (!x || !H || !out || count <= 0)
        return MSOSM_ERR_ARG;
    int L = 0;
    while ((1ll << L) < (long long)fftpoint)
        L++;
    if (fftpoint <= 0 || (1ll << L) != (long long)fftpoint || L < kNoallocMinLog2F || L > kNoallocMaxLog2F)
    {
        std::fprintf(stderr, "msosm_osm_filter_noalloc: fftpoint %d must be a power of two in [2^%d, 2^%d]\n",
                     fftpoint, kNoallocMinLog2F, kNoallocMaxLog2F);
        return MSOSM_ERR_UNSUPPORTED;
    }
    if ((size_t)count * (size_t)fftpoint > kNoallocMaxPoints)
    {
        std::fprintf(stderr,
                     "msosm_osm_filter_noalloc: count*fftpoint = %zu exceeds the %zu-point scratch array; "
                     "split the segment into smaller calls\n",
                     (size_t)count * (size_t)fftpoint, kNoallocMaxPoints);
        return MSOSM_ERR_UNSUPPORTED;
    }
    if (((uintptr_t)x | (uintptr_t)H | (uintptr_t)out) % sizeof(float2) != 0 || !device_pointer(x) ||
        !device_pointer(H) || !device_pointer(out))
        return MSOSM_ERR_ARG;
    void *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != MSOSM_OK)
        return rc;

    const int F = fftpoint, M = F / 2;
    msosm::Geom g{L, F, M, 1 << (L / 2), 1 << (L - L / 2)};
    char *base = static_cast<char *>(scratch);
    float2 *T = reinterpret_cast<float2 *>(base + kOffT);
    float2 *spec = reinterpret_cast<float2 *>(base + kOffSpec);
    uint16_t *zero_delays = reinterpret_cast<uint16_t *>(base + kOffDelay);
    float2 *tw_dev = reinterpret_cast<float2 *>(base + kOffTw);
    cudaStream_t st = (cudaStream_t)stream;

    // twiddles of this fftpoint and a zero delay map, written into the array on `st`
    // (nothing is read from host memory)
    noalloc_setup_kernel<<<64, 256, 0, st>>>(tw_dev, g.N1, g.N2, F, reinterpret_cast<uint32_t *>(zero_delays), F / 2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return MSOSM_ERR_CUDA;
    const size_t per = (size_t)2 * g.N1 + 2 * g.N2;
    const msosm::Twiddles fwd{tw_dev, tw_dev + g.N1, tw_dev + g.N1 + g.N2, tw_dev + g.N1 + 2 * g.N2};
    const msosm::Twiddles inv{tw_dev + per, tw_dev + per + g.N1, tw_dev + per + g.N1 + g.N2,
                              tw_dev + per + g.N1 + 2 * g.N2};

    // windows b = 0..count-1 cover x[b*M, b*M + 2M): the first M samples act as
    // the previous call's tail, the rest as the new input
    const float2 *xin = static_cast<const float2 *>(x);
    e = msosm::launch_forward_p1(g, fwd, msosm::IN_C64, xin + M, xin, spec, T, count, st);
    if (e == cudaSuccess)
        e = msosm::launch_forward_p2(g, fwd, T, spec, 0, count, st);
    msosm::InvArgs a{};
    a.ring = spec;
    a.H = static_cast<const float2 *>(H);
    a.delays = zero_delays;
    a.T = T;
    a.rbi = 0;
    a.fbs = count;
    a.B = count;
    a.out_mode = msosm::OUT_C64;
    a.out_c64 = static_cast<float2 *>(out);
    a.out_u16 = nullptr;
    if (e == cudaSuccess)
        e = msosm::launch_inverse_p1(g, inv, a, 0, count, st);
    if (e == cudaSuccess)
        e = msosm::launch_inverse_p2(g, inv, a, 0, count, st);
    return e == cudaSuccess ? MSOSM_OK : MSOSM_ERR_CUDA;
}
