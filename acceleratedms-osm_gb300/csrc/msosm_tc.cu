// Tensor-core pieces of the MS-OSM engine (tcgen05, sm_103a).
//
// This file holds:
//  * the W_32 operand image of the split-precision transform: the real 64 x 64 form
//    of the 32-point inverse DFT, split into 16-bit hi and lo parts (FP64 inside),
//    written in the K-major 128-byte-swizzled layout of umma.cuh;
//  * the running bound on the spectra that sets the FP16 operand scale;
//  * the operand-layout self-test: one CTA stages a 128 x 64 A tile and a 64 x 64 B
//    tile in that layout, runs four K = 16 MMAs into tensor memory and reads the FP32
//    accumulator back, so a host test can compare D = A x B^T with a CPU product.
#include "msosm_tc.cuh"
#include "umma.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace msosm {

namespace {

// B[n][kk] of the real form of W_32^(b*k) = exp(+2 pi i b k / 32): n = 2k + (0 re, 1 im
// of the output), kk = 2b + (0 re, 1 im of the input):
//   [re_out] = [ cos  -sin ] [re_in]
//   [im_out]   [ sin   cos ] [im_in]
// hi = round(w), lo = round(w - hi), both in the 16-bit type; hi image then lo image.
__global__ void tc_operand_kernel(uint16_t *out, int bf16)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 64 * 64)
        return;
    const int n = e >> 6, kk = e & 63;
    const int k = n >> 1, co = n & 1, b = kk >> 1, ci = kk & 1;
    double sn, cs;
    sincospi((double)((b * k) & 31) / 16.0, &sn, &cs);
    const double w = co == 0 ? (ci == 0 ? cs : -sn) : (ci == 0 ? sn : cs);
    uint16_t hi, lo;
    if (bf16)
    {
        const __nv_bfloat16 h = __double2bfloat16(w);
        const __nv_bfloat16 l = __double2bfloat16(w - (double)__bfloat162float(h));
        hi = __bfloat16_as_ushort(h);
        lo = __bfloat16_as_ushort(l);
    }
    else
    {
        const __half h = __double2half(w);
        const __half l = __double2half(w - (double)__half2float(h));
        hi = __half_as_ushort(h);
        lo = __half_as_ushort(l);
    }
    const uint32_t off = umma::sw128_offset(n, kk) >> 1;
    out[off] = hi;
    out[4096 + off] = lo;
}

// *out = max(*out, max |component| of p[0 .. n4)) as float bits (non-negative floats
// order like their bit patterns).
__global__ void absmax_kernel(const float4 *__restrict__ p, size_t n4, unsigned *out)
{
    float m = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x)
    {
        const float4 q = __ldcs(p + i);
        m = fmaxf(m, fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fmaxf(fabsf(q.z), fabsf(q.w))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f)
        atomicMax(out, __float_as_uint(m));
}

__global__ void __launch_bounds__(128, 1)
    umma_selftest_kernel(const uint16_t *__restrict__ A, const uint16_t *__restrict__ B, float *__restrict__ D, int n,
                         int b_row0, uint32_t idesc, int *err, unsigned long long timeout_ns)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    // operand regions on 1024-byte boundaries of the shared window
    const uint32_t pad = (1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u;
    unsigned char *sA = smem_raw + pad;  // 128 rows x 128 B
    unsigned char *sB = sA + 128 * 128;  // 64 rows x 128 B
    for (int idx = threadIdx.x; idx < 128 * 8; idx += blockDim.x)
    {
        const int r = idx >> 3, j = idx & 7;
        *reinterpret_cast<uint4 *>(sA + umma::sw128_offset(r, 8 * j)) =
            *reinterpret_cast<const uint4 *>(A + r * 64 + 8 * j);
    }
    for (int idx = threadIdx.x; idx < 64 * 8; idx += blockDim.x)
    {
        const int r = idx >> 3, j = idx & 7;
        *reinterpret_cast<uint4 *>(sB + umma::sw128_offset(r, 8 * j)) =
            *reinterpret_cast<const uint4 *>(B + r * 64 + 8 * j);
    }
    if (threadIdx.x < 32)
        umma::tmem_alloc(&tmem_base, 64);
    if (threadIdx.x == 0)
        umma::mbar_init(&mbar, 1);
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tbase = tmem_base;
    if (threadIdx.x == 0)
    {
        const uint32_t a0 = umma::smem_addr(sA), b0 = umma::smem_addr(sB) + (uint32_t)b_row0 * 128u;
#pragma unroll
        for (int k = 0; k < 4; k++)
            umma::mma_f16(tbase, umma::desc_sw128(a0 + 32u * k), umma::desc_sw128(b0 + 32u * k), idesc, k > 0);
        umma::commit(&mbar);
    }
    const bool ok = umma::mbar_wait(&mbar, 0, timeout_ns);
    if (!ok)
        atomicExch(err, 1);
    umma::fence_after_sync();
    if (ok)
    {
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const uint32_t taddr = tbase + ((uint32_t)(32 * w) << 16);
        for (int c = 0; c < n; c += 32)
        {
            float v[32];
            umma::tmem_ld32(taddr + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 32; i++)
                D[(size_t)(32 * w + lane) * n + c + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32)
        umma::tmem_dealloc(tbase, 64);
}

} // namespace

cudaError_t tc_build_operand(void *dst, int bf16, cudaStream_t st)
{
    tc_operand_kernel<<<16, 256, 0, st>>>(static_cast<uint16_t *>(dst), bf16);
    return cudaGetLastError();
}

cudaError_t tc_absmax(const float2 *p, size_t n, unsigned *out, cudaStream_t st)
{
    if (n % 2 || ((uintptr_t)p % 16))
        return cudaErrorInvalidValue;
    absmax_kernel<<<4 * 152, 256, 0, st>>>(reinterpret_cast<const float4 *>(p), n / 2, out);
    return cudaGetLastError();
}

cudaError_t tc_selftest_umma(int bf16, int n, int b_row0, const uint16_t *A, const uint16_t *B, float *D,
                             int *timed_out)
{
    if ((n != 32 && n != 64) || b_row0 < 0 || b_row0 + n > 64 || (b_row0 % 8) != 0)
        return cudaErrorInvalidValue;
    struct Buf
    {
        uint16_t a[128 * 64];
        uint16_t b[64 * 64];
        float d[128 * 64];
        int err;
    };
    Buf *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(Buf));
    if (e != cudaSuccess)
        return e;
    e = cudaMemset(d, 0, sizeof(Buf));
    if (e == cudaSuccess)
        e = cudaMemcpy(d->a, A, sizeof(d->a), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d->b, B, sizeof(d->b), cudaMemcpyHostToDevice);
    const size_t smem = 1024 + 128 * 128 + 64 * 128;
    if (e == cudaSuccess)
    {
        const uint32_t idesc = umma::idesc_f16(128, n, bf16 != 0);
        umma_selftest_kernel<<<1, 128, smem>>>(d->a, d->b, d->d, n, b_row0, idesc, &d->err, 1000000000ull);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(D, d->d, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(timed_out, &d->err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

} // namespace msosm
