// Tensor-core pieces of the MS-OSM engine (tcgen05, sm_103a).
//
// This file holds the operand-layout self-test: one CTA stages a 128 x 64 A tile
// and a 64 x 64 B tile in the K-major 128-byte-swizzled layout of umma.cuh, runs
// four K = 16 MMAs into tensor memory and reads the FP32 accumulator back, so a
// host test can compare D = A x B^T with a CPU product.
#include "msosm_tc.cuh"
#include "umma.cuh"

#include <cuda_runtime.h>

namespace msosm {

namespace {

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
