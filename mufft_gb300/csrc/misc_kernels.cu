// Small element-wise kernels: the in-place real-to-complex fix-up used after a
// multi-pass transform, the spectral multiply behind mufft_get_convolve_func,
// and an L2 flush for honest HBM timing.
#include "fft_device.cuh"
#include "misc_kernels.h"

namespace mgb {

// In-place real-to-complex fix-up over Z[0..M) (kernel.c:47-82).  Thread k
// owns bins k and M-k (and their upper copies), so no other thread reads what
// it overwrites.
__global__ void r2c_fixup_inplace(float2 *z, const float2 *__restrict__ rtw, long long M,
                                  long long dist, int full)
{
    float2 *zb = z + (long long)blockIdx.y * dist;
    const long long half = M / 2;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= half;
         k += (long long)gridDim.x * blockDim.x) {
        if (k == 0) {
            float2 z0 = zb[0];
            zb[0] = make_float2(z0.x + z0.y, 0.f);
            zb[M] = make_float2(z0.x - z0.y, 0.f);
            continue;
        }
        const long long km = M - k;
        float2 zk = zb[k], zm = zb[km];
        float2 lo_k, hi_k, lo_m, hi_m;
        r2c_bins(zk, zm, __ldg(&rtw[k]), lo_k, hi_k);
        if (km != k)
            r2c_bins(zm, zk, __ldg(&rtw[km]), lo_m, hi_m);
        zb[k] = lo_k;
        if (full)
            zb[k + M] = hi_k;
        if (km != k) {
            zb[km] = lo_m;
            if (full)
                zb[km + M] = hi_m;
        }
    }
}

// out[i] = s * a[i] * b[i]  (kernel.c:22-34)
__global__ void spectral_multiply(float2 *out, const float2 *__restrict__ a, const float2 *__restrict__ b,
                                  float s, unsigned long long n)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        out[i] = cscale(cmul(a[i], b[i]), s);
}

__global__ void fill_u32(unsigned *p, unsigned v, unsigned long long n)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        p[i] = v;
}

cudaError_t launch_r2c_fixup_inplace(float2 *z, const float2 *rtw, long long M, long long dist,
                                     unsigned batch, int full, cudaStream_t st)
{
    long long work = M / 2 + 1;
    unsigned blocks = (unsigned)((work + 255) / 256);
    if (blocks > 4096)
        blocks = 4096;
    r2c_fixup_inplace<<<dim3(blocks, batch), 256, 0, st>>>(z, rtw, M, dist, full);
    return cudaGetLastError();
}

cudaError_t launch_spectral_multiply(float2 *out, const float2 *a, const float2 *b, float s,
                                     unsigned long long n, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    unsigned long long blocks = (n + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    spectral_multiply<<<(unsigned)blocks, 256, 0, st>>>(out, a, b, s, n);
    return cudaGetLastError();
}

cudaError_t launch_fill_u32(unsigned *p, unsigned v, unsigned long long n, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    unsigned long long blocks = (n + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    fill_u32<<<(unsigned)blocks, 256, 0, st>>>(p, v, n);
    return cudaGetLastError();
}

}  // namespace mgb
