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

// Filter adjoint, frequency-domain reduction over a chunk of signals, for
// bins k = 0 .. N/2 of the real filter's gradient spectrum:
//   mono (r2c spectra, k <= N/2):  acc[k] (+)= s * sum_i G_i[k] conj(A_i[k])
//   stereo (full c2c spectra):     acc[k] (+)= s/2 * sum_i (G_i[k] conj(A_i[k])
//                                               + conj(G_i[N-k] conj(A_i[N-k])))
// The stereo form is the Hermitian part of the correlation spectrum, whose
// c2r inverse is the real part of the complex correlation.  Signals are
// summed in index order (deterministic).
__global__ void adjoint_filter_reduce(float2 *acc, const float2 *__restrict__ g, long long gdist,
                                      const float2 *__restrict__ a, long long adist, unsigned count,
                                      unsigned N, int stereo, float s, int accumulate)
{
    const unsigned nb = N / 2 + 1;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x) {
        const unsigned km = (N - k) & (N - 1);
        float2 sum = make_float2(0.f, 0.f);
        for (unsigned i = 0; i < count; i++) {
            const float2 *gi = g + (long long)i * gdist, *ai = a + (long long)i * adist;
            const float2 gk = gi[k], ak = ai[k];
            sum.x += gk.x * ak.x + gk.y * ak.y;  // G conj(A)
            sum.y += gk.y * ak.x - gk.x * ak.y;
            if (stereo) {
                const float2 gm = gi[km], am = ai[km];
                sum.x += gm.x * am.x + gm.y * am.y;  // conj(G conj(A)) at N-k
                sum.y -= gm.y * am.x - gm.x * am.y;
            }
        }
        const float f = stereo ? 0.5f * s : s;
        float2 r = make_float2(sum.x * f, sum.y * f);
        if (accumulate) {
            r.x += acc[k].x;
            r.y += acc[k].y;
        }
        acc[k] = r;
    }
}

// Uniformly partitioned overlap-save, one block k: multiply-accumulate of
// the current input spectrum and the previous P-1 ones (a ring of P slots,
// block j in slot j % P) with the P filter-partition spectra, scaled; the
// current spectrum then replaces block k-P in the ring.  Ring and filter
// rows have a pitch of whole 64-bin groups (pad bins zero).  A CTA covers 64
// bins (two per lane, 16-byte loads) and a range of partitions, which its 8
// warps split round-robin; the warps' sums are added in shared memory in
// warp order and written as the CTA's partial.  The last CTA of a bin group
// (ticket) adds the partials in range order (deterministic), and the last
// CTA overall advances the block counter.  Tickets never wait.
//   tickets[0] = k, tickets[1] = CTAs done, tickets[2 + x] = bin group x done.
constexpr int kMacWarps = 8;
constexpr unsigned kMacBins = 64;

__device__ __forceinline__ void cmac2(float4 &acc, const float4 a, const float4 b)
{
    acc.x += a.x * b.x - a.y * b.y;
    acc.y += a.x * b.y + a.y * b.x;
    acc.z += a.z * b.z - a.w * b.w;
    acc.w += a.z * b.w + a.w * b.z;
}

__device__ __forceinline__ float4 add4(float4 a, const float4 b)
{
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
    return a;
}

__global__ void __launch_bounds__(kMacWarps * 32) upols_mac(float2 *__restrict__ y, const float2 *__restrict__ xcur,
                                                            float2 *fdl, const float2 *__restrict__ h, float2 *part,
                                                            unsigned nb, unsigned pitch, unsigned P,
                                                            unsigned *tickets, float s)
{
    __shared__ float4 red[kMacWarps][32];
    __shared__ unsigned s_last;
    const unsigned k = *(volatile unsigned *)&tickets[0];
    const unsigned cur = k % P;
    const unsigned G = gridDim.y, g = blockIdx.y;
    const unsigned p0 = (unsigned)((unsigned long long)P * g / G), p1 = (unsigned)((unsigned long long)P * (g + 1) / G);
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b = blockIdx.x * kMacBins + 2 * lane;  // bins b, b + 1 (b < pitch, pitch even)
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b + 1 < nb) {
        const float2 x0 = xcur[b], x1 = xcur[b + 1];
        x = make_float4(x0.x, x0.y, x1.x, x1.y);
    } else if (b < nb) {
        const float2 x0 = xcur[b];
        x = make_float4(x0.x, x0.y, 0.f, 0.f);
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    // several partitions' loads in flight at once
#pragma unroll 8
    for (unsigned p = p0 + w; p < p1; p += kMacWarps) {
        const unsigned slot = cur >= p ? cur - p : cur + P - p;  // block k - p
        const float4 xp = p == 0 ? x : __ldg((const float4 *)&fdl[(size_t)slot * pitch + b]);
        const float4 hp = __ldg((const float4 *)&h[(size_t)p * pitch + b]);
        cmac2(acc, xp, hp);
    }
    red[w][lane] = acc;
    __syncthreads();
    if (w == 0) {
        float4 t = red[0][lane];
#pragma unroll
        for (int q = 1; q < kMacWarps; q++)
            t = add4(t, red[q][lane]);
        *(float4 *)&part[(size_t)g * pitch + b] = t;
        if (g == 0)
            *(float4 *)&fdl[(size_t)cur * pitch + b] = x;  // slot of block k - P: no CTA reads it for block k
        __threadfence();  // the writers' stores are visible before the ticket
    }
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = atomicAdd(&tickets[2 + blockIdx.x], 1u) == G - 1;
    __syncthreads();
    if (!s_last)
        return;
    // the other CTAs' partials, read from L2
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    for (unsigned q = w; q < G; q += kMacWarps)
        t = add4(t, __ldcg((const float4 *)&part[(size_t)q * pitch + b]));
    red[w][lane] = t;
    __syncthreads();
    if (w == 0) {
        float4 r = red[0][lane];
#pragma unroll
        for (int q = 1; q < kMacWarps; q++)
            r = add4(r, red[q][lane]);
        if (b < nb)
            y[b] = make_float2(r.x * s, r.y * s);
        if (b + 1 < nb)
            y[b + 1] = make_float2(r.z * s, r.w * s);
    }
    if (threadIdx.x == 0) {
        tickets[2 + blockIdx.x] = 0;
        __threadfence();
        if (atomicAdd(&tickets[1], 1u) == gridDim.x - 1) {
            tickets[1] = 0;
            tickets[0] = k + 1;
            __threadfence();
        }
    }
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

cudaError_t launch_adjoint_filter_reduce(float2 *acc, const float2 *g, long long gdist, const float2 *a,
                                         long long adist, unsigned count, unsigned N, int stereo, float s,
                                         int accumulate, cudaStream_t st)
{
    const unsigned nb = N / 2 + 1;
    unsigned blocks = (nb + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    adjoint_filter_reduce<<<blocks, 256, 0, st>>>(acc, g, gdist, a, adist, count, N, stereo, s, accumulate);
    return cudaGetLastError();
}

unsigned upols_pitch(unsigned nb) { return (nb + kMacBins - 1) / kMacBins * kMacBins; }

unsigned upols_groups(unsigned nb) { return (nb + kMacBins - 1) / kMacBins; }

cudaError_t launch_upols_mac(float2 *y, const float2 *xcur, float2 *fdl, const float2 *h, float2 *part, unsigned nb,
                             unsigned P, unsigned G, unsigned *tickets, float s, cudaStream_t st)
{
    upols_mac<<<dim3(upols_groups(nb), G), kMacWarps * 32, 0, st>>>(y, xcur, fdl, h, part, nb, upols_pitch(nb), P,
                                                                    tickets, s);
    return cudaGetLastError();
}

unsigned upols_chunks(unsigned nb, unsigned P, int sms)
{
    const unsigned gx = upols_groups(nb);
    const unsigned want = 4u * (unsigned)(sms > 0 ? sms : 152);
    unsigned G = (want + gx - 1) / gx;
    return G < 1 ? 1 : (G > P ? P : G);
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
