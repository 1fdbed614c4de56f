// mufft_gb_execute_c2c_noalloc: a complex FFT that allocates no memory.
//
// Who needs it: callers that may not allocate GPU memory at the point where
// they transform -- a real-time audio callback (muFFT's main use is block
// convolution) cannot afford cudaMalloc's unbounded latency or its implicit
// device synchronisation; a plugin running inside a host application that
// owns and budgets all device memory may not allocate behind the host's
// back.  Such callers hold device buffers already; what the plan-based API
// would still allocate is the plan itself, its twiddle tables and, for
// transforms longer than one on-chip tile, the scratch between the two
// passes of the four-step algorithm.  Here all of that lives in file-scope
// device arrays of a fixed, modest size instead.
//
// Limits and sharing:
//   - N is a power of two, 2 <= N <= kNoAllocMaxPoints (2^20 complex points,
//     8 MiB of scratch).  Every GPU that loads the library holds the scratch
//     and the twiddle table (about 8.6 MB) until the process exits.
//   - Every call on a device shares the one scratch array, which keeps the
//     previous call's contents; the second pass reads only what the first
//     pass of the same call wrote, so nothing needs clearing.  Two calls whose
//     kernels overlap on the GPU (different streams, or different host
//     threads) race on the scratch: serialise them, e.g. on one stream.
//   - The first call on a device does the set-up: it looks up the device
//     addresses of the arrays (cudaGetSymbolAddress), fills the twiddle table
//     with a kernel and synchronises the device.  Make that first call before
//     any stream capture.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <mutex>

#include "../../include/mufft_gb300.h"
#include "fft_device.cuh"
#include "registry.h"

namespace mgb {
namespace {

constexpr unsigned kNoAllocMaxLog2 = 20;
constexpr unsigned kNoAllocMaxPoints = 1u << kNoAllocMaxLog2;

static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocMaxPoints];
static __device__ __align__(256) float2 g_noalloc_twiddles[kStageTableFloat2];

// Stage twiddle table (layout: common.h, stage_table_base) in FP64, rounded
// once to float: entry (r, p, k, e) = exp(-2*pi*i * (2^e * k mod r*p) / (r*p)).
__global__ void noalloc_fill_twiddles(float2 *t)
{
    const int n = kStageTableFloat2;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int per_radix = kStageTableK * 4;
        const int ri = idx / per_radix;
        const int kk = (idx % per_radix) / 4, e = idx % 4;
        const int r = 2 << ri;
        const int p = kk < 16 ? 16 : (kk < 272 ? 256 : 4096);
        const int k = kk - stage_p_offset(p);
        const long long rp = (long long)r * p;
        const long long m = ((long long)(1 << e) * k) % rp;
        double s, c;
        sincospi(2.0 * (double)m / (double)rp, &s, &c);
        t[idx] = make_float2((float)c, (float)-s);
    }
}

struct NoAllocDevice {
    std::atomic<bool> ready{false};  // set (release) once the fields below are final
    float2 *scratch = nullptr;   // device address of g_noalloc_scratch
    float2 *twiddles = nullptr;  // device address of g_noalloc_twiddles
    // per log2(N): single-pass tile, or the two four-step tiles
    const TileKernel *single[kNoAllocMaxLog2 + 1] = {};
    const TileKernel *cols[kNoAllocMaxLog2 + 1] = {};
    const TileKernel *rows[kNoAllocMaxLog2 + 1] = {};
};

constexpr int kMaxDev = 64;
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc[kMaxDev];

int set_up(int dev)
{
    NoAllocDevice &d = g_noalloc[dev];
    cudaError_t e = cudaGetSymbolAddress((void **)&d.scratch, g_noalloc_scratch);
    if (e != cudaSuccess)
        return (int)e;
    e = cudaGetSymbolAddress((void **)&d.twiddles, g_noalloc_twiddles);
    if (e != cudaSuccess)
        return (int)e;
    for (unsigned lg = 1; lg <= kNoAllocMaxLog2; lg++) {
        const unsigned N = 1u << lg;
        const TileKernel *ks[2] = {nullptr, nullptr};
        if (N <= kMaxSinglePass) {
            d.single[lg] = ks[0] = find_tile((int)N, ALONG, ALONG, 0, 0, 1);
        } else {
            const unsigned N1 = 1u << (lg / 2), N2 = N / N1;
            d.cols[lg] = ks[0] = find_tile((int)N1, ACROSS, ACROSS, 0, 0, 1);
            d.rows[lg] = ks[1] = find_tile((int)N2, ALONG, ACROSS, 0, 0, 1);
            if (!ks[1])
                return MUFFT_GB_ERR_UNSUPPORTED;
        }
        if (!ks[0])
            return MUFFT_GB_ERR_UNSUPPORTED;
        for (const TileKernel *k : ks) {
            if (k && k->Q != 1)
                return MUFFT_GB_ERR_UNSUPPORTED;
            if (k && k->smem > 48 * 1024) {
                e = cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k->smem);
                if (e != cudaSuccess)
                    return (int)e;
            }
        }
    }
    noalloc_fill_twiddles<<<(kStageTableFloat2 + 255) / 256, 256>>>(d.twiddles);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return (int)e;
    d.ready.store(true, std::memory_order_release);
    return MUFFT_GB_OK;
}

cudaError_t launch(const TileKernel *k, TileArgs &a, unsigned ntrans, cudaStream_t st)
{
    void *args[] = {&a};
    return cudaLaunchKernel(k->fn, dim3((ntrans + k->C - 1) / k->C), dim3(k->threads), args,
                            a.tw_lo ? k->smem : k->smem_ex, st);
}

// The address kernels use for p: p itself for device and managed memory, the
// mapped device address for page-locked host memory mapped into the device's
// address space; null for memory the device cannot reach.
const void *device_address(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)
        return p;
    if (at.type == cudaMemoryTypeHost && at.devicePointer)
        return at.devicePointer;
    return nullptr;
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" int mufft_gb_execute_c2c_noalloc(unsigned N, int direction, void *output, const void *input,
                                            void *stream)
{
    if (N < 2 || (N & (N - 1)) != 0 || (direction != MUFFT_FORWARD && direction != MUFFT_INVERSE) || !output ||
        !input)
        return MUFFT_GB_ERR_INVALID;
    if (N > kNoAllocMaxPoints)
        return MUFFT_GB_ERR_UNSUPPORTED;  // beyond the fixed scratch: use a plan
    input = device_address(input);
    output = const_cast<void *>(device_address(output));
    if (!input || !output)
        return MUFFT_GB_ERR_HOST_POINTER;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return (int)e;
    if (dev < 0 || dev >= kMaxDev)
        return MUFFT_GB_ERR_UNSUPPORTED;
    NoAllocDevice &d = g_noalloc[dev];
    if (!d.ready.load(std::memory_order_acquire)) {
        // first call on this device only: later calls take no lock
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!d.ready.load(std::memory_order_relaxed)) {
            int rc = set_up(dev);
            if (rc != MUFFT_GB_OK)
                return rc;
        }
    }
    unsigned lg = 0;
    while ((1u << lg) < N)
        lg++;
    cudaStream_t st = (cudaStream_t)stream;
    const bool inv = direction == MUFFT_INVERSE;
    TileArgs a{};
    a.tw = d.twiddles;
    a.scale = 1.0f;
    a.ntrans = 1;
    if (d.single[lg]) {
        a.in = (const float2 *)input;
        a.out = (float2 *)output;
        a.in_stride = a.out_stride = 1;
        a.in_dist = a.out_dist = N;
        a.conj = inv ? 3 : 0;
        e = launch(d.single[lg], a, 1, st);
        return e == cudaSuccess ? MUFFT_GB_OK : (int)e;
    }
    // Four-step, N = N1 x N2: column FFTs with the W_N^(k1*n2) twiddle into the
    // scratch array, then row FFTs with transposed stores into natural order.
    const unsigned N1 = 1u << (lg / 2), N2 = N / N1;
    a.in = (const float2 *)input;
    a.out = d.scratch;
    a.in_stride = a.out_stride = N2;
    a.in_dist = a.out_dist = 1;
    a.ntrans = N2;
    a.conj = inv ? 1 : 0;
    a.epilogue = EPI_TWIDDLE;
    a.tw_scale = 2.0f / (float)N;
    a.tw_mask = N - 1;
    e = launch(d.cols[lg], a, N2, st);
    if (e != cudaSuccess)
        return (int)e;
    TileArgs b{};
    b.tw = d.twiddles;
    b.scale = 1.0f;
    b.in = d.scratch;
    b.out = (float2 *)output;
    b.in_stride = 1;
    b.in_dist = N2;
    b.out_stride = N1;
    b.out_dist = 1;
    b.ntrans = N1;
    b.conj = inv ? 2 : 0;
    e = launch(d.rows[lg], b, N1, st);
    return e == cudaSuccess ? MUFFT_GB_OK : (int)e;
}
