// Launchers of the element-wise kernels in misc_kernels.cu.
#pragma once

#include <cuda_runtime.h>

namespace mgb {

cudaError_t launch_r2c_fixup_inplace(float2 *z, const float2 *rtw, long long M, long long dist,
                                     unsigned batch, int full, cudaStream_t st);
cudaError_t launch_spectral_multiply(float2 *out, const float2 *a, const float2 *b, float s,
                                     unsigned long long n, cudaStream_t st);
cudaError_t launch_adjoint_filter_reduce(float2 *acc, const float2 *g, long long gdist, const float2 *a,
                                         long long adist, unsigned count, unsigned N, int stereo, float s,
                                         int accumulate, cudaStream_t st);
// Partitioned overlap-save multiply-accumulate over (64-bin groups) x G
// partition ranges.  fdl and h: P rows of upols_pitch(nb) bins (pad bins
// zero); part: G rows of that pitch; tickets: 2 + upols_groups(nb) counters,
// zeroed; xcur, y: nb bins.
cudaError_t launch_upols_mac(float2 *y, const float2 *xcur, float2 *fdl, const float2 *h, float2 *part, unsigned nb,
                             unsigned P, unsigned G, unsigned *tickets, float s, cudaStream_t st);
unsigned upols_chunks(unsigned nb, unsigned P, int sms);
unsigned upols_pitch(unsigned nb);
unsigned upols_groups(unsigned nb);
cudaError_t launch_fill_u32(unsigned *p, unsigned v, unsigned long long n, cudaStream_t st);

}  // namespace mgb
