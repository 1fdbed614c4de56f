// Split-precision tensor-core FFT for N = 256 and 4096 (16^2, 16^3).
//
// Each radix-16 Stockham stage is a complex matrix product Y = F16 X, with
// F16[k][m] = exp(-2*pi*i*k*m/16) and X the 16 inputs of a column (already
// multiplied by the stage twiddle in FP32).  In real form
//   [Yr]   [Re F  -Im F] [Xr]
//   [Yi] = [Im F   Re F] [Xi],
// so a group of 8 columns takes, per product term, four m16n8k16 BF16 MMAs
// with FP32 accumulation (A = Re F or Im F, B = 16 rows x 8 columns of Xr,
// Xi or -Xi).  FP32 values are carried as sums of BF16 limbs (Henry, Tang and
// Heinecke, "Leveraging the bfloat16 Artificial Intelligence Datatype For
// Higher-Precision Computations", ARITH 2019):
//   3 limbs (h + m + l, 24 significant bits): the six products h*h, h*m,
//     m*h, h*l, m*m, l*h -- FP32-level error;
//   2 limbs (h + m, 16 bits): h*h, h*m, m*h -- about 1e-5 relative.
// Products are accumulated smallest first.  F's limbs come from FP64.
//
// Stockham stage s (p = 16^s) reads x[j + m*N/16] (column j, m < 16),
// multiplies by W_(16p)^(m*(j mod p)) and writes the 16 outputs to
// y[(j/p)*16p + j mod p + k*p] (the radix-r autosort form of kernel.c:84-453
// with r = 16).  A CTA holds 4096 points (one N=4096 transform or sixteen
// N=256 transforms) in shared memory, ping-ponging between two buffers.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "fft_device.cuh"
#include "split_tc.h"

namespace mgb {

namespace {

// Padded shared-memory position: the stage reads are conflict-free and the
// scattered writes take 3-4 wavefronts instead of up to 8.
__device__ __forceinline__ int spad(int e) { return e + 3 * (e >> 4) + 6 * (e >> 8); }
constexpr int kSplitBuf = 4952;  // spad(4095) + 1, rounded up to 8

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// (a, b) as a sum of LIMBS bf16x2 pairs, largest first; every residual is
// exact in FP32.
template <int LIMBS>
__device__ __forceinline__ void split_pair(float a, float b, unsigned (&o)[LIMBS])
{
#pragma unroll
    for (int l = 0; l < LIMBS; l++) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        memcpy(&o[l], &h, 4);
        if (l + 1 < LIMBS) {
            const float2 f = __bfloat1622float2(h);
            a -= f.x;
            b -= f.y;
        }
    }
}

template <int S, int LIMBS>
__global__ void __launch_bounds__(kSplitThreads, 2) split_tc_fft(const SplitArgs a)
{
    constexpr int N = S == 2 ? 256 : 4096;
    constexpr int T = kSplitPoints / N;  // transforms per CTA
    constexpr int Q = N / 16;            // columns per transform
    constexpr int NT = LIMBS == 3 ? 6 : 3;
    constexpr int G = kSplitPoints / 128 / (kSplitThreads / 32);  // 8-column groups per warp and stage
    // (A limb, B limb) of each product, smallest first
    constexpr int ta[6] = {LIMBS == 3 ? 2 : 1, LIMBS == 3 ? 1 : 0, 0, 1, 0, 0};
    constexpr int tb[6] = {0, 1, LIMBS == 3 ? 2 : 0, 0, 1, 0};

    extern __shared__ float2 sm[];
    float2 *src = sm, *dst = sm + kSplitBuf;
    // stage twiddles: t1[m][q] = W_256^(m*q), t2[m][r] = W_4096^(m*r), q, r < 16;
    // W_4096^(m*(16a + b)) = t1[m][a] * t2[m][b]
    float2 *t1 = sm + 2 * kSplitBuf, *t2 = t1 + 256;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
    const long long tr0 = (long long)blockIdx.x * T;

    // A fragments of Re F and Im F (-Im F Xi is applied as Im F (-Xi))
    unsigned af[LIMBS][2][4];
#pragma unroll
    for (int l = 0; l < LIMBS; l++)
#pragma unroll
        for (int m = 0; m < 2; m++)
#pragma unroll
            for (int r = 0; r < 4; r++)
                af[l][m][r] = __ldg(&a.afrag[((l * 3 + m) * 32 + lane) * 4 + r]);
    for (int i = threadIdx.x; i < 512; i += kSplitThreads)
        t1[i] = __ldg(&a.tw[i]);

#pragma unroll 4
    for (int e = threadIdx.x; e < kSplitPoints; e += kSplitThreads) {
        const int t = e / N, n = e % N;
        float2 v = make_float2(0.f, 0.f);
        if (tr0 + t < a.ntrans)
            v = __ldg(&a.in[(tr0 + t) * a.in_dist + n]);
        if (a.conj)
            v.y = -v.y;
        src[spad(e)] = v;
    }
    __syncthreads();

#pragma unroll
    for (int s = 0; s < S; s++) {
        const int p = 1 << (4 * s);
#pragma unroll
        for (int gi = 0; gi < G; gi++) {
            const int g = warp + gi * (kSplitThreads / 32);
            const int jj = g * 8 + gid;  // this thread's input column
            const int t = jj / Q, j = jj % Q;
            float2 x[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int m = 2 * tig + (i & 1) + (i >> 1) * 8;
                float2 v = src[spad(t * N + j + Q * m)];
                if (s == 1)
                    v = cmul(v, t1[m * 16 + (j & 15)]);
                else if (s == 2)
                    v = cmul(v, cmul(t1[m * 16 + (j >> 4)], t2[m * 16 + (j & 15)]));
                x[i] = v;
            }
            unsigned br0[LIMBS], br1[LIMBS], bi0[LIMBS], bi1[LIMBS];
            split_pair<LIMBS>(x[0].x, x[1].x, br0);
            split_pair<LIMBS>(x[2].x, x[3].x, br1);
            split_pair<LIMBS>(x[0].y, x[1].y, bi0);
            split_pair<LIMBS>(x[2].y, x[3].y, bi1);
            float dr[4] = {0.f, 0.f, 0.f, 0.f}, di[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int q = 0; q < NT; q++) {
                const int la = ta[q], lb = tb[q];
                mma_bf16(dr, af[la][0], br0[lb], br1[lb]);                              // Re F  Xr
                mma_bf16(dr, af[la][1], bi0[lb] ^ 0x80008000u, bi1[lb] ^ 0x80008000u);  // Im F (-Xi)
                mma_bf16(di, af[la][1], br0[lb], br1[lb]);                              // Im F  Xr
                mma_bf16(di, af[la][0], bi0[lb], bi1[lb]);                              // Re F  Xi
            }
            // accumulator q: frequency k = gid (+8 for q >= 2), column g*8 + 2*tig + (q & 1)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int k = gid + (q >> 1) * 8;
                const int jo = g * 8 + 2 * tig + (q & 1);
                const int to = jo / Q, jq = jo % Q;
                const int pos = to * N + (jq / p) * 16 * p + (jq & (p - 1)) + k * p;
                dst[spad(pos)] = make_float2(dr[q], di[q]);
            }
        }
        __syncthreads();
        float2 *tmp = src;
        src = dst;
        dst = tmp;
    }

#pragma unroll 4
    for (int e = threadIdx.x; e < kSplitPoints; e += kSplitThreads) {
        const int t = e / N, n = e % N;
        if (tr0 + t < a.ntrans) {
            float2 v = src[spad(e)];
            if (a.conj)
                v.y = -v.y;
            a.out[(tr0 + t) * a.out_dist + n] = v;
        }
    }
}

// Round to the nearest bf16 (ties to even), returned as a double.
double bf16_round(double v)
{
    float f = (float)v;
    unsigned u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return (double)f;
}

unsigned short bf16_bits(double v)
{
    float f = (float)v;  // exact: v is already a bf16 value
    unsigned u;
    std::memcpy(&u, &f, 4);
    return (unsigned short)(u >> 16);
}

}  // namespace

const void *split_kernel(int stages, int limbs)
{
    if (stages == 2)
        return limbs == 3 ? (const void *)&split_tc_fft<2, 3> : (const void *)&split_tc_fft<2, 2>;
    if (stages == 3)
        return limbs == 3 ? (const void *)&split_tc_fft<3, 3> : (const void *)&split_tc_fft<3, 2>;
    return nullptr;
}

size_t split_smem_bytes() { return (2 * (size_t)kSplitBuf + 512) * sizeof(float2); }

std::vector<unsigned> split_afrag_table()
{
    // [limb][Re F, Im F, -Im F][lane][register]
    std::vector<unsigned> t(3 * 3 * 32 * 4);
    for (int lane = 0; lane < 32; lane++) {
        const int gid = lane >> 2, tig = lane & 3;
        for (int r = 0; r < 4; r++) {
            const int row = gid + (r & 1) * 8, col = 2 * tig + (r >> 1) * 8;
            double limb[3][3][2];  // [matrix][limb][column pair]
            for (int c = 0; c < 2; c++) {
                const double ph = -2.0 * M_PI * (double)((row * (col + c)) % 16) / 16.0;
                const double val[3] = {std::cos(ph), std::sin(ph), -std::sin(ph)};
                for (int m = 0; m < 3; m++) {
                    double v = val[m];
                    for (int l = 0; l < 3; l++) {
                        limb[m][l][c] = bf16_round(v);
                        v -= limb[m][l][c];
                    }
                }
            }
            for (int m = 0; m < 3; m++)
                for (int l = 0; l < 3; l++)
                    t[((l * 3 + m) * 32 + lane) * 4 + r] =
                        (unsigned)bf16_bits(limb[m][l][0]) | ((unsigned)bf16_bits(limb[m][l][1]) << 16);
        }
    }
    return t;
}

std::vector<float2> split_twiddle_table()
{
    // t1[m][q] = W_256^(m*q), t2[m][r] = W_4096^(m*r) for m, q, r < 16; FP64 then rounded
    std::vector<float2> t(512);
    for (int m = 0; m < 16; m++)
        for (int q = 0; q < 16; q++) {
            const double p1 = -2.0 * M_PI * (double)(m * q) / 256.0, p2 = -2.0 * M_PI * (double)(m * q) / 4096.0;
            t[m * 16 + q] = make_float2((float)std::cos(p1), (float)std::sin(p1));
            t[256 + m * 16 + q] = make_float2((float)std::cos(p2), (float)std::sin(p2));
        }
    return t;
}

}  // namespace mgb
